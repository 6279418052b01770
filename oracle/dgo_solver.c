/*
 * dgo_solver.c -- oracle: basic spectral solver loop.
 * TEST INFRASTRUCTURE ONLY (see dgo.h).
 *
 * Follows (reference paths):
 *   src/grid/mech_solver_basic.cpp:19-108   init (F = I, constitutive at dt = 0, C_ref)
 *   src/grid/mech_solver_basic.cpp:110-161  calculate_solution
 *   src/grid/mech_solver_basic.cpp:163-220  forward
 *   src/grid/mech_solver_basic.cpp:242-284  converged
 *   src/grid/mech_solver_basic.cpp:286-339  form_residual
 *   src/grid/damask_grid.cpp:19-196         forward_fields, solve_fields, forward_time, loop
 * Nonlinear solver: PETSc SNES NGMRES (PETSc 3.12-3.20, third party, absent from the
 * reference tree) restated from its published algorithm (Oosterlee & Washio 2000; PETSc
 * SNESNGMRES defaults: m = 30, restart type "difference", select type "difference",
 * gammaA = gammaC = 2, epsilonB = 0.1, deltaB = 0.9, restart_it = 2, basic line search
 * for the x^M step).  The l x l least-squares problem is solved by an SVD with the
 * LAPACK gelss cutoff rcond = machine epsilon.
 */
#include "dgo.h"
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define I3(i, j) ((i) == (j) ? 1.0 : 0.0)

void dgo_numerics_default(dgo_numerics* n) {
  memset(n, 0, sizeof(*n));
  n->itmin = 1; n->itmax = 100; n->update_gamma = 0;
  n->eps_abs_div = 1e-4; n->eps_rel_div = 5e-4; n->eps_abs_P = 1e3; n->eps_rel_P = 1e-3;
  n->divergence_correction = DGO_DIVCORR_SIZE_GRID; n->derivative = DGO_DERIV_CONTINUOUS;
  n->stag_iter_max = 10; n->max_cut_back = 3;
  n->solver = DGO_SOLVER_NGMRES; n->ngmres_m = 30; n->snes_max_it = 50;
}

struct dgo_solver {
  int cells[3]; int64_t N; double geom[3], scaled[3], wgt;
  dgo_material mat; dgo_consts consts; dgo_numerics num; int nthreads;
  dgo_points pts;
  double *xi1st, *F, *F_last_inc, *F_dot, *r;
  double F_aim[9], F_aim_last_inc[9], F_aim_dot[9], P_aim[9], P_av[9];
  double C_volAvg[81], C_minMaxAvg[81], C_volAvgLastInc[81], C_minMaxAvgLastInc[81], C_ref[81], S[81];
  int stress_mask[9]; double rot_q[4]; double delta_t;
  double err_div, err_BC; int terminally_ill; int total_iter;
  int64_t evaluations;
  /* NGMRES work */
  int m; double **Xdot, **Fdot; double *XM, *FM, *XA, *FA, *D;
  double *q, *fnorms;
};

/* deterministic chunked dot product (independent of thread count) */
#define CHUNK 4096
static double dot(const double* a, const double* b, int64_t n) {
  int64_t nc = (n + CHUNK - 1) / CHUNK;
  double* part = (double*)malloc(sizeof(double) * (nc > 0 ? nc : 1));
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    double s = 0.0;
    int64_t hi = (c + 1) * CHUNK < n ? (c + 1) * CHUNK : n;
    for (int64_t i = c * CHUNK; i < hi; ++i) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0.0;
  for (int64_t c = 0; c < nc; ++c) s += part[c];
  free(part);
  return s;
}
static double nrm(const double* a, int64_t n) { return sqrt(dot(a, a, n)); }
static double nrm_diff(const double* a, const double* b, double* tmp, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) tmp[i] = a[i] - b[i];
  return nrm(tmp, n);
}

dgo_solver* dgo_solver_create(const int cells[3], const double geom[3], const int32_t* material_at,
                              int n_materials, const double* orientations,
                              const dgo_material* mat, const dgo_numerics* num, int nthreads) {
  dgo_solver* s = (dgo_solver*)calloc(1, sizeof(dgo_solver));
  for (int i = 0; i < 3; ++i) { s->cells[i] = cells[i]; s->geom[i] = geom[i]; }
  s->N = (int64_t)cells[0] * cells[1] * cells[2];
  s->wgt = pow((double)s->N, -1.0);
  s->mat = *mat; s->num = *num; s->nthreads = nthreads;
  dgo_consts_build(mat, &s->consts);
  dgo_scaled_geom(cells, geom, num->divergence_correction, s->scaled);
  size_t nh = (size_t)(cells[0] / 2 + 1) * cells[1] * cells[2];
  s->xi1st = (double*)malloc(sizeof(double) * 6 * nh);
  dgo_xi(cells, geom, num->derivative, s->xi1st, NULL);
  dgo_points_alloc(&s->pts, s->N);
  double* q = (double*)malloc(sizeof(double) * 4 * s->N);
  for (int64_t e = 0; e < s->N; ++e) {
    int ma = material_at[e];
    if (ma < 0 || ma >= n_materials) ma = 0;
    memcpy(q + 4 * e, orientations + 4 * ma, 4 * sizeof(double));
  }
  dgo_points_init(mat, &s->pts, q);
  free(q);
  size_t b = sizeof(double) * 9 * s->N;
  s->F = (double*)malloc(b); s->F_last_inc = (double*)malloc(b); s->F_dot = (double*)calloc(9 * s->N, sizeof(double));
  s->r = (double*)malloc(b);
  s->m = num->ngmres_m > 0 ? num->ngmres_m : 1;
  s->Xdot = (double**)malloc(sizeof(double*) * s->m); s->Fdot = (double**)malloc(sizeof(double*) * s->m);
  for (int i = 0; i < s->m; ++i) { s->Xdot[i] = (double*)malloc(b); s->Fdot[i] = (double*)malloc(b); }
  s->XM = (double*)malloc(b); s->FM = (double*)malloc(b); s->XA = (double*)malloc(b); s->FA = (double*)malloc(b);
  s->D = (double*)malloc(b);
  s->q = (double*)calloc((size_t)s->m * s->m, sizeof(double)); s->fnorms = (double*)calloc(s->m, sizeof(double));
  for (int k = 0; k < 9; ++k) { s->F_aim[k] = s->F_aim_last_inc[k] = I3(k % 3, k / 3); s->F_aim_dot[k] = 0; s->P_aim[k] = 0; }
  s->rot_q[0] = 1; s->rot_q[1] = s->rot_q[2] = s->rot_q[3] = 0;
  return s;
}

void dgo_solver_free(dgo_solver* s) {
  if (!s) return;
  dgo_points_free(&s->pts);
  free(s->xi1st); free(s->F); free(s->F_last_inc); free(s->F_dot); free(s->r);
  for (int i = 0; i < s->m; ++i) { free(s->Xdot[i]); free(s->Fdot[i]); }
  free(s->Xdot); free(s->Fdot); free(s->XM); free(s->FM); free(s->XA); free(s->FA); free(s->D);
  free(s->q); free(s->fnorms);
  free(s);
}

const dgo_points* dgo_solver_points(const dgo_solver* s) { return &s->pts; }
int64_t dgo_solver_total_evaluations(const dgo_solver* s) { return s->evaluations; }

void dgo_solver_get(const dgo_solver* s, const char* name, double* out) {
  size_t b9 = sizeof(double) * 9 * s->N;
  if (!strcmp(name, "F")) memcpy(out, s->F, b9);
  else if (!strcmp(name, "P")) memcpy(out, s->pts.P, b9);
  else if (!strcmp(name, "Fp")) memcpy(out, s->pts.Fp, b9);
  else if (!strcmp(name, "Lp")) memcpy(out, s->pts.Lp, b9);
  else if (!strcmp(name, "Fe")) memcpy(out, s->pts.Fe, b9);
  else if (!strcmp(name, "S")) memcpy(out, s->pts.S, b9);
  else if (!strcmp(name, "xi")) memcpy(out, s->pts.xi, sizeof(double) * 12 * s->N);
  else if (!strcmp(name, "gamma")) memcpy(out, s->pts.gamma, sizeof(double) * 12 * s->N);
  else if (!strcmp(name, "P_av")) memcpy(out, s->P_av, 9 * sizeof(double));
  else if (!strcmp(name, "F_aim")) memcpy(out, s->F_aim, 9 * sizeof(double));
  else if (!strcmp(name, "C_volAvg")) memcpy(out, s->C_volAvg, 81 * sizeof(double));
  else if (!strcmp(name, "C_minMaxAvg")) memcpy(out, s->C_minMaxAvg, 81 * sizeof(double));
  else if (!strcmp(name, "C_ref")) memcpy(out, s->C_ref, 81 * sizeof(double));
  else if (!strcmp(name, "S_compliance")) memcpy(out, s->S, 81 * sizeof(double));
  else if (!strcmp(name, "dPdF")) memcpy(out, s->pts.dPdF, sizeof(double) * 81 * s->N);
}

/* Spectral::constitutive_response: P into out, averages into the solver */
static void constitutive_response(dgo_solver* s, const double* F, double dt, double* P_out) {
  s->evaluations++;
  int ill = dgo_constitutive_response(&s->mat, &s->consts, &s->pts, F, dt, 1, s->nthreads);
  if (ill) s->terminally_ill = 1;
  dgo_averages(s->N, s->pts.P, s->pts.dPdF, s->P_av, s->C_volAvg, s->C_minMaxAvg);
  if (!(s->rot_q[0] == 1.0 && s->rot_q[1] == 0.0 && s->rot_q[2] == 0.0 && s->rot_q[3] == 0.0)) {
    double t[9];
    dgo_rotate2(s->rot_q, s->P_av, t, 0);
    memcpy(s->P_av, t, sizeof(t));
  }
  if (P_out) memcpy(P_out, s->pts.P, sizeof(double) * 9 * s->N);
}

void dgo_solver_init_state(dgo_solver* s) {
  for (int64_t e = 0; e < s->N; ++e)
    for (int k = 0; k < 9; ++k) s->F_last_inc[9 * e + k] = s->F[9 * e + k] = I3(k % 3, k / 3);
  constitutive_response(s, s->F, 0.0, NULL);
  for (int k = 0; k < 81; ++k) s->C_ref[k] = s->C_minMaxAvg[k] / s->wgt;
  memcpy(s->C_minMaxAvgLastInc, s->C_minMaxAvg, sizeof(s->C_minMaxAvg));
  memcpy(s->C_volAvgLastInc, s->C_volAvg, sizeof(s->C_volAvg));
}

/* form_residual: r = Gamma * P(F) with zero frequency <- rotated delta F_aim */
static void form_residual(dgo_solver* s, const double* X, double* R) {
  constitutive_response(s, X, s->delta_t, R);
  s->err_div = dgo_divergence_rms(s->cells, s->geom, s->scaled, s->xi1st, R);
  double rotated[9];
  s->err_BC = dgo_form_residual_bc(s->S, s->P_av, s->P_aim, s->stress_mask, s->rot_q, s->F_aim, rotated);
  dgo_gamma_convolution(s->cells, s->xi1st, s->C_ref, rotated, R);
}

/* returns >0 converged, <0 diverged, 0 iterating */
static int converged(dgo_solver* s) {
  double mx = -DBL_MAX;
  for (int k = 0; k < 9; ++k) if (s->P_av[k] > mx) mx = s->P_av[k];
  double divTol = fmax(mx * s->num.eps_rel_div, s->num.eps_abs_div);
  double BCTol = fmax(mx * s->num.eps_rel_P, s->num.eps_abs_P);
  double e = fmax(s->err_div / divTol, s->err_BC / BCTol);
  if ((s->total_iter >= s->num.itmin && e < 1.0) || s->terminally_ill) return 1;
  if (s->total_iter >= s->num.itmax) return -1;
  return 0;
}

/* ---------------------------------------------------------------- small SVD least squares */
/* minimum-norm least-squares solution of H x = b (H: l x l column-major), singular
 * values below eps * s_max dropped -- one-sided Jacobi SVD */
static void lsq_svd(int l, const double* H, double* b) {
  double U[900], V[900], sv[30], x[30];
  memcpy(U, H, sizeof(double) * l * l);
  for (int i = 0; i < l * l; ++i) V[i] = 0.0;
  for (int i = 0; i < l; ++i) V[i + l * i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < l - 1; ++p)
      for (int q = p + 1; q < l; ++q) {
        double a = 0, bb = 0, c = 0;
        for (int i = 0; i < l; ++i) { a += U[i + l * p] * U[i + l * p]; bb += U[i + l * q] * U[i + l * q]; c += U[i + l * p] * U[i + l * q]; }
        if (c == 0.0) continue;
        double ratio = fabs(c) / sqrt(a * bb);
        if (ratio > off) off = ratio;
        if (ratio < 1e-15) continue;
        double zeta = (bb - a) / (2.0 * c);
        double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
        for (int i = 0; i < l; ++i) {
          double up = U[i + l * p], uq = U[i + l * q];
          U[i + l * p] = cs * up - sn * uq; U[i + l * q] = sn * up + cs * uq;
          double vp = V[i + l * p], vq = V[i + l * q];
          V[i + l * p] = cs * vp - sn * vq; V[i + l * q] = sn * vp + cs * vq;
        }
      }
    if (off < 1e-15) break;
  }
  double smax = 0.0;
  for (int j = 0; j < l; ++j) {
    double n2 = 0.0;
    for (int i = 0; i < l; ++i) n2 += U[i + l * j] * U[i + l * j];
    sv[j] = sqrt(n2);
    if (sv[j] > smax) smax = sv[j];
  }
  double cut = DBL_EPSILON * smax;
  for (int j = 0; j < l; ++j) {
    double c = 0.0;
    if (sv[j] > cut && sv[j] > 0.0) {
      for (int i = 0; i < l; ++i) c += U[i + l * j] / sv[j] * b[i];
      c /= sv[j];
    }
    x[j] = c;
  }
  for (int i = 0; i < l; ++i) {
    double v = 0.0;
    for (int j = 0; j < l; ++j) v += V[i + l * j] * x[j];
    b[i] = v;
  }
}

/* ---------------------------------------------------------------- NGMRES */
static int snes_solve(dgo_solver* s, double* X) {
  int64_t n = 9 * s->N;
  double* F = s->r;
  int m = s->m;
  double beta[30], xi[30], H[900];
  s->total_iter = 0;
  form_residual(s, X, F);
  double fnorm = nrm(F, n);
  if (!isfinite(fnorm)) return -2;
  double fminnorm = fnorm;
  int reason = converged(s);
  if (reason) return reason;
  if (s->num.solver == DGO_SOLVER_FIXED_POINT) {
    for (int k = 1; k <= s->num.snes_max_it; ++k) {
      for (int64_t i = 0; i < n; ++i) X[i] -= F[i];
      s->total_iter = k;
      form_residual(s, X, F);
      if (!isfinite(nrm(F, n))) return -2;
      reason = converged(s);
      if (reason) return reason;
    }
    return -1;
  }
  /* update subspace 0 */
  memcpy(s->Fdot[0], F, sizeof(double) * n); memcpy(s->Xdot[0], X, sizeof(double) * n); s->fnorms[0] = fnorm;
  int k_restart = 1, l = 1, ivec = 0, restart_count = 0;
  for (int k = 1; k <= s->num.snes_max_it; ++k) {
    /* x^M: basic line search, lambda = 1 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) s->XM[i] = X[i] - F[i];
    s->total_iter = k;
    form_residual(s, s->XM, s->FM);
    double fMnorm = nrm(s->FM, n);
    if (!isfinite(fMnorm)) return -2;
    /* combined solution */
    double nu = fMnorm * fMnorm;
    for (int i = 0; i < l; ++i) xi[i] = dot(s->FM, s->Fdot[i], n);
    for (int i = 0; i < l; ++i) beta[i] = dot(s->Fdot[ivec], s->Fdot[i], n);
    for (int i = 0; i < l; ++i) { s->q[i + m * ivec] = beta[i]; s->q[ivec + m * i] = beta[i]; }
    for (int i = 0; i < l; ++i) beta[i] = nu - xi[i];
    for (int j = 0; j < l; ++j)
      for (int i = 0; i < l; ++i) H[i + l * j] = s->q[i + m * j] - xi[i] - xi[j] + nu;
    if (l == 1) beta[0] = H[0] != 0.0 ? beta[0] / H[0] : 0.0;
    else lsq_svd(l, H, beta);
    for (int i = 0; i < l; ++i) if (!isfinite(beta[i])) return -3;
    double alph_total = 0.0;
    for (int i = 0; i < l; ++i) alph_total += beta[i];
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; ++e) {
      double v = s->XM[e] * (1.0 - alph_total);
      for (int i = 0; i < l; ++i) v += beta[i] * s->Xdot[i][e];
      s->XA[e] = v;
    }
    form_residual(s, s->XA, s->FA);
    if (fminnorm > fMnorm) fminnorm = fMnorm;
    /* norms for the difference selection / restart */
    double fAnorm = nrm(s->FA, n);
    double dnorm = nrm_diff(s->XA, s->XM, s->D, n);
    double dminnorm = -1.0;
    for (int i = 0; i < l; ++i) {
      double d = nrm_diff(s->Xdot[i], s->XA, s->D, n);
      if (d < dminnorm || dminnorm < 0.0) dminnorm = d;
    }
    /* select */
    int selectA = 1;
    if (fAnorm >= 2.0 * fminnorm) selectA = 0;
    if (!(0.1 * dnorm < dminnorm || sqrt(fnorm) < 0.9 * sqrt(fminnorm))) selectA = 0;
    if (selectA) {
      fnorm = fAnorm;
      memcpy(F, s->FA, sizeof(double) * n); memcpy(X, s->XA, sizeof(double) * n);
    } else {
      fnorm = fMnorm;
      memcpy(F, s->FM, sizeof(double) * n); memcpy(X, s->XM, sizeof(double) * n);
    }
    ivec = k_restart % m;
    /* restart conditions (difference type) */
    int selectRestart = 0;
    if (0.1 * dnorm > dminnorm && sqrt(fAnorm) > 0.9 * sqrt(fminnorm) && l > 0) selectRestart = 1;
    if (sqrt(fAnorm) > 2.0 * sqrt(fminnorm)) selectRestart = 1;
    restart_count = selectRestart ? restart_count + 1 : 0;
    if (restart_count >= 2) {
      restart_count = 0; k_restart = 1; l = 1; ivec = 0;
      memcpy(s->Fdot[0], s->FM, sizeof(double) * n); memcpy(s->Xdot[0], s->XM, sizeof(double) * n);
      s->fnorms[0] = fMnorm;
    } else {
      if (l < m) l++;
      k_restart++;
      if (fminnorm > fnorm) fminnorm = fnorm;
      memcpy(s->Fdot[ivec], F, sizeof(double) * n); memcpy(s->Xdot[ivec], X, sizeof(double) * n);
      s->fnorms[ivec] = fnorm;
    }
    reason = converged(s);
    if (reason) return reason;
  }
  return -1;
}

int dgo_solver_solve(dgo_solver* s, int* iterations, int* terminally_ill) {
  dgo_masked_compliance(s->C_volAvg, s->rot_q, s->stress_mask, s->S);
  if (s->num.update_gamma)
    for (int k = 0; k < 81; ++k) s->C_ref[k] = s->C_minMaxAvg[k] / s->wgt;
  int reason = snes_solve(s, s->F);
  if (iterations) *iterations = s->total_iter;
  if (terminally_ill) *terminally_ill = s->terminally_ill;
  int conv = reason > 0;
  int ill = s->terminally_ill;
  s->terminally_ill = 0;
  for (int k = 0; k < 9; ++k) if (s->stress_mask[k]) s->P_aim[k] = s->P_av[k];
  return conv && !ill;
}

int dgo_solver_forward(dgo_solver* s, int cutback, int guess, double dt, double dt_old,
                       double t_remaining, const dgo_loadstep* ls) {
  if (cutback) {
    memcpy(s->C_volAvg, s->C_volAvgLastInc, sizeof(s->C_volAvg));
    memcpy(s->C_minMaxAvg, s->C_minMaxAvgLastInc, sizeof(s->C_minMaxAvg));
  } else {
    memcpy(s->C_volAvgLastInc, s->C_volAvg, sizeof(s->C_volAvg));
    memcpy(s->C_minMaxAvgLastInc, s->C_minMaxAvg, sizeof(s->C_minMaxAvg));
    for (int k = 0; k < 9; ++k) {
      double aim_diff = (s->F_aim[k] - s->F_aim_last_inc[k]) / dt_old;
      double stress_comp = ls->stress_mask[k] ? 0.0 : aim_diff;
      s->F_aim_dot[k] = guess ? stress_comp : 0.0;
    }
    memcpy(s->F_aim_last_inc, s->F_aim, sizeof(s->F_aim));
    double step[9];
    if (ls->def_type == DGO_BC_L) {
      /* Fortran: dot F_aim = L F_aim_lastInc */
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
        double a = 0.0;
        for (int k = 0; k < 3; ++k) a += ls->def_values[i + 3 * k] * s->F_aim_last_inc[k + 3 * j];
        step[i + 3 * j] = a;
      }
    } else if (ls->def_type == DGO_BC_DOT_F) {
      memcpy(step, ls->def_values, sizeof(step));
    } else {
      for (int k = 0; k < 9; ++k) step[k] = (ls->def_values[k] - s->F_aim_last_inc[k]) / t_remaining;
    }
    for (int k = 0; k < 9; ++k) s->F_aim_dot[k] += ls->def_mask[k] ? 0.0 : step[k];
    double rotated[9];
    dgo_rotate2(ls->rot_q, s->F_aim_dot, rotated, 1);
    /* F0 of the grid = current F; rate from the previous increment */
    dgo_calculate_rate(s->N, guess, s->F_last_inc, s->F, dt_old, rotated, s->F_dot);
    memcpy(s->F_last_inc, s->F, sizeof(double) * 9 * s->N);
  }
  for (int k = 0; k < 9; ++k) s->F_aim[k] = s->F_aim_last_inc[k] + s->F_aim_dot[k] * dt;
  for (int k = 0; k < 9; ++k) {
    if (ls->stress_type == DGO_BC_P)
      s->P_aim[k] += ls->stress_mask[k] ? (ls->stress_values[k] - s->P_aim[k]) / t_remaining * dt : 0.0;
    else
      s->P_aim[k] += ls->stress_mask[k] ? ls->stress_values[k] * dt : 0.0;
  }
  double rotated[9];
  dgo_rotate2(ls->rot_q, s->F_aim, rotated, 0);
  dgo_forward_field(s->N, dt, s->F_last_inc, s->F_dot, rotated, s->F);
  memcpy(s->stress_mask, ls->stress_mask, sizeof(s->stress_mask));
  memcpy(s->rot_q, ls->rot_q, sizeof(s->rot_q));
  s->delta_t = dt;
  return 0;
}

static double forward_time(double dt_prev_unused, const dgo_loadstep* ls, int inc, int sub_step_factor, int cut_back_level) {
  (void)dt_prev_unused;
  double dt;
  if (fabs(ls->r - 1.0) < 1.e-9) dt = ls->t / ls->N;
  else dt = ls->t * (pow(ls->r, inc) - pow(ls->r, inc + 1)) / (1.0 - pow(ls->r, ls->N));
  dt *= pow((double)sub_step_factor, -(double)cut_back_level);
  return dt;
}

int dgo_solver_run(dgo_solver* s, int nsteps, const dgo_loadstep* steps, dgo_inc_record* rec, int max_rec) {
  dgo_solver_init_state(s);
  int cut_back = 0, sub_step_factor = 2, cut_back_level = 0, total_inc = 0, nrec = 0;
  double t = 0.0, dt = 1.0, dt_prev = 0.0, t_remaining = 0.0;
  for (int l = 0; l < nsteps; ++l) {
    const dgo_loadstep* ls = &steps[l];
    double t_0 = t;
    int guess = ls->estimate_rate && l > 0;
    for (int inc = 0; inc < ls->N; ++inc) {
      total_inc++;
      dt_prev = dt;
      dt = forward_time(dt, ls, inc, sub_step_factor, cut_back_level);
      int step_fraction = 0, iters = 0, cutbacks = 0;
      int64_t ev0 = s->evaluations;
      struct timespec ts0, ts1;
      clock_gettime(CLOCK_MONOTONIC, &ts0);
      while (step_fraction < (int)pow(sub_step_factor, cut_back_level)) {
        t_remaining = ls->t + t_0 - t;
        t += dt;
        step_fraction++;
        dgo_solver_forward(s, cut_back, guess, dt, dt_prev, t_remaining, ls);
        if (!cut_back) dgo_points_commit(&s->pts);
        int it = 0, ill = 0;
        int found = dgo_solver_solve(s, &it, &ill);
        iters += it;
        if (found) {
          dt_prev = dt; cut_back = 0; guess = 1;
        } else if (cut_back_level < s->num.max_cut_back) {
          cut_back = 1; step_fraction = (step_fraction - 1) * sub_step_factor; cut_back_level++;
          t -= dt; dt /= sub_step_factor; cutbacks++;
        } else {
          return -(total_inc);
        }
      }
      cut_back_level = cut_back - 1 > 0 ? cut_back - 1 : 0;
      clock_gettime(CLOCK_MONOTONIC, &ts1);
      if (rec && nrec < max_rec) {
        rec[nrec].seconds = (double)(ts1.tv_sec - ts0.tv_sec) + 1e-9 * (double)(ts1.tv_nsec - ts0.tv_nsec);
        dgo_inc_record* r = &rec[nrec];
        r->t = t; r->dt = dt;
        memcpy(r->P_av, s->P_av, sizeof(r->P_av));
        memcpy(r->F_aim, s->F_aim, sizeof(r->F_aim));
        for (int k = 0; k < 9; ++k) {
          double a = 0.0;
          for (int64_t e = 0; e < s->N; ++e) a += s->F[9 * e + k];
          r->F_av[k] = a * s->wgt;
        }
        r->iterations = iters; r->evaluations = (int)(s->evaluations - ev0);
        r->converged = 1; r->cutbacks = cutbacks; r->err_div = s->err_div; r->err_BC = s->err_BC;
      }
      nrec++;
    }
  }
  return nrec;
}
