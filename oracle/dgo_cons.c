/*
 * dgo_cons.c -- oracle: per-material-point constitutive response.
 * TEST INFRASTRUCTURE ONLY (see dgo.h).
 *
 * Literal FP64 restatement, keeping the general Fi/Li structure of the
 * Fortran core (Li == 0: no eigenstrain kinematics), full 3x3x3x3 algebra and
 * LU solves.  Follows (reference paths):
 *   src/phase_mechanical.f90:380-604    integrateStress (Li loop around Lp Newton)
 *   src/phase_mechanical.f90:611-693    integrateStateFPI + damper
 *   src/phase.f90:626-636               converged (state)
 *   src/phase_mechanical.f90:1013-1100  phase_mechanical_constitutive (cutback)
 *   src/phase_mechanical.f90:1106-1131  mechanical_restore (includeL = false)
 *   src/phase_mechanical.f90:1137-1258  phase_mechanical_dPdF (analytic tangent)
 *   src/phase_mechanical.f90:992-1007   mechanical_forward (commit)
 *   src/phase_mechanical.f90:248-263    initial Fp = O, Fe = V_e Fp^T, Fi = O(V_e^-1)
 *   src/phase_mechanical_elastic.f90:157-195  Hooke S, dS/dFe, dS/dFi
 *   src/phase_mechanical_plastic.f90:233-339  Mp, dLp/dS, dLp/dFi, dotState
 *   src/phase_mechanical_plastic_phenopowerlaw.f90:298-394, 444-483  Lp, dLp/dMp, dotState, kinetics
 *   src/homogenization.f90:219-324, src/homogenization_mechanical.f90:94-151  per-cell loop
 *   src/grid/spectral.cpp:160-217       P_av, C_volAvg, C_minMaxAvg
 */
#include "dgo.h"
#include <math.h>
#include <string.h>
#include <stdlib.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define I3(i, j) ((i) == (j) ? 1.0 : 0.0)

static int64_t g_cnt_state = 0, g_cnt_lp = 0, g_cnt_eval = 0, g_cnt_tangent = 0;
void dgo_counters(int64_t out[4]) { out[0] = g_cnt_eval; out[1] = g_cnt_state; out[2] = g_cnt_lp; out[3] = g_cnt_tangent; }
void dgo_counters_reset(void) { g_cnt_state = g_cnt_lp = g_cnt_eval = g_cnt_tangent = 0; }

/* ---------------------------------------------------------------- 3x3 helpers */
static void mm(const double* A, const double* B, double* C) {      /* C = A B */
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += A[i + 3 * k] * B[k + 3 * j];
      t[i + 3 * j] = s;
    }
  memcpy(C, t, sizeof(t));
}
static void tr(const double* A, double* T) {
  double t[9];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) t[i + 3 * j] = A[j + 3 * i];
  memcpy(T, t, sizeof(t));
}
static double norm2_9(const double* A) {
  double s = 0.0;
  for (int i = 0; i < 9; ++i) s += A[i] * A[i];
  return sqrt(s);
}
static int has_nan(const double* a, int n) {
  for (int i = 0; i < n; ++i) if (isnan(a[i])) return 1;
  return 0;
}
static double det33(const double* m) {
  return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2])
       + m[6] * (m[1] * m[5] - m[4] * m[2]);
}
/* math_mul3333xx3333: C(i,j,k,l) = sum_mn A(i,j,m,n) B(m,n,k,l) */
static void mul3333(const double* A, const double* B, double* C) {
  double t[81];
  for (int ij = 0; ij < 9; ++ij)
    for (int kl = 0; kl < 9; ++kl) {
      double s = 0.0;
      for (int mn = 0; mn < 9; ++mn) s += A[ij + 9 * mn] * B[mn + 9 * kl];
      t[ij + 9 * kl] = s;
    }
  memcpy(C, t, sizeof(t));
}
/* solve A x = b (dgesv), A 9x9 column-major, b overwritten */
static int solve9(const double* A0, double* b) {
  double A[81];
  memcpy(A, A0, sizeof(A));
  int piv[9];
  for (int k = 0; k < 9; ++k) {
    int p = k; double mx = fabs(A[k + 9 * k]);
    for (int i = k + 1; i < 9; ++i) if (fabs(A[i + 9 * k]) > mx) { mx = fabs(A[i + 9 * k]); p = i; }
    piv[k] = p;
    if (A[p + 9 * k] == 0.0) return 1;
    if (p != k) for (int j = 0; j < 9; ++j) { double t = A[k + 9 * j]; A[k + 9 * j] = A[p + 9 * j]; A[p + 9 * j] = t; }
    for (int i = k + 1; i < 9; ++i) {
      A[i + 9 * k] /= A[k + 9 * k];
      for (int j = k + 1; j < 9; ++j) A[i + 9 * j] -= A[i + 9 * k] * A[k + 9 * j];
    }
  }
  for (int k = 0; k < 9; ++k) { int p = piv[k]; if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; } }
  for (int i = 0; i < 9; ++i) for (int j = 0; j < i; ++j) b[i] -= A[i + 9 * j] * b[j];
  for (int i = 8; i >= 0; --i) {
    for (int j = i + 1; j < 9; ++j) b[i] -= A[i + 9 * j] * b[j];
    b[i] /= A[i + 9 * i];
  }
  return 0;
}
static void v33to9(const double* m, double* v) { for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) v[3 * a + b] = m[a + 3 * b]; }
static void v9to33(const double* v, double* m) { for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) m[a + 3 * b] = v[3 * a + b]; }

/* ---------------------------------------------------------------- constitutive law */
/* phase_hooke_SandItsTangents */
static void hooke(const dgo_consts* c, const double* Fe, const double* Fi,
                  double* S, double* dS_dFe, double* dS_dFi) {
  double E[9], FeT[9], t[9], FiT[9];
  tr(Fe, FeT); mm(FeT, Fe, E);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) E[i + 3 * j] = 0.5 * (E[i + 3 * j] - I3(i, j));
  tr(Fi, FiT); mm(FiT, E, t); mm(t, Fi, t);
  double eps6[6] = {t[0], t[4], t[8], 2.0 * t[5], 2.0 * t[2], 2.0 * t[3]};
  double sig6[6];
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int j = 0; j < 6; ++j) s += c->C66[i + 6 * j] * eps6[j];
    sig6[i] = s;
  }
  S[0] = sig6[0]; S[4] = sig6[1]; S[8] = sig6[2];
  S[5] = S[7] = sig6[3]; S[2] = S[6] = sig6[4]; S[1] = S[3] = sig6[5];
  double EFi[9];
  mm(E, Fi, EFi);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double Cij[9], a[9], b[9];
      for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) Cij[k + 3 * l] = c->C[i + 3 * j + 9 * k + 27 * l];
      mm(Fi, Cij, a); mm(a, FiT, a); mm(Fe, a, b);
      for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) dS_dFe[i + 3 * j + 9 * k + 27 * l] = b[k + 3 * l];
      if (dS_dFi) {
        mm(EFi, Cij, a);
        for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) dS_dFi[i + 3 * j + 9 * k + 27 * l] = 2.0 * a[k + 3 * l];
      }
    }
}

/* kinetics_sl */
static void kinetics(const dgo_material* m, const dgo_consts* c, const double* Mp, const double* xi,
                     double* gdot, double* dgdot) {
  for (int s = 0; s < 12; ++s) {
    double tp = 0.0;
    for (int k = 0; k < 9; ++k) tp += Mp[k] * c->P_sl[s][k];
    double tn = 0.0;
    for (int k = 0; k < 9; ++k) tn += Mp[k] * (-c->P_sl[s][k]);
    double tmax = tp > tn ? tp : tn;
    gdot[s] = (tp > tn ? 1.0 : -1.0) * m->dot_gamma_0 * pow(tmax / xi[s], m->n);
    if (dgdot) dgdot[s] = (fabs(gdot[s]) > DBL_MIN * 10.0) ? gdot[s] * m->n / tmax : 0.0;
  }
}

/* plastic_LpAndItsTangents (phenopowerlaw) */
static void lp_and_tangents(const dgo_material* m, const dgo_consts* c, const double* S, const double* Fi,
                            const double* xi, double* Lp, double* dLp_dS, double* dLp_dFi) {
  double FiT[9], FtF[9], Mp[9];
  tr(Fi, FiT); mm(FiT, Fi, FtF); mm(FtF, S, Mp);
  double gdot[12], dg[12];
  kinetics(m, c, Mp, xi, gdot, dg);
  double dLp_dMp[81];
  memset(Lp, 0, 9 * sizeof(double));
  memset(dLp_dMp, 0, sizeof(dLp_dMp));
  for (int s = 0; s < 12; ++s) {
    const double* P = c->P_sl[s];
    double sgn = gdot[s] > 0.0 ? 1.0 : -1.0;
    for (int k = 0; k < 9; ++k) Lp[k] += gdot[s] * P[k];
    for (int kl = 0; kl < 9; ++kl)
      for (int mn = 0; mn < 9; ++mn) dLp_dMp[kl + 9 * mn] += dg[s] * P[kl] * (sgn * P[mn]);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double D[9], DT[9], a[9], b[9];
      for (int k = 0; k < 9; ++k) D[k] = dLp_dMp[i + 3 * j + 9 * k];
      if (dLp_dFi) {
        double FiS[9];
        mm(Fi, S, FiS); tr(D, DT); mm(FiS, DT, a);
        mm(Fi, D, b); mm(b, S, b);
        for (int k = 0; k < 9; ++k) dLp_dFi[i + 3 * j + 9 * k] = a[k] + b[k];
      }
      mm(FtF, D, a);
      for (int k = 0; k < 9; ++k) dLp_dS[i + 3 * j + 9 * k] = a[k];
    }
}

/* phenopowerlaw_dotState: [dot_xi(12), dot_gamma(12)] */
static void dot_state(const dgo_material* m, const dgo_consts* c, const double* S, const double* Fi,
                      const double* xi, double* dot) {
  double FiT[9], FtF[9], Mp[9], gdot[12];
  tr(Fi, FiT); mm(FiT, Fi, FtF); mm(FtF, S, Mp);
  kinetics(m, c, Mp, xi, gdot, NULL);
  for (int s = 0; s < 12; ++s) gdot[s] = fabs(gdot[s]);
  for (int s = 0; s < 12; ++s) {
    double x = 1.0 - xi[s] / (m->xi_inf + 0.0);
    double left = copysign(pow(fabs(x), m->a), x);
    double hsum = 0.0;
    for (int b = 0; b < 12; ++b) hsum += c->h[s][b] * gdot[b];
    dot[s] = m->h_0 * (1.0 + m->c_1 * pow(0.0, m->c_2)) * left * hsum;
    dot[12 + s] = gdot[s];
  }
}

/* per-point working view */
typedef struct pt {
  double *F, *F0, *Fp, *Fp0, *Fi, *Fi0, *Fe, *Lp, *Lp0, *Li, *Li0, *S, *S0, *P;
  double *xi, *xi0, *gamma, *gamma0, *dPdF;
  double state[24];   /* plasticState%state  = [xi, gamma] */
  double state0[24];  /* plasticState%state0 */
} pt;

/* integrateStress: returns 1 if broken */
static int integrate_stress(const dgo_material* m, const dgo_consts* c, pt* p,
                            const double* F, const double* Fp0, const double* Fi0, double dt) {
  double Lpguess[9], Liguess[9], invFp_current[9], invFi_current[9], A[9];
  memcpy(Lpguess, p->Lp, sizeof(Lpguess));
  memcpy(Liguess, p->Li, sizeof(Liguess));
  if (dgo_invert33(Fp0, invFp_current, NULL)) return 1;
  if (dgo_invert33(Fi0, invFi_current, NULL)) return 1;
  mm(F, invFp_current, A);

  double invFi_new[9], Fi_new[9], B[9], Fe[9], S[9];
  double dS_dFe[81], dS_dFi[81], Lp_c[9], dLp_dS[81], dLp_dFi[81];
  double residuumLp[9], residuumLp_old[9], Lpguess_old[9], deltaLp[9] = {0};
  double Li_c[9] = {0}, residuumLi[9], residuumLi_old[9], Liguess_old[9];
  double steplengthLi = 1.0;
  memset(residuumLi_old, 0, sizeof(residuumLi_old));
  memcpy(Liguess_old, Liguess, sizeof(Liguess_old));
  int itLi = 0;
  for (;;) {                                           /* LiLoop */
    if (++itLi > m->N_iter_Lp_max) return 1;         /* N_iter_Li_max defaults to 40 */
    double t[9];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) t[i + 3 * j] = I3(i, j) - dt * Liguess[i + 3 * j];
    mm(invFi_current, t, invFi_new);
    if (dgo_invert33(invFi_new, Fi_new, NULL)) memset(Fi_new, 0, sizeof(Fi_new));

    int jacoCounterLp = 0;
    double steplengthLp = 1.0;
    memset(residuumLp_old, 0, sizeof(residuumLp_old));
    memcpy(Lpguess_old, Lpguess, sizeof(Lpguess_old));
    int itLp = 0;
    for (;;) {                                         /* LpLoop */
      if (++itLp > m->N_iter_Lp_max) return 1;
#pragma omp atomic
      g_cnt_lp++;
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) B[i + 3 * j] = I3(i, j) - dt * Lpguess[i + 3 * j];
      mm(A, B, Fe); mm(Fe, invFi_new, Fe);
      hooke(c, Fe, Fi_new, S, dS_dFe, dS_dFi);
      lp_and_tangents(m, c, S, Fi_new, p->state, Lp_c, dLp_dS, dLp_dFi);
      double nLg = norm2_9(Lpguess), nLc = norm2_9(Lp_c);
      double atol_Lp = m->eps_rel_Lp * (nLg > nLc ? nLg : nLc);
      if (atol_Lp < m->eps_abs_Lp) atol_Lp = m->eps_abs_Lp;
      for (int k = 0; k < 9; ++k) residuumLp[k] = Lpguess[k] - Lp_c[k];
      double nr = norm2_9(residuumLp);
      if (has_nan(residuumLp, 9)) return 1;
      else if (nr < atol_Lp) break;
      else if (itLp == 1 || nr < norm2_9(residuumLp_old)) {
        memcpy(residuumLp_old, residuumLp, sizeof(residuumLp));
        memcpy(Lpguess_old, Lpguess, sizeof(Lpguess));
        steplengthLp = 1.0;
      } else {
        steplengthLp = m->r_linesearch_Lp * steplengthLp;
        for (int k = 0; k < 9; ++k) Lpguess[k] = Lpguess_old[k] + deltaLp[k] * steplengthLp;
        continue;
      }
      if (jacoCounterLp % m->f_update_jacobi_Lp == 0) {
        jacoCounterLp++;
        double dFe_dLp[81], tmp[81], J99[81], M99[81], v[9];
        for (int o = 0; o < 3; ++o) for (int pp = 0; pp < 3; ++pp)
          for (int j = 0; j < 3; ++j) for (int l = 0; l < 3; ++l)
            dFe_dLp[o + 3 * j + 9 * pp + 27 * l] = -dt * A[o + 3 * pp] * invFi_new[l + 3 * j];
        mul3333(dLp_dS, dS_dFe, tmp);
        mul3333(tmp, dFe_dLp, tmp);
        dgo_3333to99(tmp, M99);
        for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j) J99[i + 9 * j] = I3(i, j) - M99[i + 9 * j];
        v33to9(residuumLp, v);
        if (solve9(J99, v)) return 1;
        v9to33(v, deltaLp);
        for (int k = 0; k < 9; ++k) deltaLp[k] = -deltaLp[k];
      }
      for (int k = 0; k < 9; ++k) Lpguess[k] = Lpguess[k] + deltaLp[k] * steplengthLp;
    }

    /* phase_LiAndItsTangents: no eigenstrain kinematics -> Li = 0 */
    memset(Li_c, 0, sizeof(Li_c));
    double nLg = norm2_9(Liguess), nLc = norm2_9(Li_c);
    double atol_Li = m->eps_rel_Lp * (nLg > nLc ? nLg : nLc);
    if (atol_Li < m->eps_abs_Lp) atol_Li = m->eps_abs_Lp;
    for (int k = 0; k < 9; ++k) residuumLi[k] = Liguess[k] - Li_c[k];
    if (has_nan(residuumLi, 9)) return 1;
    if (norm2_9(residuumLi) < atol_Li) break;
    /* with Li == 0 the Li correction is a pure relaxation towards zero; the
     * reference's Jacobian reduces to the identity in that case */
    if (itLi == 1 || norm2_9(residuumLi) < norm2_9(residuumLi_old)) {
      memcpy(residuumLi_old, residuumLi, sizeof(residuumLi));
      memcpy(Liguess_old, Liguess, sizeof(Liguess));
      steplengthLi = 1.0;
    } else {
      steplengthLi *= 0.5;
    }
    for (int k = 0; k < 9; ++k) Liguess[k] = Liguess_old[k] - residuumLi[k] * steplengthLi;
  }

  double invFp_new[9], Fp_new[9], t1[9], t2[9], invFpT[9];
  mm(invFp_current, B, invFp_new);
  if (dgo_invert33(invFp_new, Fp_new, NULL)) return 1;
  tr(invFp_new, invFpT);
  mm(F, invFp_new, t1); mm(S, invFpT, t2); mm(t1, t2, p->P);
  memcpy(p->S, S, sizeof(S));
  memcpy(p->Lp, Lpguess, sizeof(Lpguess));
  memcpy(p->Li, Liguess, sizeof(Liguess));
  double s = pow(det33(Fp_new), 1.0 / 3.0);
  for (int k = 0; k < 9; ++k) p->Fp[k] = Fp_new[k] / s;
  memcpy(p->Fi, Fi_new, sizeof(Fi_new));
  mm(F, invFp_new, t1); mm(t1, invFi_new, p->Fe);
  return 0;
}

static double damper(const double* o0, const double* o1, const double* o2) {
  double d12 = 0, d22 = 0, d01 = 0;
  for (int i = 0; i < 24; ++i) {
    d12 += (o0[i] - o1[i]) * (o1[i] - o2[i]);
    d22 += (o1[i] - o2[i]) * (o1[i] - o2[i]);
    d01 += o0[i] * o1[i];
  }
  if (((d01 < d12) ? d01 : d12) < 0.0 && d22 > 0.0) return 0.75 + 0.25 * tanh(2.0 + 4.0 * d12 / d22);
  return 1.0;
}

/* integrateStateFPI: returns 1 if broken */
static int integrate_state_fpi(const dgo_material* m, const dgo_consts* c, pt* p, const double* F,
                               const double* Fp0, const double* Fi0, const double* state0, double dt) {
  double dot[24], last1[24], last2[24], r[24];
  int broken = 1;
#pragma omp atomic
  g_cnt_state++;
  dot_state(m, c, p->S, p->Fi, p->state, dot);
  if (has_nan(dot, 24)) return 1;
  for (int i = 0; i < 24; ++i) p->state[i] = state0[i] + dot[i] * dt;
  for (int it = 1; it <= m->N_iter_state_max; ++it) {
    for (int i = 0; i < 24; ++i) { last2[i] = it > 1 ? last1[i] : 0.0; last1[i] = dot[i]; }
    broken = integrate_stress(m, c, p, F, Fp0, Fi0, dt);
    if (broken) break;
    dot_state(m, c, p->S, p->Fi, p->state, dot);
    if (has_nan(dot, 24)) break;
    double z = damper(dot, last1, last2);
    for (int i = 0; i < 24; ++i) dot[i] = dot[i] * z + last1[i] * (1.0 - z);
    for (int i = 0; i < 24; ++i) r[i] = p->state[i] - state0[i] - dot[i] * dt;
    for (int i = 0; i < 24; ++i) p->state[i] = p->state[i] - r[i];
    int conv = 1;
    for (int i = 0; i < 24; ++i) {
      double atol = i < 12 ? m->atol_xi : m->atol_gamma;
      double tol = m->eps_rel_state * fabs(p->state[i]);
      if (!(fabs(r[i]) <= (atol > tol ? atol : tol))) { conv = 0; break; }
    }
    if (conv) { broken = 0; break; }
  }
  return broken;
}

/* phase_mechanical_constitutive: returns 1 if converged */
static int constitutive(const dgo_material* m, const dgo_consts* c, pt* p, double dt) {
  double state0[24], Lp0[9], Li0[9], Fp0[9], Fi0[9], F0[9], F[9];
  memcpy(state0, p->state0, sizeof(state0));
  memcpy(Li0, p->Li0, sizeof(Li0)); memcpy(Lp0, p->Lp0, sizeof(Lp0));
  memcpy(Fp0, p->Fp0, sizeof(Fp0)); memcpy(Fi0, p->Fi0, sizeof(Fi0));
  memcpy(F0, p->F0, sizeof(F0));
  memcpy(F, p->F, sizeof(F));
  double stepFrac = 0.0, step = 1.0 / m->r_cutback;
  int converged = 0, todo = 1;
  while (todo) {
    if (converged) {
      stepFrac += step;
      step = (1.0 - stepFrac) < m->r_increase * step ? (1.0 - stepFrac) : m->r_increase * step;
      todo = step > 0.0;
      if (todo) {
        memcpy(F0, F, sizeof(F0));
        memcpy(Lp0, p->Lp, sizeof(Lp0)); memcpy(Li0, p->Li, sizeof(Li0));
        memcpy(Fp0, p->Fp, sizeof(Fp0)); memcpy(Fi0, p->Fi, sizeof(Fi0));
        memcpy(state0, p->state, sizeof(state0));
      }
    } else {
      step = m->r_cutback * step;
      memcpy(p->Fp, Fp0, sizeof(Fp0)); memcpy(p->Fi, Fi0, sizeof(Fi0));
      memcpy(p->S, p->S0, 9 * sizeof(double));
      if (step < 1.0) { memcpy(p->Lp, Lp0, sizeof(Lp0)); memcpy(p->Li, Li0, sizeof(Li0)); }
      memcpy(p->state, state0, sizeof(state0));
      todo = step > m->r_cutback_min;
    }
    if (todo) {
      for (int k = 0; k < 9; ++k) F[k] = F0[k] + step * (p->F[k] - p->F0[k]);
      converged = !integrate_state_fpi(m, c, p, F, Fp0, Fi0, state0, step * dt);
    }
  }
  return converged;
}

/* phase_mechanical_dPdF with dLi/dS == 0 */
static void tangent(const dgo_material* m, const dgo_consts* c, pt* p, double dt, double* dPdF) {
  double dSdFe[81], dSdFi[81], devNull[9], dLpdS[81], dLpdFi[81], dFidS[81];
  hooke(c, p->Fe, p->Fi, devNull, dSdFe, dSdFi);
  double invFp[9], invFi[9], invSubFp0[9], invSubFi0[9];
  dgo_invert33(p->Fp, invFp, NULL); dgo_invert33(p->Fi, invFi, NULL);
  dgo_invert33(p->Fp0, invSubFp0, NULL); dgo_invert33(p->Fi0, invSubFi0, NULL);
  memset(dFidS, 0, sizeof(dFidS));                 /* sum(abs(dLidS)) < tol */
  lp_and_tangents(m, c, p->S, p->Fi, p->state, devNull, dLpdS, dLpdFi);
  double tmp[81];
  mul3333(dLpdFi, dFidS, tmp);
  for (int k = 0; k < 81; ++k) dLpdS[k] = tmp[k] + dLpdS[k];

  double t1[9], t2[9], t3[9], a[9];
  mm(invFp, invFi, a); tr(a, t1);
  mm(p->F, invSubFp0, t2);
  mm(p->F, invFp, a); mm(a, invSubFi0, t3);
  double rhs[81], temp[81], lhs[81];
  for (int o = 0; o < 3; ++o) for (int pp = 0; pp < 3; ++pp) {
    double D[9], r[9], X[9];
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) D[k + 3 * l] = dSdFe[pp + 3 * o + 9 * k + 27 * l];
    mm(D, t1, r);
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) rhs[pp + 3 * o + 9 * k + 27 * l] = r[k + 3 * l];
    for (int k = 0; k < 9; ++k) D[k] = dLpdS[k + 9 * (pp + 3 * o)];
    mm(t2, D, X); mm(X, invFi, X);
    for (int k = 0; k < 9; ++k) temp[k + 9 * (pp + 3 * o)] = X[k];        /* + t3 * dLidS(=0) */
  }
  double l1[81], l2[81];
  mul3333(dSdFe, temp, l1);
  mul3333(dSdFi, dFidS, l2);
  for (int k = 0; k < 81; ++k) lhs[k] = l1[k] * dt + l2[k];
  double M99[81], I99[81], inv99[81], inv3333[81], dSdF[81];
  dgo_3333to99(lhs, M99);
  for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j) I99[i + 9 * j] = I3(i, j) + M99[i + 9 * j];
  if (dgo_invert(9, I99, inv99)) {
    memcpy(dSdF, rhs, sizeof(dSdF));
  } else {
    dgo_99to3333(inv99, inv3333);
    mul3333(inv3333, rhs, dSdF);
  }
  double dFpinvdF[81];
  mul3333(dLpdS, dSdF, temp);
  for (int o = 0; o < 3; ++o) for (int pp = 0; pp < 3; ++pp) {
    double D[9], X[9];
    for (int k = 0; k < 9; ++k) D[k] = temp[k + 9 * (pp + 3 * o)];
    mm(D, invFi, X); mm(invSubFp0, X, X);
    for (int k = 0; k < 9; ++k) dFpinvdF[k + 9 * (pp + 3 * o)] = -X[k] * dt;
  }
  double invFpT[9], u1[9], u2[9], u3[9];
  tr(invFp, invFpT);
  mm(p->S, invFpT, u1);
  mm(p->F, invFp, u2);
  mm(u2, p->S, u3);
  memset(dPdF, 0, 81 * sizeof(double));
  double w[9], wT[9];
  mm(invFp, u1, w); tr(w, wT);
  for (int q = 0; q < 3; ++q)
    for (int j = 0; j < 3; ++j) for (int l = 0; l < 3; ++l) dPdF[q + 3 * j + 9 * q + 27 * l] = wT[j + 3 * l];
  for (int o = 0; o < 3; ++o) for (int pp = 0; pp < 3; ++pp) {
    double D[9], X[9], Y[9], Z[9], DT[9], dS[9];
    for (int k = 0; k < 9; ++k) D[k] = dFpinvdF[k + 9 * (pp + 3 * o)];
    for (int k = 0; k < 9; ++k) dS[k] = dSdF[k + 9 * (pp + 3 * o)];
    mm(p->F, D, X); mm(X, u1, X);
    mm(u2, dS, Y); mm(Y, invFpT, Y);
    tr(D, DT); mm(u3, DT, Z);
    for (int k = 0; k < 9; ++k) dPdF[k + 9 * (pp + 3 * o)] += X[k] + Y[k] + Z[k];
  }
}

/* ---------------------------------------------------------------- points */
int dgo_points_alloc(dgo_points* p, int64_t n) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  double** f9[] = {&p->F, &p->F0, &p->Fp, &p->Fp0, &p->Fi, &p->Fi0, &p->Fe, &p->Lp, &p->Lp0,
                   &p->Li, &p->Li0, &p->S, &p->S0, &p->P};
  for (size_t i = 0; i < sizeof(f9) / sizeof(f9[0]); ++i) {
    *f9[i] = (double*)calloc((size_t)(9 * n), sizeof(double));
    if (!*f9[i]) return 1;
  }
  double** f12[] = {&p->xi, &p->xi0, &p->gamma, &p->gamma0};
  for (size_t i = 0; i < 4; ++i) {
    *f12[i] = (double*)calloc((size_t)(12 * n), sizeof(double));
    if (!*f12[i]) return 1;
  }
  p->dPdF = (double*)calloc((size_t)(81 * n), sizeof(double));
  p->status = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  return (p->dPdF && p->status) ? 0 : 1;
}

void dgo_points_free(dgo_points* p) {
  double* f[] = {p->F, p->F0, p->Fp, p->Fp0, p->Fi, p->Fi0, p->Fe, p->Lp, p->Lp0, p->Li, p->Li0,
                 p->S, p->S0, p->P, p->xi, p->xi0, p->gamma, p->gamma0, p->dPdF};
  for (size_t i = 0; i < sizeof(f) / sizeof(f[0]); ++i) free(f[i]);
  free(p->status);
  memset(p, 0, sizeof(*p));
}

void dgo_points_init(const dgo_material* m, dgo_points* p, const double* q) {
  for (int64_t e = 0; e < p->n; ++e) {
    double R[9], RT[9], Fi[9];
    dgo_qu2om(q + 4 * e, R);
    tr(R, RT);
    mm(R, RT, Fi);                                 /* O.rotate(inv(V_e)) with V_e = I */
    for (int k = 0; k < 9; ++k) {
      p->F[9 * e + k] = p->F0[9 * e + k] = I3(k % 3, k / 3);
      p->Fp[9 * e + k] = p->Fp0[9 * e + k] = R[k];
      p->Fe[9 * e + k] = RT[k];                    /* V_e Fp^T */
      p->Fi[9 * e + k] = p->Fi0[9 * e + k] = Fi[k];
      p->Lp[9 * e + k] = p->Lp0[9 * e + k] = p->Li[9 * e + k] = p->Li0[9 * e + k] = 0.0;
      p->S[9 * e + k] = p->S0[9 * e + k] = p->P[9 * e + k] = 0.0;
    }
    for (int s = 0; s < 12; ++s) {
      p->xi[12 * e + s] = p->xi0[12 * e + s] = m->xi_0;
      p->gamma[12 * e + s] = p->gamma0[12 * e + s] = 0.0;
    }
  }
}

void dgo_points_commit(dgo_points* p) {
  size_t b9 = (size_t)p->n * 9 * sizeof(double), b12 = (size_t)p->n * 12 * sizeof(double);
  memcpy(p->Fi0, p->Fi, b9); memcpy(p->Fp0, p->Fp, b9); memcpy(p->F0, p->F, b9);
  memcpy(p->Li0, p->Li, b9); memcpy(p->Lp0, p->Lp, b9); memcpy(p->S0, p->S, b9);
  memcpy(p->xi0, p->xi, b12); memcpy(p->gamma0, p->gamma, b12);
}

static void bind(dgo_points* P, int64_t e, pt* p) {
  p->F = P->F + 9 * e; p->F0 = P->F0 + 9 * e; p->Fp = P->Fp + 9 * e; p->Fp0 = P->Fp0 + 9 * e;
  p->Fi = P->Fi + 9 * e; p->Fi0 = P->Fi0 + 9 * e; p->Fe = P->Fe + 9 * e; p->Lp = P->Lp + 9 * e;
  p->Lp0 = P->Lp0 + 9 * e; p->Li = P->Li + 9 * e; p->Li0 = P->Li0 + 9 * e; p->S = P->S + 9 * e;
  p->S0 = P->S0 + 9 * e; p->P = P->P + 9 * e; p->dPdF = P->dPdF + 81 * e;
  p->xi = P->xi + 12 * e; p->xi0 = P->xi0 + 12 * e; p->gamma = P->gamma + 12 * e; p->gamma0 = P->gamma0 + 12 * e;
}

int dgo_constitutive_response(const dgo_material* m, const dgo_consts* c, dgo_points* P,
                              const double* F, double dt, int want_dPdF, int nthreads) {
  int ill = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp atomic
  g_cnt_eval++;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : ill)
  for (int64_t e = 0; e < P->n; ++e) {
    pt p;
    bind(P, e, &p);
    /* phase_restore(ce, includeL = .false.) */
    memcpy(p.Fp, p.Fp0, 9 * sizeof(double)); memcpy(p.Fi, p.Fi0, 9 * sizeof(double));
    memcpy(p.S, p.S0, 9 * sizeof(double));
    memcpy(p.state0, p.xi0, 12 * sizeof(double)); memcpy(p.state0 + 12, p.gamma0, 12 * sizeof(double));
    memcpy(p.state, p.state0, sizeof(p.state));
    /* mechanical_partition (pass / isostrain with one constituent) */
    memcpy(p.F, F + 9 * e, 9 * sizeof(double));
    int ok = constitutive(m, c, &p, dt);
    memcpy(p.xi, p.state, 12 * sizeof(double)); memcpy(p.gamma, p.state + 12, 12 * sizeof(double));
    P->status[e] = ok ? 0 : 1;
    if (!ok) ill = 1;
    /* mechanical_homogenize: P = v P_phase, dPdF = v dPdF_phase with v = 1 */
    if (want_dPdF) {
#pragma omp atomic
      g_cnt_tangent++;
      tangent(m, c, &p, dt, p.dPdF);
    }
  }
  return ill;
}

void dgo_averages(int64_t n, const double* P, const double* dPdF,
                  double P_av[9], double C_volAvg[81], double C_minMaxAvg[81]) {
  double wgt = 1.0 / (double)n;
  for (int k = 0; k < 9; ++k) {
    double s = 0.0;
    for (int64_t e = 0; e < n; ++e) s += P[9 * e + k];
    P_av[k] = s * wgt;
  }
  if (!dPdF) return;
  double nmax = 0.0, nmin = DBL_MAX;
  int64_t imax = -1, imin = -1;
  for (int64_t e = 0; e < n; ++e) {
    double s = 0.0;
    for (int k = 0; k < 81; ++k) s += dPdF[81 * e + k] * dPdF[81 * e + k];
    if (nmax < s) { nmax = s; imax = e; }
    if (nmin > s) { nmin = s; imin = e; }
  }
  for (int k = 0; k < 81; ++k) {
    double mx = imax >= 0 ? dPdF[81 * imax + k] : 0.0;
    double mn = imin >= 0 ? dPdF[81 * imin + k] : DBL_MAX;
    C_minMaxAvg[k] = 0.5 * (mx + mn);
    double s = 0.0;
    for (int64_t e = 0; e < n; ++e) s += dPdF[81 * e + k];
    C_volAvg[k] = s * wgt;
  }
}
