/*
 * dgo_const.c -- oracle: dense FP64 helpers, crystal tables, rotations.
 * TEST INFRASTRUCTURE ONLY (see dgo.h).
 *
 * Follows (reference paths):
 *   src/math.f90:485-600   math_inv33 / math_invert33 (Cramer), math_invert (LU)
 *   src/math.f90:686-846   det33, 33to9, 3333to99, 99to3333 (MAPPLAIN row-major)
 *   src/math.f90:910-995   Voigt maps (MAPVOIGT 11,22,33,23,13,12)
 *   src/crystal.f90:41-63  cF <110>{111} slip systems
 *   src/crystal.f90:613-646, 1853-1890  cF slip-slip interaction types, buildInteraction
 *   src/crystal.f90:1353-1431, 1897-1961 Schmid matrices from normalised d (x) n
 *   src/crystal.f90:1680-1719 crystal_symmetrize_C66
 *   src/rotations.f90:289-330, 423-447 rotTensor2/4, qu2om (P = -1 convention)
 */
#include "dgo.h"
#include <math.h>
#include <string.h>
#include <float.h>

#define A33(A, i, j) (A)[(i) + 3 * (j)]

void dgo_material_default(dgo_material* m) {
  memset(m, 0, sizeof(*m));
  m->C11 = 106.75e9; m->C12 = 60.41e9; m->C44 = 28.34e9;
  m->xi_0 = 31.e6; m->xi_inf = 63.e6; m->h_0 = 75.e6; m->n = 20.0;
  m->dot_gamma_0 = 1.e-3; m->a = 2.25; m->c_1 = 0.0; m->c_2 = 1.0;
  const double h[7] = {1, 1, 1.4, 1.4, 1.4, 1.4, 1.4};
  memcpy(m->h_sl_sl, h, sizeof(h));
  m->atol_xi = 1.0; m->atol_gamma = 1.e-6;
  m->r_cutback_min = 1.e-3; m->r_cutback = 0.25; m->r_increase = 1.5; m->eps_rel_state = 1.e-6;
  m->N_iter_state_max = 20; m->N_iter_Lp_max = 40;
  m->r_linesearch_Lp = 0.5; m->eps_rel_Lp = 1.e-6; m->eps_abs_Lp = 1.e-8;
  m->f_update_jacobi_Lp = 1;
}

/* cF slip systems: direction (3) then plane normal (3), order of crystal.f90:41-63 */
static const int CF_SLIP[12][6] = {
  { 0, 1,-1,  1, 1, 1}, {-1, 0, 1,  1, 1, 1}, { 1,-1, 0,  1, 1, 1},
  { 0,-1,-1, -1,-1, 1}, { 1, 0, 1, -1,-1, 1}, {-1, 1, 0, -1,-1, 1},
  { 0,-1, 1,  1,-1,-1}, {-1, 0,-1,  1,-1,-1}, { 1, 1, 0,  1,-1,-1},
  { 0, 1, 1, -1, 1,-1}, { 1, 0,-1, -1, 1,-1}, {-1,-1, 0, -1, 1,-1}};

/* interaction type for (reacting row, acting column), octahedral block of
 * crystal.f90:615-626 (types 1 self, 2 coplanar, 3 collinear, 4 Hirth,
 * 5/6 glissile, 7 Lomer) */
static const int CF_INTERACT[12][12] = {
  {1,2,2,4,7,5,3,5,5,4,6,7}, {2,1,2,7,4,5,6,4,7,5,3,5}, {2,2,1,5,5,3,6,7,4,7,6,4},
  {4,7,6,1,2,2,4,6,7,3,5,5}, {7,4,6,2,1,2,5,3,5,6,4,7}, {5,5,3,2,2,1,7,6,4,6,7,4},
  {3,5,5,4,6,7,1,2,2,4,7,6}, {6,4,7,5,3,5,2,1,2,7,4,6}, {6,7,4,7,6,4,2,2,1,5,5,3},
  {4,6,7,3,5,5,4,7,6,1,2,2}, {5,3,5,6,4,7,7,4,6,2,1,2}, {7,6,4,6,7,4,5,5,3,2,2,1}};

static const int VOIGT[6][2] = {{0,0},{1,1},{2,2},{1,2},{0,2},{0,1}};

void dgo_consts_build(const dgo_material* m, dgo_consts* c) {
  memset(c, 0, sizeof(*c));
  for (int s = 0; s < 12; ++s) {
    double d[3], nn[3], ld = 0, ln = 0;
    for (int i = 0; i < 3; ++i) { d[i] = CF_SLIP[s][i]; nn[i] = CF_SLIP[s][3 + i]; }
    for (int i = 0; i < 3; ++i) { ld += d[i] * d[i]; ln += nn[i] * nn[i]; }
    ld = sqrt(ld); ln = sqrt(ln);
    for (int i = 0; i < 3; ++i) { d[i] /= ld; nn[i] /= ln; }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) c->P_sl[s][i + 3 * j] = d[i] * nn[j];
  }
  for (int r = 0; r < 12; ++r)
    for (int a = 0; a < 12; ++a) c->h[r][a] = m->h_sl_sl[CF_INTERACT[r][a] - 1];
  /* cubic symmetrised C66 */
  double* C66 = c->C66;
  C66[0 + 6 * 0] = C66[1 + 6 * 1] = C66[2 + 6 * 2] = m->C11;
  C66[0 + 6 * 1] = C66[0 + 6 * 2] = C66[1 + 6 * 2] = m->C12;
  C66[3 + 6 * 3] = C66[4 + 6 * 4] = C66[5 + 6 * 5] = m->C44;
  for (int i = 0; i < 6; ++i)
    for (int j = i + 1; j < 6; ++j) C66[j + 6 * i] = C66[i + 6 * j];
  /* math_Voigt66to3333_stiffness */
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      int a = VOIGT[i][0], b = VOIGT[i][1], cc = VOIGT[j][0], d = VOIGT[j][1];
      double v = C66[i + 6 * j];
      c->C[a + 3 * b + 9 * cc + 27 * d] = v;
      c->C[b + 3 * a + 9 * cc + 27 * d] = v;
      c->C[a + 3 * b + 9 * d + 27 * cc] = v;
      c->C[b + 3 * a + 9 * d + 27 * cc] = v;
    }
}

/* ------------------------------------------------------------------ 3x3 */
int dgo_invert33(const double A[9], double inv[9], double* det) {
  double I[9];
  I[0 + 3 * 0] =  A33(A,1,1) * A33(A,2,2) - A33(A,1,2) * A33(A,2,1);
  I[1 + 3 * 0] = -A33(A,1,0) * A33(A,2,2) + A33(A,1,2) * A33(A,2,0);
  I[2 + 3 * 0] =  A33(A,1,0) * A33(A,2,1) - A33(A,1,1) * A33(A,2,0);
  double D = A33(A,0,0) * I[0] + A33(A,0,1) * I[1] + A33(A,0,2) * I[2];
  if (fabs(D) <= DBL_MIN * 10.0) {
    for (int i = 0; i < 9; ++i) inv[i] = 0.0;
    if (det) *det = 0.0;
    return 1;
  }
  I[0 + 3 * 1] = -A33(A,0,1) * A33(A,2,2) + A33(A,0,2) * A33(A,2,1);
  I[1 + 3 * 1] =  A33(A,0,0) * A33(A,2,2) - A33(A,0,2) * A33(A,2,0);
  I[2 + 3 * 1] = -A33(A,0,0) * A33(A,2,1) + A33(A,0,1) * A33(A,2,0);
  I[0 + 3 * 2] =  A33(A,0,1) * A33(A,1,2) - A33(A,0,2) * A33(A,1,1);
  I[1 + 3 * 2] = -A33(A,0,0) * A33(A,1,2) + A33(A,0,2) * A33(A,1,0);
  I[2 + 3 * 2] =  A33(A,0,0) * A33(A,1,1) - A33(A,0,1) * A33(A,1,0);
  for (int i = 0; i < 9; ++i) inv[i] = I[i] / D;
  if (det) *det = D;
  return 0;
}

/* LU with partial pivoting (dgetrf + dgetri semantics): returns nonzero on a
 * zero pivot.  A, inv column-major n x n. */
int dgo_invert(int n, const double* A, double* inv) {
  double LU[900];
  int piv[30];
  if (n > 30) return -1;
  memcpy(LU, A, sizeof(double) * n * n);
  int err = 0;
  for (int k = 0; k < n; ++k) {
    int p = k; double mx = fabs(LU[k + n * k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(LU[i + n * k]) > mx) { mx = fabs(LU[i + n * k]); p = i; }
    piv[k] = p;
    if (LU[p + n * k] == 0.0) { err = 1; continue; }
    if (p != k)
      for (int j = 0; j < n; ++j) { double t = LU[k + n * j]; LU[k + n * j] = LU[p + n * j]; LU[p + n * j] = t; }
    for (int i = k + 1; i < n; ++i) {
      LU[i + n * k] /= LU[k + n * k];
      double l = LU[i + n * k];
      for (int j = k + 1; j < n; ++j) LU[i + n * j] -= l * LU[k + n * j];
    }
  }
  if (err) { for (int i = 0; i < n * n; ++i) inv[i] = 0.0; return 1; }
  /* solve LU X = P I column by column */
  for (int c = 0; c < n; ++c) {
    double x[30];
    for (int i = 0; i < n; ++i) x[i] = (i == c) ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k) { int p = piv[k]; if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; } }
    for (int i = 0; i < n; ++i) for (int j = 0; j < i; ++j) x[i] -= LU[i + n * j] * x[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) x[i] -= LU[i + n * j] * x[j];
      x[i] /= LU[i + n * i];
    }
    for (int i = 0; i < n; ++i) inv[i + n * c] = x[i];
  }
  return 0;
}

/* MAPPLAIN: 9-index = 3*row + col */
void dgo_3333to99(const double* T, double* M) {
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      int a = i / 3, b = i % 3, c = j / 3, d = j % 3;
      M[i + 9 * j] = T[a + 3 * b + 9 * c + 27 * d];
    }
}
void dgo_99to3333(const double* M, double* T) {
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      int a = i / 3, b = i % 3, c = j / 3, d = j % 3;
      T[a + 3 * b + 9 * c + 27 * d] = M[i + 9 * j];
    }
}

void dgo_mul3333xx33(const double A[81], const double B[9], double out[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) s += A[i + 3 * j + 9 * k + 27 * l] * B[k + 3 * l];
      out[i + 3 * j] = s;
    }
}

/* unit quaternion (w,x,y,z) to rotation matrix, DAMASK P = -1 convention:
 * the matrix is transposed relative to the P = +1 form and renormalised by
 * det^(1/3) */
void dgo_qu2om(const double q[4], double om[9]) {
  double qq = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double o[9];
  A33(o,0,0) = qq + 2.0 * q[1] * q[1];
  A33(o,1,1) = qq + 2.0 * q[2] * q[2];
  A33(o,2,2) = qq + 2.0 * q[3] * q[3];
  A33(o,0,1) = 2.0 * (q[1] * q[2] - q[0] * q[3]);
  A33(o,1,2) = 2.0 * (q[2] * q[3] - q[0] * q[1]);
  A33(o,2,0) = 2.0 * (q[3] * q[1] - q[0] * q[2]);
  A33(o,1,0) = 2.0 * (q[2] * q[1] + q[0] * q[3]);
  A33(o,2,1) = 2.0 * (q[3] * q[2] + q[0] * q[1]);
  A33(o,0,2) = 2.0 * (q[1] * q[3] + q[0] * q[2]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) om[i + 3 * j] = o[j + 3 * i];
  double det = om[0] * (om[4] * om[8] - om[7] * om[5]) - om[3] * (om[1] * om[8] - om[7] * om[2])
             + om[6] * (om[1] * om[5] - om[4] * om[2]);
  double s = pow(det, 1.0 / 3.0);
  for (int i = 0; i < 9; ++i) om[i] /= s;
}

/* passive: R T R^T ; active: R^T T R */
void dgo_rotate2(const double q[4], const double T[9], double out[9], int active) {
  double R[9], t[9];
  dgo_qu2om(q, R);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += (active ? R[k + 3 * i] : R[i + 3 * k]) * T[k + 3 * j];
      t[i + 3 * j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += t[i + 3 * k] * (active ? R[k + 3 * j] : R[j + 3 * k]);
      out[i + 3 * j] = s;
    }
}

void dgo_rotate4(const double q[4], const double T[81], double out[81], int active) {
  double om[9], R[9];
  dgo_qu2om(q, om);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) R[i + 3 * j] = active ? om[j + 3 * i] : om[i + 3 * j];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) {
    double s = 0.0;
    for (int m = 0; m < 3; ++m) for (int n = 0; n < 3; ++n) for (int o = 0; o < 3; ++o) for (int p = 0; p < 3; ++p)
      s += R[i + 3 * m] * R[j + 3 * n] * R[k + 3 * o] * R[l + 3 * p] * T[m + 3 * n + 9 * o + 27 * p];
    out[i + 3 * j + 9 * k + 27 * l] = s;
  }
}

/* ------------------------------------------------------------------ orientation output
 * Rotational part R of F (polar decomposition F = R U) in the closed form of the
 * reference (src/math.f90:1117-1156, invariants of C = F^T F and of U, Hoger &
 * Carlson 1984), then the crystal orientation written to the results:
 * quaternion of R^T (src/phase.f90:590, rotations.f90:518-546: trace branch, w >= 0,
 * P = -1 sign convention on the vector part, normalised). */
static double clip(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

void dgo_rotational_part(const double F[9], double R[9]) {
  double C[9], FF[9];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double c = 0.0, f = 0.0;
    for (int k = 0; k < 3; ++k) { c += F[k + 3 * i] * F[k + 3 * j]; f += F[i + 3 * k] * F[k + 3 * j]; }
    C[i + 3 * j] = c; FF[i + 3 * j] = f;
  }
  double I1 = C[0] + C[4] + C[8];
  double I2 = C[0] * C[4] + C[4] * C[8] + C[8] * C[0] - C[3] * C[3] - C[7] * C[7] - C[6] * C[6];
  double I3 = C[0] * (C[4] * C[8] - C[7] * C[5]) - C[3] * (C[1] * C[8] - C[7] * C[2]) + C[6] * (C[1] * C[5] - C[4] * C[2]);
  double trF = F[0] + F[4] + F[8], trFF = FF[0] + FF[4] + FF[8];
  double IF1 = trF, IF2 = 0.5 * (trF * trF - trFF);
  double x = pow(clip(I1 * I1 - 3.0 * I2, 0.0, INFINITY), 1.5);
  double lam[3];
  if (x != 0.0) {
    double Phi = acos(clip((I1 * I1 * I1 - 4.5 * I1 * I2 + 13.5 * I3) / x, -1.0, 1.0));
    for (int k = 0; k < 3; ++k) {
      double l = I1 + (2.0 * sqrt(clip(I1 * I1 - 3.0 * I2, 0.0, INFINITY))) *
                 cos((Phi - 6.283185307179586476925286766559 * (k + 1.0)) / 3.0);
      lam[k] = sqrt(clip(l, 0.0, INFINITY) / 3.0);
    }
  } else {
    for (int k = 0; k < 3; ++k) lam[k] = sqrt(I1 / 3.0);
  }
  double IU1 = lam[0] + lam[1] + lam[2];
  double IU2 = lam[0] * lam[1] + lam[1] * lam[2] + lam[2] * lam[0];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double FC = 0.0;
    for (int k = 0; k < 3; ++k) FC += F[i + 3 * k] * C[k + 3 * j];
    R[i + 3 * j] = (i == j ? IU1 * IF2 : 0.0) + (IU1 * IU1 - IU2) * F[i + 3 * j] - IU1 * IF1 * F[j + 3 * i]
                 + IU1 * FF[j + 3 * i] - FC;
  }
  double d = R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]);
  double s = pow(d, -1.0 / 3.0);
  for (int k = 0; k < 9; ++k) R[k] *= s;
}

void dgo_om2qu(const double om[9], double qu[4]) {
#define OM(i, j) om[(i - 1) + 3 * (j - 1)]
  double tr = OM(1, 1) + OM(2, 2) + OM(3, 3), s;
  if (tr > 0.0) {
    s = 0.5 / sqrt(tr + 1.0);
    qu[0] = 0.25 / s; qu[1] = (OM(3, 2) - OM(2, 3)) * s; qu[2] = (OM(1, 3) - OM(3, 1)) * s; qu[3] = (OM(2, 1) - OM(1, 2)) * s;
  } else if (OM(1, 1) > OM(2, 2) && OM(1, 1) > OM(3, 3)) {
    s = 2.0 * sqrt(1.0 + OM(1, 1) - OM(2, 2) - OM(3, 3));
    qu[0] = (OM(3, 2) - OM(2, 3)) / s; qu[1] = 0.25 * s; qu[2] = (OM(1, 2) + OM(2, 1)) / s; qu[3] = (OM(1, 3) + OM(3, 1)) / s;
  } else if (OM(2, 2) > OM(3, 3)) {
    s = 2.0 * sqrt(1.0 + OM(2, 2) - OM(1, 1) - OM(3, 3));
    qu[0] = (OM(1, 3) - OM(3, 1)) / s; qu[1] = (OM(1, 2) + OM(2, 1)) / s; qu[2] = 0.25 * s; qu[3] = (OM(2, 3) + OM(3, 2)) / s;
  } else {
    s = 2.0 * sqrt(1.0 + OM(3, 3) - OM(1, 1) - OM(2, 2));
    qu[0] = (OM(2, 1) - OM(1, 2)) / s; qu[1] = (OM(1, 3) + OM(3, 1)) / s; qu[2] = (OM(2, 3) + OM(3, 2)) / s; qu[3] = 0.25 * s;
  }
#undef OM
  if (copysign(1.0, qu[0]) < 0.0) for (int k = 0; k < 4; ++k) qu[k] = -qu[k];
  for (int k = 1; k < 4; ++k) if (qu[k] != 0.0) qu[k] = -qu[k];           /* P = -1 */
  double n = sqrt(qu[0] * qu[0] + qu[1] * qu[1] + qu[2] * qu[2] + qu[3] * qu[3]);
  for (int k = 0; k < 4; ++k) qu[k] /= n;
}

/* O written for a point: quaternion of (rotational part of Fe)^T */
void dgo_orientation_output(const double Fe[9], double qu[4]) {
  double R[9], Rt[9];
  dgo_rotational_part(Fe, R);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Rt[i + 3 * j] = R[j + 3 * i];
  dgo_om2qu(Rt, qu);
}
