// ref_stiffness.cpp -- reference stiffness C_minMaxAvg at F = I, dt = 0, evaluated
// with the reference's literal FP64 operation order (host, no FMA contraction).
//
// Why: Spectral::constitutive_response (reference src/grid/spectral.cpp:189-214)
// takes C_minMaxAvg = (dPdF[argmax |dPdF|_F] + dPdF[argmin |dPdF|_F]) / 2 over all
// cells, and MechSolverBasic::init (mech_solver_basic.cpp:95-106) turns the value
// at F = I into the Gamma operator's reference stiffness C_ref.  At F = I every
// cubic grain has the same Frobenius norm of its rotated stiffness, so the picks
// are decided by FP64 rounding (spread ~4e-15 relative).  Reproducing the
// reference's Gamma operator therefore needs the reference's rounding: this file
// evaluates the dt = 0 response and tangent of one representative cell per
// material with the operation order of the Fortran core
// (phase_mechanical.f90:380-604 integrateStress, :1137-1258 phase_mechanical_dPdF,
// phase_mechanical_elastic.f90:157-195 Hooke, math.f90:491-545 Cramer inverse,
// rotations.f90:423-447 qu2om), including Fi = O (V_e^-1) O^T with V_e = I.
// All cells of a material share their state at F = I, so the per-cell scan of
// the reference reduces to one norm per material and the first index of ties.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace dgx_ref {

static void mm(const double* A, const double* B, double* C) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += A[i + 3 * k] * B[k + 3 * j];
      t[i + 3 * j] = s;
    }
  std::memcpy(C, t, sizeof(t));
}
static void tr(const double* A, double* T) {
  double t[9];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) t[i + 3 * j] = A[j + 3 * i];
  std::memcpy(T, t, sizeof(t));
}
static bool inv33(const double* A, double* inv) {
  double I[9];
  I[0] = A[4] * A[8] - A[7] * A[5];
  I[1] = -A[1] * A[8] + A[7] * A[2];
  I[2] = A[1] * A[5] - A[4] * A[2];
  double D = A[0] * I[0] + A[3] * I[1] + A[6] * I[2];
  if (std::fabs(D) <= DBL_MIN * 10.0) { for (int k = 0; k < 9; ++k) inv[k] = 0.0; return false; }
  I[3] = -A[3] * A[8] + A[6] * A[5];
  I[4] = A[0] * A[8] - A[6] * A[2];
  I[5] = -A[0] * A[5] + A[3] * A[2];
  I[6] = A[3] * A[7] - A[6] * A[4];
  I[7] = -A[0] * A[7] + A[6] * A[1];
  I[8] = A[0] * A[4] - A[3] * A[1];
  for (int k = 0; k < 9; ++k) inv[k] = I[k] / D;
  return true;
}
static double det33(const double* m) {
  return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) + m[6] * (m[1] * m[5] - m[4] * m[2]);
}

void qu2om_ref(const double* q, double* om) {
  double qq = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double o[9];
  o[0] = qq + 2.0 * q[1] * q[1];
  o[4] = qq + 2.0 * q[2] * q[2];
  o[8] = qq + 2.0 * q[3] * q[3];
  o[3] = 2.0 * (q[1] * q[2] - q[0] * q[3]);
  o[7] = 2.0 * (q[2] * q[3] - q[0] * q[1]);
  o[2] = 2.0 * (q[3] * q[1] - q[0] * q[2]);
  o[1] = 2.0 * (q[2] * q[1] + q[0] * q[3]);
  o[5] = 2.0 * (q[3] * q[2] + q[0] * q[1]);
  o[6] = 2.0 * (q[1] * q[3] + q[0] * q[2]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) om[i + 3 * j] = o[j + 3 * i];
  double s = std::pow(det33(om), 1.0 / 3.0);
  for (int i = 0; i < 9; ++i) om[i] /= s;
}

struct Stiff { double C66[36]; double C[81]; };

static void stiffness(double C11, double C12, double C44, Stiff* st) {
  std::memset(st, 0, sizeof(*st));
  double* c = st->C66;
  c[0] = c[7] = c[14] = C11;
  c[6] = c[12] = c[13] = C12;
  c[21] = c[28] = c[35] = C44;
  for (int i = 0; i < 6; ++i) for (int j = i + 1; j < 6; ++j) c[j + 6 * i] = c[i + 6 * j];
  const int V[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) {
    int a = V[i][0], b = V[i][1], cc = V[j][0], d = V[j][1];
    double v = c[i + 6 * j];
    st->C[a + 3 * b + 9 * cc + 27 * d] = v; st->C[b + 3 * a + 9 * cc + 27 * d] = v;
    st->C[a + 3 * b + 9 * d + 27 * cc] = v; st->C[b + 3 * a + 9 * d + 27 * cc] = v;
  }
}

// Hooke S and dS/dFe for general Fi
static void hooke(const Stiff& st, const double* Fe, const double* Fi, double* S, double* dS_dFe) {
  double E[9], FeT[9], t[9], FiT[9];
  tr(Fe, FeT); mm(FeT, Fe, E);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) E[i + 3 * j] = 0.5 * (E[i + 3 * j] - (i == j ? 1.0 : 0.0));
  tr(Fi, FiT); mm(FiT, E, t); mm(t, Fi, t);
  double e6[6] = {t[0], t[4], t[8], 2.0 * t[5], 2.0 * t[2], 2.0 * t[3]};
  double s6[6];
  for (int i = 0; i < 6; ++i) { double s = 0.0; for (int j = 0; j < 6; ++j) s += st.C66[i + 6 * j] * e6[j]; s6[i] = s; }
  S[0] = s6[0]; S[4] = s6[1]; S[8] = s6[2];
  S[5] = S[7] = s6[3]; S[2] = S[6] = s6[4]; S[1] = S[3] = s6[5];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double Cij[9], a[9], b[9];
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) Cij[k + 3 * l] = st.C[i + 3 * j + 9 * k + 27 * l];
    mm(Fi, Cij, a); mm(a, FiT, a); mm(Fe, a, b);
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) dS_dFe[i + 3 * j + 9 * k + 27 * l] = b[k + 3 * l];
  }
}

// dPdF of one cell at F = I, dt = 0, with norm^2 (sum of squares in storage order)
static double cell_tangent(const Stiff& st, const double* q, double* dPdF) {
  double R[9], RT[9], Fi0[9], I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  qu2om_ref(q, R);
  tr(R, RT);
  mm(R, RT, Fi0);                                      // O.rotate(inv(V_e)), V_e = I
  // integrateStress(F = I, Fp0 = R, Fi0, dt = 0): converges in the first Lp iteration
  double invFp_cur[9], invFi_cur[9], A[9], invFi_new[9], Fi_new[9], Fe[9], S[9], dS_dFe[81], B[9];
  inv33(R, invFp_cur);
  inv33(Fi0, invFi_cur);
  mm(I, invFp_cur, A);
  double t[9];
  for (int k = 0; k < 9; ++k) t[k] = I[k] - 0.0 * 0.0;
  mm(invFi_cur, t, invFi_new);
  inv33(invFi_new, Fi_new);
  for (int k = 0; k < 9; ++k) B[k] = I[k] - 0.0 * 0.0;
  mm(A, B, Fe); mm(Fe, invFi_new, Fe);
  hooke(st, Fe, Fi_new, S, dS_dFe);
  double invFp_new[9], Fp_new[9], Fp[9], FeOut[9];
  mm(invFp_cur, B, invFp_new);
  inv33(invFp_new, Fp_new);
  double s = std::pow(det33(Fp_new), 1.0 / 3.0);
  for (int k = 0; k < 9; ++k) Fp[k] = Fp_new[k] / s;
  double a1[9];
  mm(I, invFp_new, a1); mm(a1, invFi_new, FeOut);
  // phase_mechanical_dPdF with dt = 0 (dLp/dS terms carry a factor dt; M = I exactly)
  double dSdFe[81], Sdev[9];
  hooke(st, FeOut, Fi_new, Sdev, dSdFe);
  double invFp[9], invFi[9];
  inv33(Fp, invFp); inv33(Fi_new, invFi);
  double t1[9], aa[9];
  mm(invFp, invFi, aa); tr(aa, t1);
  double dSdF[81];
  for (int o = 0; o < 3; ++o) for (int p = 0; p < 3; ++p) {
    double D[9], r[9];
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) D[k + 3 * l] = dSdFe[p + 3 * o + 9 * k + 27 * l];
    mm(D, t1, r);
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) dSdF[p + 3 * o + 9 * k + 27 * l] = r[k + 3 * l];
  }
  double invFpT[9], u1[9], u2[9], u3[9], w[9], wT[9];
  tr(invFp, invFpT);
  mm(S, invFpT, u1);
  mm(I, invFp, u2);
  mm(u2, S, u3);
  for (int k = 0; k < 81; ++k) dPdF[k] = 0.0;
  mm(invFp, u1, w); tr(w, wT);
  for (int q2 = 0; q2 < 3; ++q2)
    for (int j = 0; j < 3; ++j) for (int l = 0; l < 3; ++l) dPdF[q2 + 3 * j + 9 * q2 + 27 * l] = wT[j + 3 * l];
  for (int o = 0; o < 3; ++o) for (int pp = 0; pp < 3; ++pp) {
    double dS[9], Y[9];
    for (int k = 0; k < 9; ++k) dS[k] = dSdF[k + 9 * (pp + 3 * o)];
    mm(u2, dS, Y); mm(Y, invFpT, Y);
    // the dFp^-1/dF terms vanish identically at dt = 0 (signed zeros only)
    for (int k = 0; k < 9; ++k) dPdF[k + 9 * (pp + 3 * o)] += 0.0 + Y[k] + 0.0;
  }
  double n2 = 0.0;
  for (int k = 0; k < 81; ++k) n2 += dPdF[k] * dPdF[k];
  return n2;
}

}  // namespace dgx_ref

// C_minMaxAvg at F = I (fresh state), reference selection rule over cells in index order.
extern "C" int dgx_reference_stiffness(double C11, double C12, double C44, int n_mat, const double* q,
                                       const int32_t* material_at, int64_t N, double* C_minMaxAvg) {
  using namespace dgx_ref;
  Stiff st;
  stiffness(C11, C12, C44, &st);
  std::vector<double> norms(n_mat, 0.0), dP((size_t)81 * n_mat, 0.0);
  std::vector<char> used(n_mat, 0);
  for (int64_t e = 0; e < N; ++e) {
    int m = material_at[e];
    if (m < 0 || m >= n_mat) m = 0;
    used[m] = 1;
  }
  for (int m = 0; m < n_mat; ++m)
    if (used[m]) norms[m] = cell_tangent(st, q + 4 * m, dP.data() + 81 * m);
  double nmax = 0.0, nmin = DBL_MAX;
  int imax = -1, imin = -1;
  for (int64_t e = 0; e < N; ++e) {
    int m = material_at[e];
    if (m < 0 || m >= n_mat) m = 0;
    double s = norms[m];
    if (nmax < s) { nmax = s; imax = m; }
    if (nmin > s) { nmin = s; imin = m; }
  }
  for (int k = 0; k < 81; ++k) {
    double mx = imax >= 0 ? dP[81 * imax + k] : 0.0;
    double mn = imin >= 0 ? dP[81 * imin + k] : DBL_MAX;
    C_minMaxAvg[k] = 0.5 * (mx + mn);
  }
  return imax >= 0 && imin >= 0 ? 0 : 1;
}
