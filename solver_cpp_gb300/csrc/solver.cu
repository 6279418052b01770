// solver.cu -- host side of the GB300 spectral-basic solver and its C ABI.
//
// Reference behaviour (reference paths):
//   src/grid/mech_solver_basic.cpp:19-339  init, calculate_solution, forward, converged, form_residual
//   src/grid/mech_base.cpp:213-300, 479-497 forward_field, masked compliance, rate
//   src/grid/damask_grid.cpp:19-196        forward_fields, solve_fields, forward_time, load-case loop
//   src/grid/spectral.cpp:132-219          constitutive_response (averages, lab rotation of P_av)
// Nonlinear solver: PETSc SNES NGMRES (third-party, PETSc 3.12-3.20; absent from the
// reference tree) restated from its published algorithm with PETSc's defaults
// (m = 30, difference restart/selection, gammaA = gammaC = 2, epsilonB = 0.1,
// deltaB = 0.9, restart_it = 2, basic line search for x^M, max_it = 50).
// All long vectors (9 N doubles) live in HBM; dot products and norms are fused,
// fixed-order two-stage reductions, so every run is bitwise reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgx.h"
#include "dgx_internal.cuh"
#include "rve.cuh"
#include "spectral.cuh"


using namespace dgx;

// ref_stiffness.cpp
extern "C" int dgx_reference_stiffness(double C11, double C12, double C44, int n_mat, const double* q,
                                       const int32_t* material_at, int64_t N, double* C_minMaxAvg);

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;
namespace dgx {
void set_err(const char* fmt, ...) {
  char buf[512];
  va_list ap; va_start(ap, fmt); vsnprintf(buf, sizeof(buf), fmt, ap); va_end(ap);
  g_err = buf;
}
}  // namespace dgx
extern "C" const char* dgx_last_error(void) { return g_err.c_str(); }

// ------------------------------------------------------------------ vector kernels
namespace dgx {

__global__ void k_init_points(PointState ps, const int32_t* __restrict__ mat, const double* __restrict__ R,
                              int nmat, double xi0) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ps.n) return;
  int m = mat[e];
  if (m < 0 || m >= nmat) m = 0;
  const double* r = R + 9 * m;
  for (int k = 0; k < 9; ++k) {
    double I = (k % 4) == 0 ? 1.0 : 0.0;
    ps.F[k * ps.ld + e] = I; ps.F0[k * ps.ld + e] = I;
    ps.Fp[k * ps.ld + e] = r[k]; ps.Fp0[k * ps.ld + e] = r[k];
    ps.Fe[k * ps.ld + e] = r[(k / 3) + 3 * (k % 3)];
    ps.Lp[k * ps.ld + e] = 0.0; ps.Lp0[k * ps.ld + e] = 0.0;
    ps.S[k * ps.ld + e] = 0.0; ps.S0[k * ps.ld + e] = 0.0;
  }
  for (int i = 0; i < 24; ++i) {
    double v = i < 12 ? xi0 : 0.0;
    ps.st[i * ps.ld + e] = v; ps.st0[i * ps.ld + e] = v;
  }
  ps.status[e] = 0;
}

// AoS (w per point) <-> planar (ld)
__global__ void k_aos2planar(const double* __restrict__ a, int w, int64_t n, double* __restrict__ p, int64_t ld) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * w) return;
  int64_t e = t / w; int c = (int)(t - e * w);
  p[c * ld + e] = a[t];
}
__global__ void k_planar2aos(const double* __restrict__ p, int64_t ld, int w, int64_t n, double* __restrict__ a) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * w) return;
  int64_t e = t / w; int c = (int)(t - e * w);
  a[t] = p[c * ld + e];
}

__global__ void k_fill_identity(double* __restrict__ X, int64_t n) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 9 * n) return;
  int c = (int)(t / n);
  X[t] = (c % 4) == 0 ? 1.0 : 0.0;
}

// z = x + a * y
__global__ void k_axpy(double* __restrict__ z, const double* __restrict__ x, double a, const double* __restrict__ y, int64_t n) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) z[t] = x[t] + a * y[t];
}

// XA = (1 - sum beta) XM + sum_i beta_i Xdot_i
__global__ void k_combine(double* __restrict__ XA, const double* __restrict__ XM, VecList Xd, int l, double c0,
                          const double* __restrict__ beta, int64_t n) {
  __shared__ double sb[32];
  if (threadIdx.x < 32) sb[threadIdx.x] = threadIdx.x < l ? beta[threadIdx.x] : 0.0;
  __syncthreads();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double v = XM[t] * c0;
    for (int i = 0; i < l; ++i) v += sb[i] * Xd.v[i][t];
    XA[t] = v;
  }
}

// K reductions in one pass: mode 0: sum a*v_k ; mode 1: sum (v_k - a)^2 ; one "a" vector
// shared by all k (plus an optional second anchor b for the first K2 entries: sum b*v_k)
__global__ void k_multi(int mode, const double* __restrict__ a, const double* __restrict__ b, VecList vl, int K,
                        int K2, int64_t n, double* __restrict__ part) {
  double acc[32], acc2[32];
  for (int k = 0; k < K; ++k) { acc[k] = 0.0; acc2[k] = 0.0; }
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double av = a[t];
    double bv = b ? b[t] : 0.0;
    for (int k = 0; k < K; ++k) {
      double x = vl.v[k][t];
      if (mode == 0) acc[k] = fma(av, x, acc[k]);
      else { double d = x - av; acc[k] = fma(d, d, acc[k]); }
      if (k < K2) acc2[k] = fma(bv, x, acc2[k]);
    }
  }
  __shared__ double red[RB];
  int KT = K + K2;
  for (int k = 0; k < KT; ++k) {
    red[threadIdx.x] = k < K ? acc[k] : acc2[k - K];
    __syncthreads();
    for (int s = RB / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x * KT + k] = red[0];
    __syncthreads();
  }
}

// one block (warp) per component, fixed summation order
__global__ void k_multi_finish(const double* __restrict__ part, int nb, int K, double* __restrict__ out) {
  int k = blockIdx.x;
  if (k >= K) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) s += part[b * K + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) out[k] = s;
}

// forward_field: F = last + rate*dt - (avg - aim)   (two launches: sum, then shift)
__global__ void k_forward_field(double* __restrict__ F, const double* __restrict__ last, const double* __restrict__ rate,
                                double dt, int64_t n9) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n9) F[t] = last[t] + rate[t] * dt;
}
__global__ void k_shift_planes(double* __restrict__ F, const double* __restrict__ diff, int64_t n) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 9 * n) return;
  F[t] -= diff[t / n];
}
// plane sums (9 components) -> part[b*9+c]
__global__ void k_plane_sums(const double* __restrict__ F, int64_t n, double* __restrict__ part) {
  __shared__ double red[RB];
  for (int c = 0; c < 9; ++c) {
    double s = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
      s += F[c * n + t];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = RB / 2; k > 0; k >>= 1) {
      if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x * 9 + c] = red[0];
    __syncthreads();
  }
}
// rate: heterogeneous (F - F0)/dt, or the average rate in every cell
__global__ void k_rate(double* __restrict__ rate, const double* __restrict__ F0, const double* __restrict__ F, double dt,
                       int hetero, double r0, double r1, double r2, double r3, double r4, double r5, double r6,
                       double r7, double r8, int64_t n) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 9 * n) return;
  if (hetero) rate[t] = (F[t] - F0[t]) / dt;
  else {
    int c = (int)(t / n);
    double r[9] = {r0, r1, r2, r3, r4, r5, r6, r7, r8};
    rate[t] = r[c];
  }
}


// ------------------------------------------------------------------ small host math
void mm3(const double* A, const double* B, double* C) {
  double t[9];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double s = 0; for (int k = 0; k < 3; ++k) s += A[i + 3 * k] * B[k + 3 * j]; t[i + 3 * j] = s;
  }
  memcpy(C, t, sizeof(t));
}
void qu2om(const double* q, double* om) {
  double qq = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double o[9];
  o[0] = qq + 2.0 * q[1] * q[1]; o[4] = qq + 2.0 * q[2] * q[2]; o[8] = qq + 2.0 * q[3] * q[3];
  o[3] = 2.0 * (q[1] * q[2] - q[0] * q[3]); o[7] = 2.0 * (q[2] * q[3] - q[0] * q[1]); o[2] = 2.0 * (q[3] * q[1] - q[0] * q[2]);
  o[1] = 2.0 * (q[2] * q[1] + q[0] * q[3]); o[5] = 2.0 * (q[3] * q[2] + q[0] * q[1]); o[6] = 2.0 * (q[1] * q[3] + q[0] * q[2]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) om[i + 3 * j] = o[j + 3 * i];   // P = -1: transpose
  double det = om[0] * (om[4] * om[8] - om[7] * om[5]) - om[3] * (om[1] * om[8] - om[7] * om[2]) + om[6] * (om[1] * om[5] - om[4] * om[2]);
  double s = std::pow(det, 1.0 / 3.0);
  for (int k = 0; k < 9; ++k) om[k] /= s;
}
void rotate2(const double* q, const double* T, double* out, bool active) {
  double R[9], t[9];
  qu2om(q, R);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double s = 0; for (int k = 0; k < 3; ++k) s += (active ? R[k + 3 * i] : R[i + 3 * k]) * T[k + 3 * j]; t[i + 3 * j] = s;
  }
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
    double s = 0; for (int k = 0; k < 3; ++k) s += t[i + 3 * k] * (active ? R[k + 3 * j] : R[j + 3 * k]); out[i + 3 * j] = s;
  }
}
void rotate4(const double* q, const double* T, double* out) {
  double R[9];
  qu2om(q, R);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) {
    double s = 0.0;
    for (int m = 0; m < 3; ++m) for (int n = 0; n < 3; ++n) for (int o = 0; o < 3; ++o) for (int p = 0; p < 3; ++p)
      s += R[i + 3 * m] * R[j + 3 * n] * R[k + 3 * o] * R[l + 3 * p] * T[m + 3 * n + 9 * o + 27 * p];
    out[i + 3 * j + 9 * k + 27 * l] = s;
  }
}
bool invert_n(int n, const double* A, double* inv) {
  std::vector<double> LU(A, A + n * n);
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k; double mx = std::fabs(LU[k + n * k]);
    for (int i = k + 1; i < n; ++i) if (std::fabs(LU[i + n * k]) > mx) { mx = std::fabs(LU[i + n * k]); p = i; }
    piv[k] = p;
    if (LU[p + n * k] == 0.0) return false;
    if (p != k) for (int j = 0; j < n; ++j) std::swap(LU[k + n * j], LU[p + n * j]);
    for (int i = k + 1; i < n; ++i) {
      LU[i + n * k] /= LU[k + n * k];
      for (int j = k + 1; j < n; ++j) LU[i + n * j] -= LU[i + n * k] * LU[k + n * j];
    }
  }
  for (int c = 0; c < n; ++c) {
    std::vector<double> x(n, 0.0); x[c] = 1.0;
    for (int k = 0; k < n; ++k) if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int i = 0; i < n; ++i) for (int j = 0; j < i; ++j) x[i] -= LU[i + n * j] * x[j];
    for (int i = n - 1; i >= 0; --i) { for (int j = i + 1; j < n; ++j) x[i] -= LU[i + n * j] * x[j]; x[i] /= LU[i + n * i]; }
    for (int i = 0; i < n; ++i) inv[i + n * c] = x[i];
  }
  return true;
}
// MechBase::calculate_masked_compliance; mask column-major, 1 = 'x' (not prescribed)
bool masked_compliance(const double* C, const double* q, const int* mask, double* S) {
  int act[9], nred = 0;
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) { act[3 * a + b] = !mask[a + 3 * b]; nred += act[3 * a + b]; }
  double t99[81] = {0};
  bool ok = true;
  if (nred > 0) {
    double rot[81], c99[81];
    rotate4(q, C, rot);
    for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
      c99[i + 9 * j] = rot[(i / 3) + 3 * (i % 3) + 9 * (j / 3) + 27 * (j % 3)];
    std::vector<double> cred(nred * nred), sred(nred * nred);
    int idx = 0;
    for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
      if (act[i] && act[j]) { cred[(idx / nred) + nred * (idx % nred)] = c99[i + 9 * j]; ++idx; }
    ok = invert_n(nred, cred.data(), sred.data());
    idx = 0;
    for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
      if (act[i] && act[j]) { t99[i + 9 * j] = sred[(idx / nred) + nred * (idx % nred)]; ++idx; }
  }
  for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
    S[(i / 3) + 3 * (i % 3) + 9 * (j / 3) + 27 * (j % 3)] = t99[i + 9 * j];
  return ok;
}

// minimum-norm least squares H x = b (l x l), one-sided Jacobi SVD, cutoff eps * s_max
void lsq_svd(int l, const double* H, double* b) {
  std::vector<double> U(H, H + l * l), V(l * l, 0.0), sv(l), x(l);
  for (int i = 0; i < l; ++i) V[i + l * i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < l - 1; ++p)
      for (int q = p + 1; q < l; ++q) {
        double a = 0, bb = 0, c = 0;
        for (int i = 0; i < l; ++i) { a += U[i + l * p] * U[i + l * p]; bb += U[i + l * q] * U[i + l * q]; c += U[i + l * p] * U[i + l * q]; }
        if (c == 0.0) continue;
        double ratio = std::fabs(c) / std::sqrt(a * bb);
        off = std::max(off, ratio);
        if (ratio < 1e-15) continue;
        double zeta = (bb - a) / (2.0 * c);
        double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double cs = 1.0 / std::sqrt(1.0 + t * t), sn = cs * t;
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
    double n2 = 0.0; for (int i = 0; i < l; ++i) n2 += U[i + l * j] * U[i + l * j];
    sv[j] = std::sqrt(n2); smax = std::max(smax, sv[j]);
  }
  double cut = 2.220446049250313e-16 * smax;
  for (int j = 0; j < l; ++j) {
    double c = 0.0;
    if (sv[j] > cut && sv[j] > 0.0) { for (int i = 0; i < l; ++i) c += U[i + l * j] / sv[j] * b[i]; c /= sv[j]; }
    x[j] = c;
  }
  for (int i = 0; i < l; ++i) { double v = 0.0; for (int j = 0; j < l; ++j) v += V[i + l * j] * x[j]; b[i] = v; }
}

const int CF_SLIP[12][6] = {
  { 0, 1,-1,  1, 1, 1}, {-1, 0, 1,  1, 1, 1}, { 1,-1, 0,  1, 1, 1},
  { 0,-1,-1, -1,-1, 1}, { 1, 0, 1, -1,-1, 1}, {-1, 1, 0, -1,-1, 1},
  { 0,-1, 1,  1,-1,-1}, {-1, 0,-1,  1,-1,-1}, { 1, 1, 0,  1,-1,-1},
  { 0, 1, 1, -1, 1,-1}, { 1, 0,-1, -1, 1,-1}, {-1,-1, 0, -1, 1,-1}};

MatParams make_params(const dgx_material& m) {
  MatParams p;
  memset(&p, 0, sizeof(p));
  double C66[36] = {0};
  C66[0] = C66[7] = C66[14] = m.C11;
  C66[6] = C66[12] = C66[13] = m.C12;
  C66[21] = C66[28] = C66[35] = m.C44;
  for (int i = 0; i < 6; ++i) for (int j = i + 1; j < 6; ++j) C66[j + 6 * i] = C66[i + 6 * j];
  memcpy(p.C66, C66, sizeof(C66));
  for (int s = 0; s < 12; ++s) {
    double d[3], n[3], ld = 0, ln = 0;
    for (int i = 0; i < 3; ++i) { d[i] = CF_SLIP[s][i]; n[i] = CF_SLIP[s][3 + i]; ld += d[i] * d[i]; ln += n[i] * n[i]; }
    ld = std::sqrt(ld); ln = std::sqrt(ln);
    for (int i = 0; i < 3; ++i) { d[i] /= ld; n[i] /= ln; }
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) p.P[s][i + 3 * j] = d[i] * n[j];
  }
  p.xi_inf = m.xi_inf;
  p.h0 = m.h_0 * (1.0 + m.c_1 * std::pow(0.0, m.c_2));     // no twins: sum f = 0
  for (int t = 0; t < 7; ++t) p.h0h[t] = p.h0 * m.dot_gamma_0 * m.h_sl_sl[t];
  p.n = m.n; p.gdot0 = m.dot_gamma_0; p.a = m.a; p.c1 = m.c_1; p.c2 = m.c_2;
  p.atol_xi = m.atol_xi; p.atol_gamma = m.atol_gamma;
  p.r_cutback_min = m.r_cutback_min; p.r_cutback = m.r_cutback; p.r_increase = m.r_increase;
  p.eps_rel_state = m.eps_rel_state; p.r_linesearch_Lp = m.r_linesearch_Lp;
  p.eps_rel_Lp = m.eps_rel_Lp; p.eps_abs_Lp = m.eps_abs_Lp;
  p.N_iter_state_max = m.N_iter_state_max; p.N_iter_Lp_max = m.N_iter_Lp_max;
  p.f_update_jacobi_Lp = m.f_update_jacobi_Lp < 1 ? 1 : m.f_update_jacobi_Lp;
  p.n_int = (m.n == std::floor(m.n) && m.n >= 1 && m.n <= 64) ? (int)m.n : -1;
  p.C11mC12 = m.C11 - m.C12; p.C12 = m.C12; p.C44 = m.C44;
  p.hC11mC12 = 0.5 * p.C11mC12; p.hC12 = 0.5 * m.C12;
  p.ngdot0 = m.n * m.dot_gamma_0; p.rxi_inf = 1.0 / m.xi_inf;
  p.pval = std::fabs(p.P[0][1]);                       // (1/sqrt2)(1/sqrt3), as the host computed P
  p.ngdot0_p = p.ngdot0 / p.pval;
  p.pgdot0 = p.pval * m.dot_gamma_0;
  p.pgdot0_sq = p.pgdot0 * p.pgdot0;
  p.eps_rel_Lp2 = m.eps_rel_Lp * m.eps_rel_Lp; p.eps_abs_Lp2 = m.eps_abs_Lp * m.eps_abs_Lp;
  double aq = 4.0 * m.a;
  p.a_quarters = (aq == std::floor(aq) && aq >= 1 && aq <= 256) ? (int)aq : -1;
  for (int t = 0; t < 7; ++t) p.h0h_f[t] = (float)p.h0h[t];
  p.gdot0_f = (float)p.gdot0;
  p.n_f = (float)p.n; p.rpval_f = (float)(1.0 / p.pval); p.pgdot0_f = (float)p.pgdot0;
  p.pval_f = (float)p.pval; p.hC11mC12_f = (float)p.hC11mC12; p.hC12_f = (float)p.hC12; p.C44_f = (float)p.C44;
  return p;
}

}  // namespace


namespace dgx {

template <typename T>
dgx_status dalloc(dgx_rve* r, T** p, size_t count) {
  if (r->dry) { r->bytes += (int64_t)(count * sizeof(T)); *p = nullptr; return DGX_OK; }
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) { set_err("cudaMalloc(%zu): %s", count * sizeof(T), cudaGetErrorString(e)); return DGX_ERR_NOMEM; }
  r->allocs.push_back(v);
  r->bytes += (int64_t)(count * sizeof(T));
  *p = (T*)v;
  return DGX_OK;
}


// host tail of Spectral::constitutive_response (spectral.cpp:132-219) once P_av and
// the terminally-ill flag are on the host
dgx_status post_constitutive(dgx_rve* r, int ill, bool want_tangent) {
  r->tangent_fresh = false;
  if (ill) r->terminally_ill = 1;
  if (want_tangent) TRY(ensure_tangent(r));
  if (!(r->rot_q[0] == 1.0 && r->rot_q[1] == 0.0 && r->rot_q[2] == 0.0 && r->rot_q[3] == 0.0)) {
    double t[9];
    rotate2(r->rot_q, r->P_av, t, false);
    memcpy(r->P_av, t, sizeof(t));
  }
  return DGX_OK;
}

// Spectral::constitutive_response on the device for one RVE: P (ps.P), P_av (host),
// optional tangent.  Used by the initial reference-stiffness pass and the boundary
// call; the solver's residual evaluations go through the batched executor.
dgx_status constitutive_response(dgx_rve* r, const double* X, double dt, bool want_tangent) {
  r->n_eval++;
  CK(cudaMemsetAsync(r->d_ill, 0, sizeof(int), r->st));
  if (r->timing) cudaEventRecord(r->ev[0], r->st);
  launch_constitutive(r->mp, r->ps, X, r->N, dt, r->d_Ppart, r->d_ill, r->d_cnt, r->st, r->cons_block);
  if (r->timing) cudaEventRecord(r->ev[1], r->st);
  launch_pav_finish(r->d_Ppart, r->nb_cons, r->wgt, r->d_Pav, r->st);
  r->n_launch += 2;
  r->tangent_dt = dt;
  int ill = 0;
  CK(d2h(r, r->P_av, r->d_Pav, 9 * sizeof(double)));
  CK(d2h(r, &ill, r->d_ill, sizeof(int)));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  if (r->timing) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]); r->t_ms[0] += ms; r->t_n[0]++;
  }
  return post_constitutive(r, ill, want_tangent);
}

// make C_volAvg / C_minMaxAvg current (lazy tangent of the last evaluation)
dgx_status ensure_tangent(dgx_rve* r) {
  if (r->tangent_fresh) return DGX_OK;
  if (r->timing) cudaEventRecord(r->ev[4], r->st);
  launch_tangent(r->mp, r->ps, r->tangent_dt, r->d_dPdF, r->N, r->d_tpart, r->st);
  if (r->timing) cudaEventRecord(r->ev[5], r->st);
  launch_tangent_finish(r->d_tpart, r->nb_tan, r->wgt, r->d_Cvol, r->d_Cmm, r->st);
  r->n_launch += 2;
  r->n_tangent++;
  CK(d2h(r, r->C_volAvg, r->d_Cvol, 81 * sizeof(double)));
  CK(d2h(r, r->C_minMaxAvg, r->d_Cmm, 81 * sizeof(double)));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  if (r->timing) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev[4], r->ev[5]); r->t_ms[2] += ms; r->t_n[2]++;
  }
  r->tangent_fresh = true;
  return DGX_OK;
}

GammaArgs gamma_args(dgx_rve* r, bool gamma, bool div) {
  GammaArgs ga{};
  ga.xi_x = r->d_xi_x; ga.xi_y = r->d_xi_y; ga.xi_z = r->d_xi_z;
  for (int i = 0; i < 3; ++i) {
    ga.resc[i] = r->geom[i] / r->scaled[i];
    ga.fw[i] = r->d_fw[i];
    ga.fw_h4[i] = 4.0 * r->geom[i] / r->cells[i];
  }
  ga.C_ref = r->d_Cref; ga.gtab = r->d_gtab; ga.aim = r->d_aim;
  ga.do_gamma = gamma; ga.do_div = div; ga.store_fwd = 0;
  ga.div_part = r->d_divpart;
  return ga;
}

dgx_status set_reference_stiffness(dgx_rve* r) {
  CK(h2d(r, r->d_Cref, r->C_ref, 81 * sizeof(double)));
  gamma_table(r->sl.g, r->num.precision == 1, gamma_args(r, true, false), r->d_gtab, r->st);
  r->n_launch++;
  CK(cudaGetLastError());
  return DGX_OK;
}

int converged(dgx_rve* r) {
  double mx = -1.7976931348623157e308;
  for (int k = 0; k < 9; ++k) mx = std::max(mx, r->P_av[k]);
  double divTol = std::max(mx * r->num.eps_rel_div, r->num.eps_abs_div);
  double BCTol = std::max(mx * r->num.eps_rel_P, r->num.eps_abs_P);
  double e = std::max(r->err_div / divTol, r->err_BC / BCTol);
  if ((r->total_iter >= r->num.itmin && e < 1.0) || r->terminally_ill) return 1;
  if (r->total_iter >= r->num.itmax) return -1;
  return 0;
}

// MechSolverBasic::calculate_solution (mech_solver_basic.cpp:110-160) before SNESSolve
dgx_status solve_prologue(dgx_rve* r) {
  masked_compliance(r->C_volAvg, r->rot_q, r->stress_mask, r->S);
  if (r->num.update_gamma) {
    for (int k = 0; k < 81; ++k) r->C_ref[k] = r->C_minMaxAvg[k] / r->wgt;
    TRY(set_reference_stiffness(r));
  }
  // the BC state the device updates during the solve (same values as the host copy)
  BcBlock bc;
  memcpy(bc.S, r->S, sizeof(bc.S));
  memcpy(bc.F_aim, r->F_aim, sizeof(bc.F_aim));
  memcpy(bc.P_aim, r->P_aim, sizeof(bc.P_aim));
  qu2om(r->rot_q, bc.R);
  memcpy(bc.mask, r->stress_mask, sizeof(bc.mask));
  bc.rotated = !(r->rot_q[0] == 1.0 && r->rot_q[1] == 0.0 && r->rot_q[2] == 0.0 && r->rot_q[3] == 0.0);
  CK(h2d(r, r->d_bc, &bc, sizeof(bc)));
  CK(cudaStreamSynchronize(r->st));       // bc is a stack copy
  return DGX_OK;
}

// ... and after it: terminally-ill flag, stress aim of the mixed BC, solution status
void solve_epilogue(dgx_rve* r, int reason, int32_t* conv, int32_t* iterations, int32_t* ill_out) {
  int ill = r->terminally_ill;
  r->terminally_ill = 0;
  for (int k = 0; k < 9; ++k) if (r->stress_mask[k]) r->P_aim[k] = r->P_av[k];
  if (conv) *conv = (reason > 0) && !ill;
  if (iterations) *iterations = r->total_iter;
  if (ill_out) *ill_out = ill;
}

// volume average of a 9-plane field (fixed-order reduction)
dgx_status field_average(dgx_rve* r, const double* X, double out[9]) {
  k_plane_sums<<<r->nb_red, RB, 0, r->st>>>(X, r->N, r->d_redpart);
  k_multi_finish<<<9, 32, 0, r->st>>>(r->d_redpart, r->nb_red, 9, r->d_redout);
  r->n_launch += 2;
  double sums[9];
  CK(d2h(r, sums, r->d_redout, 9 * sizeof(double)));
  CK(cudaStreamSynchronize(r->st));
  for (int k = 0; k < 9; ++k) out[k] = sums[k] * r->wgt;
  return DGX_OK;
}

void launch_axpy(double* z, const double* x, double a, const double* y, int64_t n, cudaStream_t st) {
  k_axpy<<<nblk(n), 256, 0, st>>>(z, x, a, y, n);
}
void launch_combine(double* XA, const double* XM, const VecList& Xd, int l, double c0, const double* beta, int64_t n,
                    int nb, cudaStream_t st) {
  k_combine<<<nb, 256, 0, st>>>(XA, XM, Xd, l, c0, beta, n);
}

double forward_time(const dgx_loadstep* ls, int inc, int sub_step_factor, int cut_back_level) {
  double dt;
  if (std::fabs(ls->r - 1.0) < 1.e-9) dt = ls->t / ls->N;
  else dt = ls->t * (std::pow(ls->r, inc) - std::pow(ls->r, inc + 1)) / (1.0 - std::pow(ls->r, ls->N));
  return dt * std::pow((double)sub_step_factor, -(double)cut_back_level);
}

dgx_status commit(dgx_rve* r) {
  size_t b9 = sizeof(double) * 9 * r->N, b24 = sizeof(double) * 24 * r->N;
  CK(cudaMemcpyAsync(r->ps.Fp0, r->ps.Fp, b9, cudaMemcpyDeviceToDevice, r->st));
  CK(cudaMemcpyAsync(r->ps.F0, r->ps.F, b9, cudaMemcpyDeviceToDevice, r->st));
  CK(cudaMemcpyAsync(r->ps.Lp0, r->ps.Lp, b9, cudaMemcpyDeviceToDevice, r->st));
  CK(cudaMemcpyAsync(r->ps.S0, r->ps.S, b9, cudaMemcpyDeviceToDevice, r->st));
  CK(cudaMemcpyAsync(r->ps.st0, r->ps.st, b24, cudaMemcpyDeviceToDevice, r->st));
  if (r->fx_F0) {                     // exported committed F (dgx_fields), reference layout
    k_planar2aos<<<nblk(9 * r->N), 256, 0, r->st>>>(r->ps.F0, r->N, 9, r->N, r->fx_F0);
    r->n_launch++;
  }
  return DGX_OK;
}

dgx_status upload_aos(dgx_rve* r, const double* host, int w, double* planar) {
  double* tmp = r->XM;                        // scratch: 9N doubles (w <= 9)
  CK(h2d(r, tmp, host, sizeof(double) * w * r->N));
  k_aos2planar<<<nblk(w * r->N), 256, 0, r->st>>>(tmp, w, r->N, planar, r->N);
  r->n_launch++;
  return DGX_OK;
}
// planar device field -> AoS host array: transposed on the device (staging buffer of
// 12 N doubles, allocated on first use), then one copy into the caller's memory
dgx_status download_aos(dgx_rve* r, const double* planar, int w, double* host) {
  if (w <= 12) {
    if (!r->d_aos) TRY(dalloc(r, &r->d_aos, 12 * r->N));
    k_planar2aos<<<nblk(w * r->N), 256, 0, r->st>>>(planar, r->N, w, r->N, r->d_aos);
    r->n_launch++;
    CK(d2h(r, host, r->d_aos, sizeof(double) * w * r->N));
    CK(cudaStreamSynchronize(r->st));
    CK(cudaGetLastError());
    return DGX_OK;
  }
  std::vector<double> tmp((size_t)w * r->N);
  CK(d2h(r, tmp.data(), planar, sizeof(double) * w * r->N));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  for (int64_t e = 0; e < r->N; ++e)
    for (int c = 0; c < w; ++c) host[(size_t)w * e + c] = tmp[(size_t)c * r->N + e];
  return DGX_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" void dgx_material_default(dgx_material* m) {
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

extern "C" void dgx_numerics_default(dgx_numerics* n) {
  memset(n, 0, sizeof(*n));
  n->itmin = 1; n->itmax = 100; n->update_gamma = 0;
  n->eps_abs_div = 1e-4; n->eps_rel_div = 5e-4; n->eps_abs_P = 1e3; n->eps_rel_P = 1e-3;
  n->divergence_correction = 2; n->derivative = 0;
  n->stag_iter_max = 10; n->max_cut_back = 3;
  n->solver = 0; n->ngmres_m = 30; n->snes_max_it = 50;
  n->precision = 0; n->lazy_tangent = 1;
}

extern "C" void dgx_rve_destroy(dgx_rve* r) {
  if (!r) return;
  if (r->ex) executor_destroy(r->ex);
  for (auto p : r->allocs) cudaFree(p);
  for (int i = 0; i < 3; ++i) axis_destroy(&r->ax[i]);
  for (int i = 0; i < 6; ++i) if (r->ev[i]) cudaEventDestroy(r->ev[i]);
  if (r->owns_stream && r->st) cudaStreamDestroy(r->st);
  delete r;
}

// Every device buffer of an RVE.  With r->dry set nothing is allocated and r->bytes
// only adds up the sizes: the footprint used for admission control.
static dgx_status allocate_buffers(dgx_rve* r, const int32_t cells[3], const dgx_numerics* num, int n_materials) {
  const int64_t N = r->N;
  dgx_status s = DGX_OK;
#define AL(p, c) do { s = dalloc(r, p, c); if (s != DGX_OK) return s; } while (0)
  r->ps.n = N; r->ps.ld = N;
  AL(&r->ps.F, 9 * N); AL(&r->ps.F0, 9 * N); AL(&r->ps.Fp0, 9 * N); AL(&r->ps.Lp0, 9 * N); AL(&r->ps.S0, 9 * N);
  AL(&r->ps.st0, 24 * N); AL(&r->ps.Fp, 9 * N); AL(&r->ps.Lp, 9 * N); AL(&r->ps.S, 9 * N); AL(&r->ps.Fe, 9 * N);
  AL(&r->ps.st, 24 * N); AL(&r->ps.P, 9 * N); AL(&r->ps.status, N);
  AL(&r->X, 9 * N); AL(&r->R, 9 * N); AL(&r->XM, 9 * N); AL(&r->FM, 9 * N); AL(&r->XA, 9 * N); AL(&r->FA, 9 * N);
  AL(&r->F_last_inc, 9 * N); AL(&r->F_dot, 9 * N);
  int m = num->solver == 0 ? num->ngmres_m : 0;
  r->Xdot.resize(m); r->Fdot.resize(m);
  for (int i = 0; i < m; ++i) { AL(&r->Xdot[i], 9 * N); AL(&r->Fdot[i], 9 * N); }
  bool fp32 = num->precision == 1;
  r->sl = spec_launch(cells[0], cells[1], cells[2], fp32 ? sizeof(float2) : sizeof(double2));
  {
    double* sp = nullptr;
    AL(&sp, (fp32 ? 1 : 2) * 9 * r->sl.g.Nh);
    r->spec = sp;
  }
  r->nb_cons = (int)((N + 31) / 32);            // P_av partials: one per 32 cells
  {
    const char* env = std::getenv("DGX_CONS_BLOCK");
    int b = env ? std::atoi(env) : 128;
    r->cons_block = (b == 32 || b == 64 || b == 256) ? b : 128;
    r->cons_block_forced = env != nullptr;
  }
  r->nb_tan = (int)((N + 63) / 64);
  r->nb_red = (int)std::min<int64_t>(608, std::max<int64_t>(1, (9 * N + 1023) / 1024));
  AL(&r->d_Ppart, 9 * (int64_t)r->nb_cons);
  AL(&r->d_tpart, r->nb_tan);
  AL(&r->d_divpart, r->sl.ndiv);
  AL(&r->d_redpart, 128 * (int64_t)r->nb_red);   // two concurrent fused reductions of up to 64 sums
  AL(&r->d_redout, 128); AL(&r->d_beta, 32);
  AL(&r->d_bc, 1);
  AL(&r->d_Pav, 9); AL(&r->d_Cvol, 81); AL(&r->d_Cmm, 81); AL(&r->d_Cref, 81); AL(&r->d_aim, 9); AL(&r->d_rms, 1);
  AL(&r->d_ill, 1); AL(&r->d_cnt, 1);
  AL(&r->d_xi_x, cells[0] / 2 + 1); AL(&r->d_xi_y, cells[1]); AL(&r->d_xi_z, cells[2]);
  if (num->derivative == 2) {
    AL(&r->d_fw[0], 4 * (cells[0] / 2 + 1)); AL(&r->d_fw[1], 4 * cells[1]); AL(&r->d_fw[2], 4 * cells[2]);
  }
  AL(&r->d_gtab, (gamma_table_bytes(r->sl.g, fp32, num->derivative == 2) + 7) / 8);
  AL(&r->d_mat, N); AL(&r->d_Rm, 9 * (int64_t)n_materials);
#undef AL
  return DGX_OK;
}

extern "C" dgx_status dgx_rve_create(const int32_t cells[3], const double size[3], const int32_t* material_at,
                                     int32_t n_materials, const double* orientations, const dgx_material* mat,
                                     const dgx_numerics* num, dgx_rve** out) {
  if (!cells || !size || !material_at || !orientations || !mat || !num || !out || n_materials <= 0) {
    set_err("dgx_rve_create: null argument"); return DGX_ERR_ARG;
  }
  for (int i = 0; i < 3; ++i) if (cells[i] < 1 || !(size[i] > 0.0)) { set_err("dgx_rve_create: bad cells/size"); return DGX_ERR_ARG; }
  if (num->derivative < 0 || num->derivative > 2) { set_err("derivative must be 0, 1 or 2"); return DGX_ERR_ARG; }
  if (num->divergence_correction < 0 || num->divergence_correction > 2) { set_err("divergence_correction must be 0, 1 or 2"); return DGX_ERR_ARG; }
  if (num->ngmres_m < 1 || num->ngmres_m > 30) { set_err("ngmres_m must be in [1, 30]"); return DGX_ERR_ARG; }
  for (int i = 0; i < 3; ++i) if (cells[i] > 4096) { set_err("cells > 4096"); return DGX_ERR_ARG; }
  dgx_rve* r = new dgx_rve();
  *out = nullptr;
  for (int i = 0; i < 3; ++i) { r->cells[i] = cells[i]; r->geom[i] = size[i]; }
  r->N = (int64_t)cells[0] * cells[1] * cells[2];
  r->wgt = std::pow((double)r->N, -1.0);
  r->mat = *mat; r->num = *num;
  r->mp = make_params(*mat);
  // the mixed form also evaluates the Lp Jacobian and the hardening rate in FP32;
  // DGX_MIXED_CONS=0 keeps the FP64 constitutive kernel under FP32 spectra (A/B runs)
  {
    const char* mc = getenv("DGX_MIXED_CONS");
    r->mp.mixed = (num->precision == 1 && !(mc && mc[0] == '0')) ? 1 : 0;
  }
  // the kernels fold the cF Schmid sparsity at compile time: the host table must agree
  for (int a = 0; a < 12; ++a)
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) {
        int sg = CF_SLIP[a][k] * CF_SLIP[a][3 + l];
        if (r->mp.P[a][k + 3 * l] != sg * r->mp.pval) { set_err("Schmid table mismatch"); delete r; return DGX_ERR_STATE; }
      }
  // divergence correction (MechBase::base_init, mech_base.cpp:11-43)
  scaled_geometry(cells, size, num->divergence_correction, r->scaled);
  cudaError_t ce = cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking);
  if (ce != cudaSuccess) { set_err("cudaStreamCreate: %s", cudaGetErrorString(ce)); delete r; return DGX_ERR_CUDA; }
  r->owns_stream = true;
  for (int i = 0; i < 6; ++i) cudaEventCreate(&r->ev[i]);
  dgx_status s = allocate_buffers(r, cells, num, n_materials);
  if (s != DGX_OK) { dgx_rve_destroy(r); return s; }
  const int64_t N = r->N;
  bool fp32 = num->precision == 1;
  for (int i = 0; i < 3; ++i)
    if (!axis_create(&r->ax[i], cells[i])) { set_err("FFT plan for length %d failed", cells[i]); dgx_rve_destroy(r); return DGX_ERR_UNSUPPORTED; }
  if (!spec_prepare(r->sl, fp32)) {
    set_err("grid %dx%dx%d: FFT line tiles exceed the device's shared memory", cells[0], cells[1], cells[2]);
    dgx_rve_destroy(r); return DGX_ERR_UNSUPPORTED;
  }
  // xi1st per axis (imaginary parts; continuous or central difference)
  {
    double* dst[3] = {r->d_xi_x, r->d_xi_y, r->d_xi_z};
    for (int p = 0; p < 3; ++p) {
      std::vector<double> v;
      xi_axis(p, cells, size, num->derivative == 2 ? 0 : num->derivative, v);
      if (cudaMemcpy(dst[p], v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_err("xi upload failed"); dgx_rve_destroy(r); return DGX_ERR_CUDA;
      }
      if (num->derivative == 2) {
        fw_axis(p, cells, v);
        if (cudaMemcpy(r->d_fw[p], v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
          set_err("xi upload failed"); dgx_rve_destroy(r); return DGX_ERR_CUDA;
        }
      }
    }
  }
  // orientations -> initial Fp per material
  r->n_materials = n_materials;
  r->h_mat.assign(material_at, material_at + N);
  r->h_orient.assign(orientations, orientations + 4 * (size_t)n_materials);
  {
    std::vector<double> Rm(9 * (size_t)n_materials);
    for (int m2 = 0; m2 < n_materials; ++m2) qu2om(orientations + 4 * m2, Rm.data() + 9 * m2);
    if (cudaMemcpy(r->d_Rm, Rm.data(), sizeof(double) * Rm.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(r->d_mat, material_at, sizeof(int32_t) * N, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_err("material upload failed"); dgx_rve_destroy(r); return DGX_ERR_CUDA;
    }
    k_init_points<<<nblk(N), 256, 0, r->st>>>(r->ps, r->d_mat, r->d_Rm, n_materials, mat->xi_0);
    cudaMemsetAsync(r->d_cnt, 0, sizeof(ConsCounters), r->st);
    if (cudaStreamSynchronize(r->st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      set_err("point init failed"); dgx_rve_destroy(r); return DGX_ERR_CUDA;
    }
  }
  for (int k = 0; k < 9; ++k) {
    r->F_aim[k] = r->F_aim_last_inc[k] = (k % 4) == 0 ? 1.0 : 0.0;
    r->F_aim_dot[k] = 0.0; r->P_aim[k] = 0.0; r->P_av[k] = 0.0; r->stress_mask[k] = 1;
  }
  memset(r->S, 0, sizeof(r->S));
  r->rot_q[0] = 1; r->rot_q[1] = r->rot_q[2] = r->rot_q[3] = 0;
  *out = r;
  return DGX_OK;
}

extern "C" dgx_status dgx_rve_footprint(const int32_t cells[3], const dgx_numerics* num, int32_t n_materials,
                                        int64_t* bytes) {
  if (!cells || !num || !bytes || n_materials < 1) return DGX_ERR_ARG;
  for (int i = 0; i < 3; ++i) if (cells[i] < 1 || cells[i] > 4096) return DGX_ERR_ARG;
  dgx_rve r;
  r.dry = true;
  r.N = (int64_t)cells[0] * cells[1] * cells[2];
  TRY(allocate_buffers(&r, cells, num, n_materials));
  *bytes = r.bytes;
  return DGX_OK;
}

extern "C" int64_t dgx_rve_points(const dgx_rve* r) { return r ? r->N : 0; }
extern "C" int64_t dgx_rve_device_bytes(const dgx_rve* r) { return r ? r->bytes : 0; }

extern "C" dgx_status dgx_constitutive_response(dgx_rve* r, const double* F, double dt, int32_t first, int32_t count,
                                                double* P, double* dPdF, int32_t* terminally_ill) {
  if (!r || !F) { set_err("null argument"); return DGX_ERR_ARG; }
  if (first != 0 || count != r->N) { set_err("dgx_constitutive_response: whole RVE only (first=0, count=N)"); return DGX_ERR_UNSUPPORTED; }
  TRY(upload_aos(r, F, 9, r->XA));
  r->terminally_ill = 0;
  TRY(constitutive_response(r, r->XA, dt, true));
  if (P) TRY(download_aos(r, r->ps.P, 9, P));
  if (dPdF) {
    if (!r->d_dPdF) {
      double* d = nullptr;
      TRY(dalloc(r, &d, 81 * r->N));
      r->d_dPdF = d;
    }
    launch_tangent(r->mp, r->ps, dt, r->d_dPdF, r->N, r->d_tpart, r->st);
    launch_tangent_finish(r->d_tpart, r->nb_tan, r->wgt, r->d_Cvol, r->d_Cmm, r->st);
    r->n_launch += 2;
    TRY(download_aos(r, r->d_dPdF, 81, dPdF));
  }
  if (terminally_ill) *terminally_ill = r->terminally_ill;
  return DGX_OK;
}

extern "C" dgx_status dgx_fields(dgx_rve* r, int32_t with_dPdF, dgx_field_ptrs* out) {
  if (!r || !out) { set_err("dgx_fields: null argument"); return DGX_ERR_ARG; }
  if (r->in_batch) { set_err("dgx_fields: the RVE is a batch member"); return DGX_ERR_STATE; }
  const int64_t N = r->N;
  if (!r->fx_F) {
    double* ill = nullptr;
    TRY(dalloc(r, &r->fx_F0, 9 * N));
    TRY(dalloc(r, &r->fx_F, 9 * N));
    TRY(dalloc(r, &r->fx_P, 9 * N));
    TRY(dalloc(r, &ill, 1));
    r->fx_ill = reinterpret_cast<int32_t*>(ill);
    // F0 and F start as the committed deformation gradient, P as the last stress
    k_planar2aos<<<nblk(9 * N), 256, 0, r->st>>>(r->ps.F0, N, 9, N, r->fx_F0);
    k_planar2aos<<<nblk(9 * N), 256, 0, r->st>>>(r->ps.F0, N, 9, N, r->fx_F);
    k_planar2aos<<<nblk(9 * N), 256, 0, r->st>>>(r->ps.P, N, 9, N, r->fx_P);
    r->n_launch += 3;
    CK(cudaMemsetAsync(r->fx_ill, 0, sizeof(int32_t), r->st));
  }
  if (with_dPdF && !r->fx_dPdF) {
    TRY(dalloc(r, &r->fx_dPdF, 81 * N));
    CK(cudaMemsetAsync(r->fx_dPdF, 0, sizeof(double) * 81 * N, r->st));
  }
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  out->n = N;
  out->F0 = r->fx_F0;
  out->F = r->fx_F;
  out->P = r->fx_P;
  out->dPdF = r->fx_dPdF;
  out->terminally_ill = r->fx_ill;
  out->stream = (void*)r->st;
  return DGX_OK;
}

extern "C" dgx_status dgx_constitutive_response_fields(dgx_rve* r, double dt, int32_t first, int32_t count,
                                                       int32_t want_dPdF) {
  if (!r) { set_err("null argument"); return DGX_ERR_ARG; }
  if (!r->fx_F) { set_err("dgx_constitutive_response_fields: call dgx_fields first"); return DGX_ERR_STATE; }
  if (r->in_batch) { set_err("dgx_constitutive_response_fields: the RVE is a batch member"); return DGX_ERR_STATE; }
  if (first != 0 || count != r->N) { set_err("dgx_constitutive_response_fields: whole RVE only (first=0, count=N)"); return DGX_ERR_UNSUPPORTED; }
  if (want_dPdF && !r->fx_dPdF) { set_err("dgx_constitutive_response_fields: dgx_fields was called without dPdF"); return DGX_ERR_STATE; }
  const int64_t N = r->N;
  // the caller's F (reference layout, library-owned) -> planes, on the RVE's stream
  k_aos2planar<<<nblk(9 * N), 256, 0, r->st>>>(r->fx_F, 9, N, r->XA, N);
  r->n_launch++;
  r->terminally_ill = 0;
  TRY(constitutive_response(r, r->XA, dt, true));
  k_planar2aos<<<nblk(9 * N), 256, 0, r->st>>>(r->ps.P, N, 9, N, r->fx_P);
  r->n_launch++;
  if (want_dPdF) {
    if (!r->d_dPdF) {
      double* d = nullptr;
      TRY(dalloc(r, &d, 81 * N));
      r->d_dPdF = d;
    }
    launch_tangent(r->mp, r->ps, dt, r->d_dPdF, N, r->d_tpart, r->st);
    launch_tangent_finish(r->d_tpart, r->nb_tan, r->wgt, r->d_Cvol, r->d_Cmm, r->st);
    k_planar2aos<<<nblk(81 * N), 256, 0, r->st>>>(r->d_dPdF, N, 81, N, r->fx_dPdF);
    r->n_launch += 3;
  }
  const int32_t ill = r->terminally_ill ? 1 : 0;
  CK(cudaMemcpyAsync(r->fx_ill, &ill, sizeof(int32_t), cudaMemcpyHostToDevice, r->st));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  return DGX_OK;
}

extern "C" dgx_status dgx_averages(dgx_rve* r, double P_av[9], double C_volAvg[81], double C_minMaxAvg[81]) {
  if (!r) return DGX_ERR_ARG;
  if (C_volAvg || C_minMaxAvg) TRY(ensure_tangent(r));
  if (P_av) memcpy(P_av, r->P_av, 9 * sizeof(double));
  if (C_volAvg) memcpy(C_volAvg, r->C_volAvg, 81 * sizeof(double));
  if (C_minMaxAvg) memcpy(C_minMaxAvg, r->C_minMaxAvg, 81 * sizeof(double));
  return DGX_OK;
}

extern "C" dgx_status dgx_commit_increment(dgx_rve* r) {
  if (!r) return DGX_ERR_ARG;
  TRY(commit(r));
  CK(cudaStreamSynchronize(r->st));
  return DGX_OK;
}

extern "C" dgx_status dgx_update_gamma(dgx_rve* r, const double C[81]) {
  if (!r || !C) return DGX_ERR_ARG;
  for (int k = 0; k < 81; ++k) r->C_ref[k] = C[k] / r->wgt;
  TRY(set_reference_stiffness(r));
  return DGX_OK;
}

extern "C" dgx_status dgx_divergence_rms(dgx_rve* r, const double* P, double* rms) {
  if (!r || !P || !rms) return DGX_ERR_ARG;
  TRY(upload_aos(r, P, 9, r->XA));
  GammaArgs ga = gamma_args(r, false, true);
  spec_convolve(r->sl, r->num.precision == 1, r->ax[0].plan, r->ax[1].plan, r->ax[2].plan, r->XA, r->XA, r->N, r->spec,
                ga, r->st);
  spec_div_finish(r->d_divpart, r->sl.ndiv, r->wgt, r->cells[0], r->d_rms, r->st);
  r->n_launch += 4;
  CK(d2h(r, rms, r->d_rms, sizeof(double)));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  return DGX_OK;
}

extern "C" dgx_status dgx_gamma_convolution(dgx_rve* r, double* field, const double aim[9]) {
  if (!r || !field || !aim) return DGX_ERR_ARG;
  TRY(upload_aos(r, field, 9, r->XA));
  CK(h2d(r, r->d_aim, aim, 9 * sizeof(double)));
  GammaArgs ga = gamma_args(r, true, false);
  spec_convolve(r->sl, r->num.precision == 1, r->ax[0].plan, r->ax[1].plan, r->ax[2].plan, r->XA, r->XA, r->N, r->spec,
                ga, r->st);
  r->n_launch += 5;
  TRY(download_aos(r, r->XA, 9, field));
  CK(cudaGetLastError());
  return DGX_OK;
}

extern "C" dgx_status dgx_fft_forward(dgx_rve* r, const double* field, double* spectrum) {
  if (!r || !field || !spectrum) return DGX_ERR_ARG;
  if (r->num.precision == 1) { set_err("dgx_fft_forward: FP64 RVEs only"); return DGX_ERR_UNSUPPORTED; }
  TRY(upload_aos(r, field, 9, r->XA));
  GammaArgs ga = gamma_args(r, false, false);
  ga.store_fwd = 1;
  spec_convolve(r->sl, false, r->ax[0].plan, r->ax[1].plan, r->ax[2].plan, r->XA, r->XA, r->N, r->spec, ga, r->st);
  r->n_launch += 3;
  const SpecGeom& g = r->sl.g;
  std::vector<double2> h(9 * g.Nh);
  CK(d2h(r, h.data(), r->spec, sizeof(double2) * 9 * g.Nh));
  CK(cudaStreamSynchronize(r->st));
  // device: spec[c*Nh + i + N0r*(y + N1*z)] -> reference (l,m,i,k=z,j=y) interleaved
  for (int c = 0; c < 9; ++c)
    for (int z = 0; z < g.N2; ++z)
      for (int y = 0; y < g.N1; ++y)
        for (int i = 0; i < g.N0r; ++i) {
          double2 v = h[c * g.Nh + i + (long long)g.N0r * (y + (long long)g.N1 * z)];
          long long o = c + 9LL * (i + (long long)g.N0r * (z + (long long)g.N2 * y));
          spectrum[2 * o] = v.x; spectrum[2 * o + 1] = v.y;
        }
  return DGX_OK;
}

extern "C" dgx_status dgx_solver_init(dgx_rve* r) {
  if (!r) return DGX_ERR_ARG;
  // fresh material-point state (init of the reference runs on a fresh state)
  k_init_points<<<nblk(r->N), 256, 0, r->st>>>(r->ps, r->d_mat, r->d_Rm, r->n_materials, r->mat.xi_0);
  k_fill_identity<<<nblk(9 * r->N), 256, 0, r->st>>>(r->X, r->N);
  k_fill_identity<<<nblk(9 * r->N), 256, 0, r->st>>>(r->F_last_inc, r->N);
  r->n_launch += 3;
  for (int k = 0; k < 9; ++k) {
    r->F_aim[k] = r->F_aim_last_inc[k] = (k % 4) == 0 ? 1.0 : 0.0;
    r->F_aim_dot[k] = 0.0; r->P_aim[k] = 0.0;
  }
  r->terminally_ill = 0;
  TRY(constitutive_response(r, r->X, 0.0, true));
  // the argmax/argmin of |dPdF| at F = I is a tie broken by FP64 rounding: take it
  // with the reference's operation order (see ref_stiffness.cpp)
  if (dgx_reference_stiffness(r->mat.C11, r->mat.C12, r->mat.C44, r->n_materials, r->h_orient.data(),
                              r->h_mat.data(), r->N, r->C_minMaxAvg) != 0) {
    set_err("reference stiffness selection failed"); return DGX_ERR_STATE;
  }
  for (int k = 0; k < 81; ++k) r->C_ref[k] = r->C_minMaxAvg[k] / r->wgt;
  TRY(set_reference_stiffness(r));
  memcpy(r->C_minMaxAvgLastInc, r->C_minMaxAvg, sizeof(r->C_minMaxAvg));
  memcpy(r->C_volAvgLastInc, r->C_volAvg, sizeof(r->C_volAvg));
  r->initialized = true;
  r->cut_back = 0; r->cut_back_level = 0; r->t = 0.0; r->dt = 1.0; r->dt_prev = 0.0; r->cur_step = -1;
  return DGX_OK;
}

extern "C" dgx_status dgx_solver_forward(dgx_rve* r, int32_t cutback, int32_t guess, double dt, double dt_old,
                                         double t_remaining, const dgx_loadstep* ls) {
  if (!r || !ls) return DGX_ERR_ARG;
  if (!r->initialized) { set_err("dgx_solver_forward before dgx_solver_init"); return DGX_ERR_STATE; }
  const int64_t N = r->N;
  r->evals_in_step = 0;
  if (cutback) {
    memcpy(r->C_volAvg, r->C_volAvgLastInc, sizeof(r->C_volAvg));
    memcpy(r->C_minMaxAvg, r->C_minMaxAvgLastInc, sizeof(r->C_minMaxAvg));
  } else {
    TRY(ensure_tangent(r));
    memcpy(r->C_volAvgLastInc, r->C_volAvg, sizeof(r->C_volAvg));
    memcpy(r->C_minMaxAvgLastInc, r->C_minMaxAvg, sizeof(r->C_minMaxAvg));
    for (int k = 0; k < 9; ++k) {
      double aim_diff = (r->F_aim[k] - r->F_aim_last_inc[k]) / dt_old;
      r->F_aim_dot[k] = guess ? (ls->stress_mask[k] ? 0.0 : aim_diff) : 0.0;
    }
    memcpy(r->F_aim_last_inc, r->F_aim, sizeof(r->F_aim));
    double step[9];
    if (ls->def_type == 2) {
      mm3(ls->def_values, r->F_aim_last_inc, step);
    } else if (ls->def_type == 1) {
      memcpy(step, ls->def_values, sizeof(step));
    } else {
      for (int k = 0; k < 9; ++k) step[k] = (ls->def_values[k] - r->F_aim_last_inc[k]) / t_remaining;
    }
    for (int k = 0; k < 9; ++k) r->F_aim_dot[k] += ls->def_mask[k] ? 0.0 : step[k];
    double rot[9];
    rotate2(ls->rot_q, r->F_aim_dot, rot, true);
    k_rate<<<nblk(9 * N), 256, 0, r->st>>>(r->F_dot, r->F_last_inc, r->X, dt_old, guess, rot[0], rot[1], rot[2],
                                          rot[3], rot[4], rot[5], rot[6], rot[7], rot[8], N);
    CK(cudaMemcpyAsync(r->F_last_inc, r->X, sizeof(double) * 9 * N, cudaMemcpyDeviceToDevice, r->st));
    r->n_launch++;
  }
  for (int k = 0; k < 9; ++k) r->F_aim[k] = r->F_aim_last_inc[k] + r->F_aim_dot[k] * dt;
  for (int k = 0; k < 9; ++k) {
    if (ls->stress_type == 0) r->P_aim[k] += ls->stress_mask[k] ? (ls->stress_values[k] - r->P_aim[k]) / t_remaining * dt : 0.0;
    else r->P_aim[k] += ls->stress_mask[k] ? ls->stress_values[k] * dt : 0.0;
  }
  double rot[9];
  rotate2(ls->rot_q, r->F_aim, rot, false);
  // forward_field: F = F_last_inc + F_dot dt, shifted so that its average is the aim
  k_forward_field<<<nblk(9 * N), 256, 0, r->st>>>(r->X, r->F_last_inc, r->F_dot, dt, 9 * N);
  k_plane_sums<<<r->nb_red, RB, 0, r->st>>>(r->X, N, r->d_redpart);
  k_multi_finish<<<9, 32, 0, r->st>>>(r->d_redpart, r->nb_red, 9, r->d_redout);
  double sums[9];
  CK(d2h(r, sums, r->d_redout, 9 * sizeof(double)));
  CK(cudaStreamSynchronize(r->st));
  double diff[9];
  for (int k = 0; k < 9; ++k) diff[k] = sums[k] * r->wgt - rot[k];
  CK(h2d(r, r->d_redout, diff, 9 * sizeof(double)));
  k_shift_planes<<<nblk(9 * N), 256, 0, r->st>>>(r->X, r->d_redout, N);
  r->n_launch += 4;
  memcpy(r->stress_mask, ls->stress_mask, sizeof(r->stress_mask));
  memcpy(r->rot_q, ls->rot_q, sizeof(r->rot_q));
  r->delta_t = dt;
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  return DGX_OK;
}

extern "C" dgx_status dgx_solver_solve(dgx_rve* r, int32_t* conv, int32_t* iterations, int32_t* ill_out) {
  if (!r) return DGX_ERR_ARG;
  if (!r->initialized) { set_err("dgx_solver_solve before dgx_solver_init"); return DGX_ERR_STATE; }
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  return run_single(r, 0, nullptr, 0, 0, nullptr, 0, nullptr, conv, iterations, ill_out);
}

extern "C" dgx_status dgx_run_increment(dgx_rve* r, const dgx_loadstep* step, int32_t step_index, int32_t inc,
                                        dgx_inc_record* record) {
  if (!r || !step) return DGX_ERR_ARG;
  if (!r->initialized) { set_err("dgx_run_increment before dgx_solver_init"); return DGX_ERR_STATE; }
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  return run_single(r, 1, step, step_index, inc, record, 1, nullptr, nullptr, nullptr, nullptr);
}

extern "C" dgx_status dgx_run_loadcase(dgx_rve* r, int32_t nsteps, const dgx_loadstep* steps, dgx_inc_record* records,
                                       int32_t max_records, int32_t* n_records) {
  if (!r || !steps || nsteps < 1) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  TRY(dgx_solver_init(r));
  return run_single(r, 2, steps, nsteps, 0, records, max_records, n_records, nullptr, nullptr, nullptr);
}

extern "C" dgx_status dgx_run_loadcase_output(dgx_rve* r, int32_t nsteps, const dgx_loadstep* steps,
                                              dgx_inc_record* records, int32_t max_records, int32_t* n_records,
                                              dgx_result* result, const char* restart_path, int32_t restart_every) {
  if (!r || !steps || nsteps < 1) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  if (restart_every > 0 && !restart_path) return DGX_ERR_ARG;
  TRY(dgx_solver_init(r));
  Output out{result, restart_path, restart_every};
  return run_single(r, 2, steps, nsteps, 0, records, max_records, n_records, nullptr, nullptr, nullptr, &out);
}

// MechSolverBasic::update_coords / MechBase::base_update_coords (mech_solver_basic.cpp:222-238,
// mech_base.cpp:45-154) on the current solution field X
dgx_status dgx::update_coords_impl(dgx_rve* r, double* u_n, double* u_p) {
  const int64_t Nn = (int64_t)(r->cells[0] + 1) * (r->cells[1] + 1) * (r->cells[2] + 1);
  if (!r->d_un) {
    TRY(dalloc(r, &r->d_un, 3 * Nn));
    TRY(dalloc(r, &r->d_up, 3 * r->N));
    TRY(dalloc(r, &r->d_Favg, 9));
  }
  spec_update_coords(r->sl, r->num.precision == 1, r->ax[0].plan, r->ax[1].plan, r->ax[2].plan, r->X, r->N, r->spec,
                     r->XA, r->geom, r->num.derivative, gamma_args(r, false, false), r->wgt, r->d_Favg, r->d_un,
                     r->d_up, r->st);
  r->n_launch += 8;
  if (u_n) CK(d2h(r, u_n, r->d_un, sizeof(double) * 3 * Nn));
  if (u_p) CK(d2h(r, u_p, r->d_up, sizeof(double) * 3 * r->N));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  return DGX_OK;
}

extern "C" dgx_status dgx_update_coords(dgx_rve* r, double* u_n, double* u_p) {
  if (!r) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  return update_coords_impl(r, u_n, u_p);
}

extern "C" dgx_status dgx_get(dgx_rve* r, const char* name, double* out) {
  if (!r || !name || !out) return DGX_ERR_ARG;
  std::string s(name);
  double* planar = nullptr; int w = 9;
  if (s == "F") planar = r->ps.F;
  else if (s == "P") planar = r->ps.P;
  else if (s == "R") planar = r->R;
  else if (s == "Fp") planar = r->ps.Fp;
  else if (s == "Lp") planar = r->ps.Lp;
  else if (s == "Fe") planar = r->ps.Fe;
  else if (s == "S") planar = r->ps.S;
  else if (s == "X") planar = r->X;
  else if (s == "xi") { planar = r->ps.st; w = 12; }
  else if (s == "gamma") { planar = r->ps.st + 12 * r->N; w = 12; }
  else if (s == "P_av") { memcpy(out, r->P_av, 72); return DGX_OK; }
  else if (s == "F_aim") { memcpy(out, r->F_aim, 72); return DGX_OK; }
  else if (s == "C_volAvg") { TRY(ensure_tangent(r)); memcpy(out, r->C_volAvg, 648); return DGX_OK; }
  else if (s == "C_minMaxAvg") { TRY(ensure_tangent(r)); memcpy(out, r->C_minMaxAvg, 648); return DGX_OK; }
  else if (s == "C_ref") { memcpy(out, r->C_ref, 648); return DGX_OK; }
  else if (s == "S_compliance") { memcpy(out, r->S, 648); return DGX_OK; }
  else { set_err("dgx_get: unknown field '%s'", name); return DGX_ERR_ARG; }
  return download_aos(r, planar, w, out);
}

extern "C" void* dgx_rve_stream(const dgx_rve* r) { return r ? (void*)r->st : nullptr; }

extern "C" dgx_status dgx_timers(const dgx_rve* r, double ms[3], int64_t launches[3]) {
  if (!r || !ms) return DGX_ERR_ARG;
  int64_t n[3] = {0, 0, 0}, l = 0, hb = 0, db = 0;
  for (int i = 0; i < 3; ++i) { ms[i] = r->t_ms[i]; n[i] = r->t_n[i]; }
  if (r->ex) executor_stats(r->ex, ms, n, &l, &hb, &db, nullptr);
  if (launches) for (int i = 0; i < 3; ++i) launches[i] = n[i];
  return DGX_OK;
}

extern "C" dgx_status dgx_counters(const dgx_rve* r, int64_t out[10]) {
  if (!r || !out) return DGX_ERR_ARG;
  ConsCounters c{};
  CK(cudaMemcpy(&c, r->d_cnt, sizeof(c), cudaMemcpyDeviceToHost));
  double ms[3] = {0, 0, 0};
  int64_t n[3] = {0, 0, 0}, l = 0, hb = 0, db = 0, gr = 0;
  if (r->ex) executor_stats(r->ex, ms, n, &l, &hb, &db, &gr);
  out[0] = r->n_eval; out[1] = (int64_t)c.state_iters; out[2] = (int64_t)c.lp_iters; out[3] = r->n_tangent;
  out[4] = r->n_launch + l; out[5] = (int64_t)c.jac_iters; out[6] = r->bytes_h2d + hb; out[7] = r->bytes_d2h + db;
  out[8] = (int64_t)c.fpi_iters; out[9] = gr;
  return DGX_OK;
}

extern "C" void dgx_flop_model(double out[4]) {
  if (!out) return;
  out[0] = FLOPS_LP; out[1] = FLOPS_JAC; out[2] = FLOPS_STATE; out[3] = FLOPS_FPI;
}
extern "C" void dgx_flop_model_mixed(double fp64[4], double fp32[4]) {
  if (fp64) {
    fp64[0] = FLOPS_LP; fp64[1] = FLOPS_MX_JAC64;
    fp64[2] = FLOPS_MX_STATE64; fp64[3] = FLOPS_MX_FPI64;
  }
  if (fp32) { fp32[0] = 0.0; fp32[1] = FLOPS_MX_JAC32; fp32[2] = FLOPS_MX_STATE32; fp32[3] = FLOPS_MX_FPI32; }
}
