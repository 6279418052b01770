// dgx_internal.cuh -- shared device/host definitions of the GB300 spectral solver.
//
// Layout in HBM (all FP64 unless stated):
//   * a "field" of n material points with w components is stored component-planar:
//     value(c, cell) = ptr[c * ld + cell], cell = x + N0 * (y + N1 * z), ld >= n.
//     3x3 components use the reference's column-major index c = i + 3 * j.
//   * per-point constitutive state is a set of such planes (structure of arrays).
// The C ABI converts to and from the reference's interleaved (3,3,N) layout.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dgx {

constexpr int NSLIP = 12;

// cF slip-slip interaction type (1..7, the index into h_sl-sl) of reacting system r and
// acting system b, the reference's interaction table (crystal.f90, FCC_INTERACTIONSLIPSLIP)
// as digits so that unrolled device loops fold it into constants.
__host__ __device__ constexpr int cf_interaction(int r, int b) {
  return "122475355467212745647535221553674764476122467355746212535647553221"
         "764674355467122476647535212746674764221553467355476122535647746212764674553221"[12 * r + b] - '0';
}

// Constitutive parameters of one phenopowerlaw cF phase, passed by value as a
// kernel parameter (constant bank, broadcast to all threads).
struct MatParams {
  double C66[36];            // column-major 6x6, Voigt 11,22,33,23,13,12
  double P[NSLIP][9];        // Schmid matrices d (x) n, column-major 3x3
  double h0h[7];             // h0 gdot0 times the seven cF slip-slip interaction values (h_sl-sl)
  double xi_inf, h0, n, gdot0, a, c1, c2;
  double C11mC12, C12;         // cubic stiffness: C11 - C12, C12
  double C44;
  double hC11mC12, hC12;       // (C11 - C12) / 2, C12 / 2
  double ngdot0, rxi_inf;      // n * gdot0, 1 / xi_inf
  double ngdot0_p;             // n * gdot0 / pval
  double pgdot0;               // pval * gdot0
  double pgdot0_sq;            // (pval * gdot0)^2
  double pval;                 // magnitude of the non-zero Schmid entries (1/sqrt2 * 1/sqrt3)
  double atol_xi, atol_gamma;
  double r_cutback_min, r_cutback, r_increase, eps_rel_state;
  double r_linesearch_Lp, eps_rel_Lp, eps_abs_Lp;
  double eps_rel_Lp2, eps_abs_Lp2;   // squared tolerances (norm tests without square roots)
  int N_iter_state_max, N_iter_Lp_max, f_update_jacobi_Lp;
  int n_int;                 // n if it is an integer in [1, 64], else -1
  int a_quarters;            // 4a if it is an integer in [1, 256], else -1
  // mixed-precision constitutive form (numerics precision 1): the Lp Newton's residual,
  // updates and convergence test and the state's accumulation stay FP64; the Newton
  // Jacobian, its first-order starts, the hardening and gamma rates, the damper and the
  // state update's residual and test are evaluated in FP32, and later evaluations of a
  // step start from the previous one.
  // 0 for the plain FP64 form.
  int mixed;
  float h0h_f[7];            // h0h in FP32 (hardening rate of the mixed form)
  float gdot0_f;             // gdot0 in FP32
  float n_f, rpval_f, pgdot0_f;   // n, 1 / pval, pval gdot0 in FP32
  float pval_f, hC11mC12_f, hC12_f, C44_f;   // pval and the halved cubic moduli in FP32
};

// Planes of the per-point constitutive state.  All pointers address component
// planes with stride `ld`.
struct PointState {
  int64_t n, ld;
  double* F;     // 9   current deformation gradient (phase F)
  double* F0;    // 9   committed F (sub-step interpolation after a cut-back)
  double* Fp0;   // 9   committed plastic deformation gradient
  double* Lp0;   // 9   committed Lp
  double* S0;    // 9   committed 2nd PK stress
  double* st0;   // 24  committed state: xi (12) then gamma (12)
  double* Fp;    // 9   out
  double* Lp;    // 9   in: warm start, out: result
  double* S;     // 9   out
  double* Fe;    // 9   out
  double* st;    // 24  out
  double* P;     // 9   out: first Piola-Kirchhoff stress
  int32_t* status;  // 0 converged, 1 terminally ill
};

// Per-block reduction record of the consistent tangent (C_volAvg, C_minMaxAvg).
struct TangentPartial {
  double sum[81];
  double nmax, nmin;
  long long imax, imin;
  double dmax[81], dmin[81];
};

// Counters of constitutive work (for the FP64 roofline), accumulated per launch.
struct ConsCounters {
  unsigned long long state_iters, lp_iters, jac_iters, points, fpi_iters;
};

// Algorithmic FP64 flops of the constitutive kernel per counted unit (FMA = 2, division,
// reciprocal and square root = 1), counted from its arithmetic: one Lp Newton iteration
// (B, Fe, Hooke, 12-system kinetics with derivatives, Lp, residual and norms: 378), one
// Jacobian step (W, the signed sums T^ scaled by the cubic moduli, B^ b and the 6 x 6
// matrix I + B^ T^, its LU with one right-hand side, the step b - T^ u: 923), one state
// integration call (Fp0^-1, F Fp0^-1, pval/xi, first dot state, predictor, and once
// the iteration ends Fp^-1, P, det and Fp scaling: 860) and one fixed-point iteration
// (pval/xi, hardening from the slip rates of the last Lp iteration summed per
// interaction type, damper, state update: 755).
constexpr double FLOPS_LP = 378.0, FLOPS_JAC = 923.0, FLOPS_STATE = 860.0, FLOPS_FPI = 755.0;
// The mixed form evaluates in FP32: the Jacobian step (all but the 5 FP64 multiplies
// of its scale factors: 918 flops); in every dot state the hardening rate and the gamma
// rate (FP64 31 flops per slip system -> FP32 24; x = 1 - xi / xi_inf stays FP64); the
// predictor's slip rates (13 per system); the damper's three dot products (144) and
// the blended rate (72); the fixed-point update's residual (D - d) dt, x_new to FP32
// and eps |x_new| (5 per state entry: 120), while the state itself accumulates in FP64
// once the iteration has converged (state0 + d dt: 48).  The iterate is formed from the
// rate history: xi = state0 + D dt and pval / xi at the head of a pass (48), xi again
// and x = 1 - xi / xi_inf after its Newton (48).  Per counted unit:
//   state: FP64 860 - 156 - 372 + 48 = 380, FP32 156 + 288 = 444
//   fpi:   FP64 48 + 48 = 96, FP32 288 + 144 + 72 + 120 = 624
// A first-order Newton start counts as one Jacobian unit (its own right-hand side, at
// most ~300 FP32 flops, is not counted), and a warm-started state integration still
// counts the explicit predictor it skips (156 FP32 flops and 12 FP64 reciprocals), so
// the mixed model counts cold evaluations exactly and warm ones approximately.
constexpr double FLOPS_MX_JAC64 = 5.0, FLOPS_MX_JAC32 = FLOPS_JAC - FLOPS_MX_JAC64;
constexpr double FLOPS_MX_STATE64 = 380.0, FLOPS_MX_STATE32 = 444.0;
constexpr double FLOPS_MX_FPI64 = 96.0, FLOPS_MX_FPI32 = 624.0;

// Stress boundary condition of one RVE's solve, resident on the device so that the
// BC step of a residual evaluation (form_residual) needs no host round trip.
struct BcBlock {
  double S[81];              // masked compliance (rotated frame)
  double F_aim[9];           // in / out: updated by every residual evaluation
  double P_aim[9];
  double R[9];               // rotation matrix of the BC frame, column-major
  int mask[9];               // 1: stress component not prescribed
  int rotated;               // the BC frame is not the identity
};

// One RVE of a batched constitutive launch (device table, ordered by tile0).
struct ConsItem {
  PointState ps;
  const double* F;           // deformation gradient planes (ld ldF)
  int64_t ldF;
  double dt;
  double wgt;                // 1 / N
  double* Ppart;             // ceil(n / 32) x 9 partial sums of P
  int* ill;                  // terminally-ill flag of this RVE
  long long tile0;           // first tile of this item in the launch
  int warm;                  // mixed form: the state planes hold the previous evaluation of
                             // the same step (its converged state seeds the state iteration)
};

// constitutive.cu launchers
void launch_constitutive(const MatParams& mp, const PointState& ps, const double* F, int64_t ldF, double dt,
                         double* Ppart, int* ill, ConsCounters* cnt, cudaStream_t st, int block);
// launch variants of the batched constitutive kernel: points per block (64, 128, 256,
// 128, 32, 128), and the blocks per SM its register allocation targets (1, 1, 1, 3, 1,
// 4: more blocks, fewer registers and more spills).  32 points per block spreads a small
// RVE over the most SMs (one warp each), which matters because one SM's FP64 unit is the
// scarce resource.  (Measured and dropped: 96 points at 5 blocks and 64 at 7, 136 and
// 144 registers: no faster than 128 at 4 in the mixed form, slower in FP64.)
constexpr int CONS_VARIANTS = 6;
__host__ __device__ constexpr int cons_variant_bs(int v) { return v == 0 ? 64 : v == 2 ? 256 : v == 4 ? 32 : 128; }
__host__ __device__ constexpr int cons_variant_minb(int v) { return v == 3 ? 3 : v == 5 ? 4 : 1; }
void launch_constitutive_batch(const MatParams& mp, const ConsItem* items, int nitems, long long ntiles,
                               unsigned long long* queue, ConsCounters* cnt, cudaStream_t st, int variant, int grid);
int constitutive_batch_resident(int variant, bool mixed);
void launch_pav_finish(const double* Ppart, int nblocks, double wgt, double* Pav, cudaStream_t st);
void launch_pav_finish_batch(const ConsItem* items, int nitems, double* Pav, cudaStream_t st);
void launch_tangent(const MatParams& mp, const PointState& ps, double dt, double* dPdF, int64_t ld_out,
                    TangentPartial* part, cudaStream_t st);
void launch_tangent_finish(const TangentPartial* part, int nblocks, double wgt, double* Cvol, double* Cmm,
                           cudaStream_t st);

}  // namespace dgx
