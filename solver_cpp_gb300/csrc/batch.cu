// batch.cu -- batched execution of the spectral solver: many RVEs of uneven size
// advanced together on one stream.
//
// The solve of one RVE (MechSolverBasic::calculate_solution with PETSc NGMRES,
// mech_solver_basic.cpp:110-339, inside DamaskGrid::loop_over_loadcase,
// damask_grid.cpp:82-196) is written here as a resumable state machine (Task).  A
// task runs its host logic until it needs the device -- a residual evaluation or a
// fused reduction -- and parks the request.  The executor then serves the requests
// of every task in one batched launch sequence:
//   residual   one persistent constitutive launch over the points of all RVEs
//              (offset-indexed tiles), one P_av reduction launch, one stress-BC
//              launch, then per group of equal grids one launch per FFT pass with
//              one blockIdx.y per RVE (FFT, divergence RMS, Gamma), one RMS launch
//   reduction  one fused multi-dot launch for all RVEs plus one finishing launch
//              (after the residuals of the same round when a task asks for both)
// with a single host synchronisation per round, and hands the results back.  Per-RVE arithmetic is identical to a batch of one
// (the same tiles, reduction partitions and summation orders), so an RVE's result
// does not depend on which other RVEs share the batch.  A single-RVE solve is a
// batch of one.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstddef>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "rve.cuh"

namespace dgx {

// ------------------------------------------------------------------ fused reductions
struct MultiItem {
  const double* a;          // anchor vector
  const double* b;          // second anchor (first K2 sums), may be null
  const double* v[32];
  int mode, K, K2, nb;      // mode 0: sum a*v_k ; mode 1: sum (v_k - a)^2 ; nb blocks
  long long n;
  double* part;             // nb x (K + K2)
  double* out;              // K + K2 results
};

// the reduction of k_multi (solver.cu) per item; blockIdx.y = item, same partition
__global__ void __launch_bounds__(RB) k_multi_batch(const MultiItem* __restrict__ items) {
  __shared__ MultiItem s;
  {
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(items + blockIdx.y);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s);
    for (int w = threadIdx.x; w < (int)(sizeof(MultiItem) / 8); w += blockDim.x) dst[w] = src[w];
  }
  __syncthreads();
  if ((int)blockIdx.x >= s.nb) return;
  const int K = s.K, K2 = s.K2;
  double acc[32], acc2[32];
  for (int k = 0; k < K; ++k) { acc[k] = 0.0; acc2[k] = 0.0; }
  const int64_t stride = (int64_t)s.nb * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < s.n; t += stride) {
    double av = s.a[t];
    double bv = s.b ? s.b[t] : 0.0;
    for (int k = 0; k < K; ++k) {
      double x = s.v[k][t];
      if (s.mode == 0) acc[k] = fma(av, x, acc[k]);
      else { double d = x - av; acc[k] = fma(d, d, acc[k]); }
      if (k < K2) acc2[k] = fma(bv, x, acc2[k]);
    }
  }
  __shared__ double red[RB];
  const int KT = K + K2;
  for (int k = 0; k < KT; ++k) {
    red[threadIdx.x] = k < K ? acc[k] : acc2[k - K];
    __syncthreads();
    for (int q = RB / 2; q > 0; q >>= 1) {
      if (threadIdx.x < q) red[threadIdx.x] += red[threadIdx.x + q];
      __syncthreads();
    }
    if (threadIdx.x == 0) s.part[blockIdx.x * KT + k] = red[0];
    __syncthreads();
  }
}

// one warp per (sum, item), fixed summation order (as k_multi_finish)
__global__ void k_multi_finish_batch(const MultiItem* __restrict__ items) {
  const MultiItem& it = items[blockIdx.y];
  const int KT = it.K + it.K2;
  const int k = blockIdx.x;
  if (k >= KT) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < it.nb; b += 32) s += it.part[b * KT + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) it.out[k] = s;
}

// ------------------------------------------------------------------ stress BC step on the device
// The BC part of form_residual (mech_solver_basic.cpp:321-334) for every RVE of a round,
// between the P_av reduction and the spectral pass, so that a residual evaluation needs
// no host round trip.  Rounded operation by operation in the host code's order (no
// contraction), so F_aim, err_BC and the zero-frequency value are bit-identical to the
// host computation.
struct BcItem {
  BcBlock* bc;
  double* Pav;        // in: volume average of P; out: in the BC frame when rotated
  double* aim;        // out: rotated dF_aim (zero frequency of Gamma * P)
  double* out;        // out: F_aim (9) and err_BC
};

__device__ void rotate2_exact(const double* R, const double* T, double* out, bool active) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = __dadd_rn(s, __dmul_rn(active ? R[k + 3 * i] : R[i + 3 * k], T[k + 3 * j]));
      t[i + 3 * j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = __dadd_rn(s, __dmul_rn(t[i + 3 * k], active ? R[k + 3 * j] : R[j + 3 * k]));
      out[i + 3 * j] = s;
    }
}

__global__ void k_bc_batch(const BcItem* __restrict__ items) {
  if (threadIdx.x != 0) return;
  const BcItem it = items[blockIdx.x];
  BcBlock* bc = it.bc;
  double P[9], dF[9], aim[9];
  for (int k = 0; k < 9; ++k) P[k] = it.Pav[k];
  if (bc->rotated) {                               // P_av into the BC frame (Spectral::constitutive_response)
    double t[9];
    rotate2_exact(bc->R, P, t, false);
    for (int k = 0; k < 9; ++k) { P[k] = t[k]; it.Pav[k] = t[k]; }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) s = __dadd_rn(s, __dmul_rn(bc->S[i + 3 * j + 9 * k + 27 * l], P[k + 3 * l]));
      dF[i + 3 * j] = s;
    }
  for (int k = 0; k < 9; ++k) { const double f = __dsub_rn(bc->F_aim[k], dF[k]); bc->F_aim[k] = f; it.out[k] = f; }
  double err = 0.0;
  for (int k = 0; k < 9; ++k) if (!bc->mask[k]) err = fmax(err, fabs(__dsub_rn(P[k], bc->P_aim[k])));
  it.out[9] = err;
  rotate2_exact(bc->R, dF, aim, true);
  for (int k = 0; k < 9; ++k) it.aim[k] = aim[k];
}

// ------------------------------------------------------------------ executor
struct ResReq { dgx_rve* r; const double* in; double* out; };
struct MultiReq {
  dgx_rve* r;
  int mode, K, K2, slot;     // slot: which of the RVE's two partial buffers
  const double* a;
  const double* b;
  const double* v[32];
  double* out;               // host, K + K2 values
};

struct IssueCount { int64_t launches = 0, h2d = 0, d2h = 0; };
struct GraphEntry {
  std::string sig;
  cudaGraphExec_t exec;
  IssueCount count;
  int64_t last_use;
};
constexpr size_t GRAPH_CACHE = 16;

constexpr int TUNE_TRIALS = 5;               // interleaved timed rounds per constitutive launch variant
// Rounds of at least this many points (two full waves of 128-point tiles at 4 blocks per
// SM) take the launch variant measured best for large work (mixed form: 128 points at 4
// blocks per SM, 1.54 ms per 64^3 launch against 1.65 at 3 and 1.81 at 2; FP64 form: 128
// points at 2 blocks per SM, 3.82 ms against 3.86 and 3.90); the online tuner decides
// for smaller rounds, where the block size and the wave count matter.
constexpr long long LARGE_ROUND_POINTS = 152LL * 128 * 4 * 2;
constexpr int LARGE_VARIANT_MIXED = 5, LARGE_VARIANT_FP64 = 1;

// ------------------------------------------------------------------ members' vector ops
// The NGMRES vector operations a member's host logic decides between two rounds
// (x^M = x - F, the combination x^A = c0 x^M + sum beta_i x_i, the history copies) are
// recorded and run at the start of the next round as one launch per position in the
// members' sequences, instead of one API call each.  The arithmetic per element is that
// of k_axpy / k_combine (solver.cu), so results are bitwise the same.
constexpr int PREOP_MAX_L = 30;       // NGMRES window (ngmres_m <= 30)
constexpr int PREOP_LEVELS = 4;       // ops a member records between two rounds (at most 3)
struct PreOp {
  int kind;                           // 0 copy z = x, 1 axpy z = x + a y, 2 combine z = a x + sum_i beta_i v_i
  int l;
  int64_t n;
  double* z;
  const double* x;
  const double* y;
  double a;
  double beta[PREOP_MAX_L];
  const double* v[PREOP_MAX_L];
};

__global__ void __launch_bounds__(256) k_preops(const PreOp* __restrict__ ops) {
  const PreOp& op = ops[blockIdx.y];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (op.kind == 0) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < op.n; t += stride) op.z[t] = op.x[t];
  } else if (op.kind == 1) {
    const double a = op.a;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < op.n; t += stride) op.z[t] = op.x[t] + a * op.y[t];
  } else {
    __shared__ double sb[32];
    if (threadIdx.x < 32) sb[threadIdx.x] = threadIdx.x < op.l ? op.beta[threadIdx.x] : 0.0;
    __syncthreads();
    const double c0 = op.a;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < op.n; t += stride) {
      double v = op.x[t] * c0;
      for (int i = 0; i < op.l; ++i) v += sb[i] * op.v[i][t];
      op.z[t] = v;
    }
  }
}

struct Executor {
  cudaStream_t st = nullptr;
  int cap = 0;                               // residual items per round; 2 cap reductions
  ConsItem* d_cons = nullptr; SpecItem* d_spec = nullptr; MultiItem* d_multi = nullptr;
  int* d_ill = nullptr; double* d_Pav = nullptr; double* d_aim = nullptr; double* d_rms = nullptr;
  double* d_mout = nullptr; unsigned long long* d_queue = nullptr;
  int qcap = 16;                               // tile queues: one per constitutive group of a round
  ConsItem* h_cons = nullptr; SpecItem* h_spec = nullptr; MultiItem* h_multi = nullptr;
  int* h_ill = nullptr; double* h_Pav = nullptr; double* h_rms = nullptr;
  double* h_mout = nullptr;
  BcItem* d_bcitem = nullptr; BcItem* h_bcitem = nullptr;
  PreOp* d_preop = nullptr; PreOp* h_preop = nullptr;   // the members' recorded vector ops, by level
  double* d_bcout = nullptr; double* h_bcout = nullptr;
  ConsCounters* cnt = nullptr;
  bool own_cnt = false;
  int cons_variant = 1, resident = 0;          // launch variant (points per block, blocks per SM)
  // autotuner: the constitutive launch variant (points per block, blocks per SM),
  // chosen online from the median cost per counted FP64 flop of five interleaved
  // rounds per variant, and per grid the FFT tile shape, timed on the first round's data
  // (results do not depend on either)
  bool tune_cons = true, tune_spec = true;
  bool variant_pinned = false;                 // DGX_CONS_VARIANT or an explicit block size
  int res_by_variant[2][CONS_VARIANTS] = {};   // [mixed form][variant]: resident blocks
  double cons_cost[CONS_VARIANTS][5] = {};     // TUNE_TRIALS per variant
  int cons_trials[CONS_VARIANTS] = {}, cons_round = 0, tune_skipped = 0;
  ConsCounters cnt_last{};
  ConsCounters* h_cnt = nullptr;
  double* h_tan = nullptr;                     // pinned: C_volAvg, C_minMaxAvg (162) per tangent request
  std::map<std::tuple<int, int, int, double, double, double, int, int, int>, SpecLaunch> spec_tuned;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // [4], [5]: a round's first and last copy
  double t_ms[3] = {0, 0, 0};
  // host wall time of the rounds (ms): [0] planning and issue, [1] waiting for the
  // device, [2] after the wait (results, tuner), [3] advancing the tasks' host logic
  double host_ms[4] = {0, 0, 0, 0};
  int64_t t_n[3] = {0, 0, 0};
  int64_t launches = 0, bytes_h2d = 0, bytes_d2h = 0, point_evals = 0, rounds = 0;
  // CUDA graphs of rounds (see ex_issue_round)
  bool use_graphs = true;
  std::vector<GraphEntry> graphs;
  std::vector<size_t> seen = std::vector<size_t>(64, 0);   // signature hashes of recent direct rounds
  size_t seen_pos = 0;
  int64_t graph_clock = 0, graph_rounds = 0, graph_captures = 0;
  std::vector<void*> dev, host;
};

void executor_destroy(Executor* e) {
  if (!e) return;
  for (GraphEntry& g : e->graphs) cudaGraphExecDestroy(g.exec);
  for (void* p : e->dev) cudaFree(p);
  for (void* p : e->host) cudaFreeHost(p);
  for (auto& v : e->ev) if (v) cudaEventDestroy(v);
  delete e;
}

template <typename T>
static dgx_status ex_alloc(Executor* e, T** d, T** h, size_t n) {
  void* p = nullptr;
  if (d) {
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) { set_err("executor: cudaMalloc failed"); return DGX_ERR_NOMEM; }
    e->dev.push_back(p); *d = (T*)p;
  }
  if (h) {
    if (cudaMallocHost(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) { set_err("executor: cudaMallocHost failed"); return DGX_ERR_NOMEM; }
    e->host.push_back(p); *h = (T*)p;
  }
  return DGX_OK;
}

dgx_status executor_create(int cap, cudaStream_t st, ConsCounters* cnt, int cons_block, Executor** out) {
  Executor* e = new Executor();
  e->st = st; e->cap = cap;
  e->cons_variant = cons_block == 64 ? 0 : cons_block == 256 ? 2 : cons_block == 32 ? 4 : 1;   // <= 0: autotuned
  dgx_status s = DGX_OK;
#define EA(d, h, n) do { s = ex_alloc(e, d, h, n); if (s != DGX_OK) { executor_destroy(e); return s; } } while (0)
  EA(&e->d_cons, &e->h_cons, cap);
  EA(&e->d_spec, &e->h_spec, cap);
  EA(&e->d_multi, &e->h_multi, 2 * cap);
  EA(&e->d_preop, &e->h_preop, (size_t)PREOP_LEVELS * cap);
  EA(&e->d_ill, &e->h_ill, cap);
  EA(&e->d_Pav, &e->h_Pav, 9 * cap);
  EA(&e->d_aim, (double**)nullptr, 9 * cap);
  EA(&e->d_rms, &e->h_rms, cap);
  EA(&e->d_mout, &e->h_mout, 64 * 2 * cap);
  EA(&e->d_bcitem, &e->h_bcitem, cap);
  EA(&e->d_bcout, &e->h_bcout, 10 * cap);
  e->qcap = std::max(16, cap);
  EA(&e->d_queue, (unsigned long long**)nullptr, e->qcap);
  EA((ConsCounters**)nullptr, &e->h_cnt, 1);
  EA((double**)nullptr, &e->h_tan, 162 * (size_t)cap);
  if (cnt) e->cnt = cnt;
  else { EA(&e->cnt, (ConsCounters**)nullptr, 1); e->own_cnt = true; cudaMemset(e->cnt, 0, sizeof(ConsCounters)); }
#undef EA
  for (auto& v : e->ev) cudaEventCreate(&v);
  for (int k = 0; k < CONS_VARIANTS; ++k)
    for (int m = 0; m < 2; ++m) e->res_by_variant[m][k] = constitutive_batch_resident(k, m == 1);
  e->resident = e->res_by_variant[0][e->cons_variant];
  const char* at = std::getenv("DGX_AUTOTUNE");
  const bool tune = !(at && at[0] == '0');
  e->tune_cons = tune && cons_block <= 0;       // an explicit block size is kept
  e->variant_pinned = cons_block > 0;
  const char* cv = std::getenv("DGX_CONS_VARIANT");   // pin a launch variant (0..4) for measurements
  if (cv && cv[0] >= '0' && cv[0] < '0' + CONS_VARIANTS && cv[1] == 0) {
    e->cons_variant = cv[0] - '0';
    e->resident = e->res_by_variant[0][e->cons_variant];
    e->tune_cons = false;
    e->variant_pinned = true;
  }
  e->tune_spec = tune;
  const char* gr = std::getenv("DGX_GRAPHS");          // 0: launch every round directly
  e->use_graphs = !(gr && gr[0] == '0');
  if (cudaMemcpyAsync(&e->cnt_last, e->cnt, sizeof(ConsCounters), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) { executor_destroy(e); set_err("executor: counters"); return DGX_ERR_CUDA; }
  *out = e;
  return DGX_OK;
}

void executor_stats(const Executor* e, double ms[3], int64_t n[3], int64_t* launches, int64_t* h2d_b, int64_t* d2h_b,
                    int64_t* graph_rounds) {
  for (int i = 0; i < 2; ++i) { ms[i] += e->t_ms[i]; n[i] += e->t_n[i]; }
  *launches += e->launches; *h2d_b += e->bytes_h2d; *d2h_b += e->bytes_d2h;
  if (graph_rounds) *graph_rounds += e->graph_rounds;
}

// equal grids (and spectral precision, derivative, geometry) share a launch
typedef std::tuple<int, int, int, double, double, double, int, int, int> GridKey;
static GridKey grid_key(const dgx_rve* r) {
  return GridKey(r->cells[0], r->cells[1], r->cells[2], r->geom[0], r->geom[1], r->geom[2], r->num.precision,
                 r->num.derivative, r->num.divergence_correction);
}

// FFT tile shape of a grid: the tuned one, or (first time, when tuning) chosen per pass.
// Each pass's time depends only on its own tile (x lines per block, x-frequencies per y
// block, x-frequencies per z block), so every dimension is scanned with the others at
// their defaults and the fastest value of each is kept.  Every candidate is timed on this group's own convolution and computes
// the same result.
static const SpecLaunch& spec_tiles(Executor* e, const GridKey& key, dgx_rve* r0, const SpecItem* items, int cnt,
                                    const GammaArgs& ga) {
  auto it = e->spec_tuned.find(key);
  if (it != e->spec_tuned.end()) return it->second;
  const SpecLaunch& base = r0->sl;
  if (!e->tune_spec) return e->spec_tuned.emplace(key, base).first->second;
  const bool fp32 = r0->num.precision == 1;
  const size_t cs = fp32 ? sizeof(float2) : sizeof(double2);
  const SpecGeom& g = base.g;
  auto time_of = [&](const SpecLaunch& L) -> float {
    if (!spec_prepare(L, fp32)) return 1e30f;
    // best of three, on at most four of the group's RVEs (the tile choice is per RVE)
    float ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e->ev[2], e->st);
      spec_convolve_batch(L, fp32, r0->ax[0].plan, r0->ax[1].plan, r0->ax[2].plan, items, std::min(cnt, 4), ga,
                          e->st);
      cudaEventRecord(e->ev[3], e->st);
      cudaEventSynchronize(e->ev[3]);
      float t = 0.f;
      cudaEventElapsedTime(&t, e->ev[2], e->ev[3]);
      ms = std::min(ms, t);
    }
    e->launches += 15;
    return cudaGetLastError() == cudaSuccess ? ms : 1e30f;
  };
  int best[3] = {base.LX, base.TIy, base.TIz};
  const float t0 = time_of(base);
  for (int d = 0; d < 3; ++d) {
    float bt = t0;
    const int v0 = d == 0 ? base.LX : d == 1 ? base.TIy : base.TIz;
    // x: 1/2 .. 8x the default; y and z: every tile width up to 16 x-frequencies (the
    // z pass holds a whole tile's 9 components in shared memory, so its width sets both
    // the blocks per SM and the number of waves), plus 2x and 4x the default for y
    int cand[24], nc = 0;
    if (d == 0) { cand[nc++] = v0 / 2; cand[nc++] = 2 * v0; cand[nc++] = 4 * v0; cand[nc++] = 8 * v0; }
    else {
      for (int v = 1; v <= 16; ++v) cand[nc++] = v;
      if (d == 1) { cand[nc++] = 2 * v0; cand[nc++] = 4 * v0; }
    }
    for (int f = 0; f < nc; ++f) {
      const int v = cand[f];
      if (v < 1 || v == v0 || (d > 0 && v > g.N0r) || (d == 0 && v > 9 * g.N1 * g.N2)) continue;
      int t[3] = {base.LX, base.TIy, base.TIz};
      t[d] = v;
      const float ms = time_of(spec_launch_tiles(g.N0, g.N1, g.N2, cs, t[0], t[1], t[2]));
      if (ms < bt) { bt = ms; best[d] = v; }
    }
  }
  SpecLaunch L = spec_launch_tiles(g.N0, g.N1, g.N2, cs, best[0], best[1], best[2]);
  if (!spec_prepare(L, fp32)) L = base;
  return e->spec_tuned.emplace(key, L).first->second;
}

// ------------------------------------------------------------------ round plan, issue and graph
// A round is planned on the host (tables staged in pinned memory, every launch
// parameter fixed) and then issued: directly, or as a CUDA graph captured from the
// same issue code.  The graph's copy nodes read the staged tables from the same
// pinned buffers at every replay, so a graph depends only on the launch parameters:
// the plan's signature lists every value a launch takes (counts, grid sizes, the
// material parameters, the FFT plans with their twiddle pointers, the Gamma
// arguments), and a graph is replayed only for a round whose signature is identical.
struct ConsGroup { int j0, cnt, grid; long long tiles; const MatParams* mp; };
struct SpecGroup {
  GridKey key;
  dgx_rve* r0;
  const SpecLaunch* L;      // null: not tuned yet (tuned while the round is issued directly)
  GammaArgs ga;
  int o, cnt;
};
struct RoundPlan {
  int n = 0, nm = 0, maxnb = 1, variant = 1;
  int npre[PREOP_LEVELS] = {0, 0, 0, 0}, prenb[PREOP_LEVELS] = {0, 0, 0, 0};   // ops and blocks per level
  bool cnt_d2h = false;
  std::vector<ConsGroup> cons;
  std::vector<SpecGroup> spec;
};

struct Sig {
  std::string b;
  void raw(const void* p, size_t n) { b.append(reinterpret_cast<const char*>(p), n); }
  template <typename T> void put(const T& v) { raw(&v, sizeof(T)); }
};
// MatParams without its tail padding (the bytes the kernel parameter carries)
constexpr size_t MATPARAMS_BYTES = offsetof(MatParams, a_quarters) + sizeof(int);

static std::string plan_signature(const RoundPlan& p) {
  Sig s;
  s.put(p.n); s.put(p.nm); s.put(p.maxnb); s.put(p.variant); s.put(p.cnt_d2h);
  for (int k = 0; k < PREOP_LEVELS; ++k) { s.put(p.npre[k]); s.put(p.prenb[k]); }
  for (const ConsGroup& c : p.cons) { s.put(c.j0); s.put(c.cnt); s.put(c.grid); s.put(c.tiles); s.raw(c.mp, MATPARAMS_BYTES); }
  for (const SpecGroup& g : p.spec) {
    const SpecLaunch& L = *g.L;
    s.put(L.g.N0); s.put(L.g.N1); s.put(L.g.N2); s.put(L.g.N0r); s.put(L.g.N); s.put(L.g.Nh);
    s.put(L.LX); s.put(L.TIy); s.put(L.TIz); s.put(L.smx); s.put(L.smy); s.put(L.smz);
    s.put(L.nbx); s.put(L.nby); s.put(L.nbz); s.put(L.ndiv);
    const GammaArgs& a = g.ga;
    s.put(a.xi_x); s.put(a.xi_y); s.put(a.xi_z); s.raw(a.resc, sizeof(a.resc)); s.put(a.C_ref); s.put(a.aim);
    s.put(a.fw[0]); s.put(a.fw[1]); s.put(a.fw[2]); s.raw(a.fw_h4, sizeof(a.fw_h4)); s.put(a.gtab);
    s.put(a.do_gamma); s.put(a.do_div); s.put(a.store_fwd); s.put(a.zsign); s.put(a.div_part);
    for (int k = 0; k < 3; ++k) {
      const AxisPlan& ap = g.r0->ax[k].plan;
      s.put(ap.n); s.put(ap.nstages); s.raw(ap.radix, sizeof(ap.radix)); s.put(ap.tw); s.put(ap.twf);
    }
    s.put(g.r0->num.precision); s.put(g.r0->sl.ndiv); s.put(g.r0->wgt); s.put(g.r0->cells[0]);
    s.put(g.o); s.put(g.cnt);
  }
  return s.b;
}

// stage the fused reductions of every request (results after the round's sync)
static dgx_status ex_multi_stage(Executor* e, std::vector<MultiReq>& q, RoundPlan& p) {
  const int n = (int)q.size();
  if (n > 2 * e->cap) { set_err("executor: %d reductions exceed capacity", n); return DGX_ERR_STATE; }
  int maxnb = 1;
  for (int i = 0; i < n; ++i) {
    dgx_rve* r = q[i].r;
    MultiItem& it = e->h_multi[i];
    it.a = q[i].a; it.b = q[i].b;
    for (int k = 0; k < 32; ++k) it.v[k] = k < q[i].K ? q[i].v[k] : nullptr;
    it.mode = q[i].mode; it.K = q[i].K; it.K2 = q[i].K2; it.nb = r->nb_red; it.n = 9 * r->N;
    it.part = r->d_redpart + (int64_t)64 * r->nb_red * q[i].slot;
    it.out = e->d_mout + 64 * i;
    maxnb = std::max(maxnb, r->nb_red);
  }
  p.nm = n; p.maxnb = maxnb;
  return DGX_OK;
}

// The device work of a planned round, in stream order: constitutive pass, P_av, stress
// BC step, spectral pass with the divergence RMS, then the fused reductions, and the
// copies of the results to the pinned host buffers.  capture: recorded into a graph
// (event records become event nodes; nothing runs until the graph is launched).
static dgx_status ex_issue(Executor* e, RoundPlan& p, bool capture, IssueCount& c) {
  cudaStream_t st = e->st;
  auto rec = [&](int k) {
    return capture ? cudaEventRecordWithFlags(e->ev[k], st, cudaEventRecordExternal) : cudaEventRecord(e->ev[k], st);
  };
  auto h2d = [&](void* d, const void* h, size_t b) { c.h2d += (int64_t)b; return cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, st); };
  auto d2h = [&](void* h, const void* d, size_t b) { c.d2h += (int64_t)b; return cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, st); };
  const int n = p.n;
  CK(rec(4));
  {
    int tot = 0;
    for (int k = 0; k < PREOP_LEVELS; ++k) tot += p.npre[k];
    if (tot > 0) {
      CK(h2d(e->d_preop, e->h_preop, sizeof(PreOp) * tot));
      int off = 0;
      for (int k = 0; k < PREOP_LEVELS; ++k) {
        if (p.npre[k] == 0) continue;
        k_preops<<<dim3(p.prenb[k], p.npre[k]), 256, 0, st>>>(e->d_preop + off);
        c.launches++;
        off += p.npre[k];
      }
    }
  }
  if (n > 0) {
    CK(cudaMemsetAsync(e->d_ill, 0, sizeof(int) * n, st));
    CK(cudaMemsetAsync(e->d_queue, 0, sizeof(unsigned long long) * e->qcap, st));
    CK(h2d(e->d_cons, e->h_cons, sizeof(ConsItem) * n));
    CK(h2d(e->d_bcitem, e->h_bcitem, sizeof(BcItem) * n));
    CK(h2d(e->d_spec, e->h_spec, sizeof(SpecItem) * n));
    CK(rec(0));
    for (size_t g = 0; g < p.cons.size(); ++g) {
      const ConsGroup& cg = p.cons[g];
      launch_constitutive_batch(*cg.mp, e->d_cons + cg.j0, cg.cnt, cg.tiles, e->d_queue + g, e->cnt, st, p.variant,
                                cg.grid);
      c.launches++;
    }
    CK(rec(1));
    launch_pav_finish_batch(e->d_cons, n, e->d_Pav, st);
    k_bc_batch<<<n, 32, 0, st>>>(e->d_bcitem);
    c.launches += 2;
    // a grid seen for the first time is tuned here, on this round's own data (direct issue only)
    for (SpecGroup& g : p.spec)
      if (!g.L) g.L = &spec_tiles(e, g.key, g.r0, e->d_spec + g.o, g.cnt, g.ga);
    CK(rec(2));
    for (const SpecGroup& g : p.spec) {
      dgx_rve* r0 = g.r0;
      spec_convolve_batch(*g.L, r0->num.precision == 1, r0->ax[0].plan, r0->ax[1].plan, r0->ax[2].plan,
                          e->d_spec + g.o, g.cnt, g.ga, st);
      spec_div_finish_batch(e->d_spec + g.o, g.cnt, r0->sl.ndiv, r0->wgt, r0->cells[0], st);
      c.launches += 6;
    }
    CK(rec(3));
    CK(d2h(e->h_Pav, e->d_Pav, sizeof(double) * 9 * n));
    CK(d2h(e->h_ill, e->d_ill, sizeof(int) * n));
    CK(d2h(e->h_rms, e->d_rms, sizeof(double) * n));
    CK(d2h(e->h_bcout, e->d_bcout, sizeof(double) * 10 * n));
    if (p.cnt_d2h) CK(d2h(e->h_cnt, e->cnt, sizeof(ConsCounters)));
  }
  if (p.nm > 0) {
    CK(h2d(e->d_multi, e->h_multi, sizeof(MultiItem) * p.nm));
    k_multi_batch<<<dim3(p.maxnb, p.nm), RB, 0, st>>>(e->d_multi);
    k_multi_finish_batch<<<dim3(64, p.nm), 32, 0, st>>>(e->d_multi);
    c.launches += 2;
    CK(d2h(e->h_mout, e->d_mout, sizeof(double) * 64 * p.nm));
  }
  CK(rec(5));
  CK(cudaGetLastError());
  return DGX_OK;
}

static void ex_count(Executor* e, const IssueCount& c) {
  e->launches += c.launches; e->bytes_h2d += c.h2d; e->bytes_d2h += c.d2h;
}

// Issue a planned round: replay the graph of an identical earlier round, capture one
// for a signature seen for the second time, else launch directly.  Graphs are kept
// per executor (least recently used out beyond GRAPH_CACHE).
static dgx_status ex_issue_round(Executor* e, RoundPlan& p) {
  bool graphable = e->use_graphs && !p.cnt_d2h && (p.n > 0 || p.nm > 0);
  for (const SpecGroup& g : p.spec) graphable &= g.L != nullptr;
  IssueCount c;
  if (!graphable) {
    TRY(ex_issue(e, p, false, c));
    ex_count(e, c);
    return DGX_OK;
  }
  std::string sig = plan_signature(p);
  for (GraphEntry& g : e->graphs)
    if (g.sig == sig) {
      g.last_use = ++e->graph_clock;
      CK(cudaGraphLaunch(g.exec, e->st));
      ex_count(e, g.count);
      e->graph_rounds++;
      return DGX_OK;
    }
  const size_t h = std::hash<std::string>{}(sig);
  bool seen = false;
  for (size_t v : e->seen) seen |= v == h;
  if (!seen) {
    e->seen[e->seen_pos++ % e->seen.size()] = h;
    TRY(ex_issue(e, p, false, c));
    ex_count(e, c);
    return DGX_OK;
  }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeRelaxed));
  dgx_status s = ex_issue(e, p, true, c);
  cudaError_t ce = cudaStreamEndCapture(e->st, &graph);
  if (s == DGX_OK && ce == cudaSuccess && graph) ce = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (s != DGX_OK || ce != cudaSuccess || !exec) {
    // capture refused: this executor launches directly from now on
    (void)cudaGetLastError();
    e->use_graphs = false;
    IssueCount d;
    TRY(ex_issue(e, p, false, d));
    ex_count(e, d);
    return DGX_OK;
  }
  if (e->graphs.size() >= GRAPH_CACHE) {
    auto lru = std::min_element(e->graphs.begin(), e->graphs.end(),
                                [](const GraphEntry& a, const GraphEntry& b) { return a.last_use < b.last_use; });
    cudaGraphExecDestroy(lru->exec);
    e->graphs.erase(lru);
  }
  e->graphs.push_back(GraphEntry{std::move(sig), exec, c, ++e->graph_clock});
  e->graph_captures++;
  CK(cudaGraphLaunch(exec, e->st));
  ex_count(e, c);
  e->graph_rounds++;
  return DGX_OK;
}

// One round of device work with a single host synchronisation: the residual
// evaluations R = Gamma * P(X) of every request (form_residual: constitutive pass,
// P_av, stress BC step, spectral pass, divergence RMS), then the fused reductions
// (which may read the residuals of this round).
static double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// npre / maxn: the members' recorded vector ops staged in h_preop by level (counts and
// the longest vector of each level)
static dgx_status ex_round(Executor* e, std::vector<ResReq>& q, std::vector<MultiReq>& mq,
                           const int npre[PREOP_LEVELS], const int64_t maxn[PREOP_LEVELS]) {
  auto h0 = std::chrono::steady_clock::now();
  const int n = (int)q.size();
  if (n > e->cap) { set_err("executor: %d residual requests exceed capacity %d", n, e->cap); return DGX_ERR_STATE; }
  int cand = -1;
  bool large_round = false;
  std::vector<int> slot_of(n);
  RoundPlan p;
  p.n = n;
  for (int k = 0; k < PREOP_LEVELS; ++k) {
    p.npre[k] = npre[k];
    p.prenb[k] = npre[k] ? (int)std::min<int64_t>(1216, (maxn[k] + 255) / 256) : 0;
  }
  if (n > 0) {
    // constitutive pass: items grouped by material, largest RVEs first in the tile queue
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      int c = memcmp(&q[a].r->mp, &q[b].r->mp, sizeof(MatParams));
      if (c != 0) return c < 0;
      return q[a].r->N > q[b].r->N;
    });
    long long round_points = 0;
    bool round_mixed = true;
    for (int i = 0; i < n; ++i) { round_points += q[i].r->N; round_mixed &= q[i].r->mp.mixed != 0; }
    large_round = !e->variant_pinned && round_points >= LARGE_ROUND_POINTS;
    if (e->tune_cons && !large_round) {
      cand = e->cons_round % CONS_VARIANTS;
      if (e->cons_trials[cand] >= TUNE_TRIALS) cand = -1;
    }
    p.variant = large_round ? (round_mixed ? LARGE_VARIANT_MIXED : LARGE_VARIANT_FP64)
                            : (cand >= 0 ? cand : e->cons_variant);
    const int BS = cons_variant_bs(p.variant);
    for (int j = 0; j < n; ++j) slot_of[order[j]] = j;
    {
      long long tiles = 0;
      int gstart = 0;
      auto close_group = [&](int jend) {
        const int resident = e->res_by_variant[q[order[gstart]].r->mp.mixed ? 1 : 0][p.variant];
        const int grid = (int)std::max<long long>(1, std::min<long long>(tiles, resident));
        p.cons.push_back(ConsGroup{gstart, jend - gstart, grid, tiles, &q[order[gstart]].r->mp});
      };
      for (int j = 0; j < n; ++j) {
        dgx_rve* r = q[order[j]].r;
        if (j > 0 && memcmp(&r->mp, &q[order[j - 1]].r->mp, sizeof(MatParams)) != 0) {
          close_group(j); gstart = j; tiles = 0;
        }
        ConsItem& it = e->h_cons[j];
        it.ps = r->ps; it.F = q[order[j]].in; it.ldF = r->N; it.dt = r->delta_t; it.wgt = r->wgt;
        it.Ppart = r->d_Ppart; it.ill = e->d_ill + j; it.tile0 = tiles;
        it.warm = (r->mp.mixed && r->evals_in_step > 0) ? 1 : 0;
        r->evals_in_step++;
        tiles += (r->N + BS - 1) / BS;
        r->n_eval++;
        r->tangent_dt = r->delta_t;
        e->point_evals += r->N;
      }
      close_group(n);
      if ((int)p.cons.size() > e->qcap) { set_err("executor: more constitutive groups than queue slots"); return DGX_ERR_STATE; }
    }
    for (int i = 0; i < n; ++i)
      e->h_bcitem[i] = BcItem{q[i].r->d_bc, e->d_Pav + 9 * slot_of[i], e->d_aim + 9 * i, e->d_bcout + 10 * i};
    // spectral items per grid group
    std::map<GridKey, std::vector<int>> gg;
    for (int i = 0; i < n; ++i) gg[grid_key(q[i].r)].push_back(i);
    int off = 0;
    for (auto& kv : gg) {
      dgx_rve* r0 = q[kv.second[0]].r;
      auto t = e->spec_tuned.find(kv.first);
      p.spec.push_back(SpecGroup{kv.first, r0, t == e->spec_tuned.end() ? nullptr : &t->second,
                                 gamma_args(r0, true, true), off, (int)kv.second.size()});
      for (int i : kv.second) {
        dgx_rve* r = q[i].r;
        SpecItem& it = e->h_spec[off++];
        it.in = r->ps.P; it.out = q[i].out; it.spec = r->spec; it.gtab = r->d_gtab; it.aim = e->d_aim + 9 * i;
        it.div_part = r->d_divpart; it.rms = e->d_rms + i;
      }
    }
    p.cnt_d2h = e->tune_cons && !large_round;
  }
  TRY(ex_multi_stage(e, mq, p));
  TRY(ex_issue_round(e, p));
  e->host_ms[0] += ms_since(h0);
  h0 = std::chrono::steady_clock::now();
  CK(cudaStreamSynchronize(e->st));
  CK(cudaGetLastError());
  e->host_ms[1] += ms_since(h0);
  h0 = std::chrono::steady_clock::now();
  struct AddOnExit {
    Executor* e; std::chrono::steady_clock::time_point t0;
    ~AddOnExit() { e->host_ms[2] += ms_since(t0); }
  } add_on_exit{e, h0};
  e->rounds++;
  if (n > 0 || p.nm > 0) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e->ev[4], e->ev[5]); e->t_ms[2] += ms; e->t_n[2]++;
  }
  if (n > 0) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]); e->t_ms[0] += ms; e->t_n[0]++;
    const float cons_ms = ms;
    cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]); e->t_ms[1] += ms; e->t_n[1]++;
    if (e->tune_cons && !large_round) {
      // cost per counted FP64 flop (the constitutive roofline's own flop model; the
      // mixed form's FP64 model when every member of the round is mixed)
      const ConsCounters& c1 = *e->h_cnt;
      bool all_mixed = true;
      for (int i = 0; i < n; ++i) all_mixed &= q[i].r->mp.mixed != 0;
      const double f_lp = FLOPS_LP, f_jac = all_mixed ? FLOPS_MX_JAC64 : FLOPS_JAC,
                   f_st = all_mixed ? FLOPS_MX_STATE64 : FLOPS_STATE, f_fpi = all_mixed ? FLOPS_MX_FPI64 : FLOPS_FPI;
      double flops = f_lp * (double)(c1.lp_iters - e->cnt_last.lp_iters) +
                     f_jac * (double)(c1.jac_iters - e->cnt_last.jac_iters) +
                     f_st * (double)(c1.state_iters - e->cnt_last.state_iters) +
                     f_fpi * (double)(c1.fpi_iters - e->cnt_last.fpi_iters);
      e->cnt_last = c1;
      // a mixed round is timed only when every member starts warm (the previous
      // evaluation of its step seeds it): cold and warm evaluations differ in cost per
      // counted flop, and nearly all of a solve's evaluations are warm (cold rounds are
      // taken too once 200 rounds have passed without completing the trials)
      bool all_warm = true;
      for (int j = 0; j < n; ++j) all_warm &= e->h_cons[j].warm != 0;
      const bool usable = !all_mixed || all_warm || ++e->tune_skipped > 200;
      if (usable) {
        if (cand >= 0 && flops > 0.0) e->cons_cost[cand][e->cons_trials[cand]++] = cons_ms / flops;
        e->cons_round++;
      }
      bool all = true;
      for (int k = 0; k < CONS_VARIANTS; ++k) all &= e->cons_trials[k] >= TUNE_TRIALS;
      if (all) {
        // median of the interleaved trials per variant
        double med[CONS_VARIANTS];
        for (int k = 0; k < CONS_VARIANTS; ++k) {
          double c[TUNE_TRIALS];
          std::copy(e->cons_cost[k], e->cons_cost[k] + TUNE_TRIALS, c);
          std::sort(c, c + TUNE_TRIALS);
          med[k] = c[TUNE_TRIALS / 2];
        }
        int best = 0;
        for (int k = 1; k < CONS_VARIANTS; ++k) if (med[k] < med[best]) best = k;
        e->cons_variant = best;
        e->resident = e->res_by_variant[0][best];
        e->tune_cons = false;
      }
    }
    // host mirrors of the device BC step and the convergence inputs
    for (int i = 0; i < n; ++i) {
      dgx_rve* r = q[i].r;
      const int j = slot_of[i];
      memcpy(r->P_av, e->h_Pav + 9 * j, 9 * sizeof(double));
      memcpy(r->F_aim, e->h_bcout + 10 * i, 9 * sizeof(double));
      r->err_BC = e->h_bcout[10 * i + 9];
      r->err_div = e->h_rms[i];
      r->tangent_fresh = false;
      if (e->h_ill[j]) r->terminally_ill = 1;
      if (!r->num.lazy_tangent) TRY(ensure_tangent(r));
    }
  }
  for (size_t i = 0; i < mq.size(); ++i)
    memcpy(mq[i].out, e->h_mout + 64 * i, sizeof(double) * (mq[i].K + mq[i].K2));
  return DGX_OK;
}

// ------------------------------------------------------------------ solver state machine
enum TState {
  T_LC_BEGIN, T_INC_BEGIN, T_SUB_CHECK, T_SOLVE_BEGIN, T_N_INIT2, T_FP_ITER, T_FP_CHECK,
  T_N_ITER, T_N_LSQ, T_N_DECIDE, T_SOLVE_END, T_SUB_AFTER, T_INC_END, T_DONE
};

struct Task {
  dgx_rve* r = nullptr;
  int mode = 0;                       // 0 one solve, 1 one increment, 2 load case
  const dgx_loadstep* steps = nullptr;
  int nsteps = 0, l = 0, inc = 0;
  dgx_inc_record* records = nullptr;
  int max_records = 0, nrec = 0;
  Output out{nullptr, nullptr, 0};    // optional result / restart output (load case mode)
  int total = 0;                      // increments completed (the results' increment number)
  int32_t conv = 0, sit = 0, sill = 0;
  TState pc = T_LC_BEGIN;
  dgx_status err = DGX_OK;
  // pending device work: bit 0 a residual evaluation, bit 1 fused reductions (run after
  // the residual of the same round when both are requested)
  int want = 0;
  const double* rin = nullptr;
  double* rout = nullptr;
  int nmq = 0;
  MultiReq mq[2];
  // increment locals (run_one_increment)
  int step_fraction = 0, iters = 0, cutbacks = 0;
  int64_t ev0 = 0;
  std::chrono::steady_clock::time_point t0;
  // SNESSolve locals
  int reason = 0, k = 0, k_restart = 1, lh = 1, ivec = 0, restart_count = 0;
  int skips = 0;                      // rounds this task's residual request was passed over
  double *X = nullptr, *F = nullptr;
  double fnorm = 0.0, fminnorm = 0.0, fMnorm = 0.0;
  std::vector<double> qm, beta, xi, tmp, tmpA;
  std::vector<PreOp> ops;             // vector ops recorded since the last round, in order
  bool done() const { return pc == T_DONE; }
  const dgx_loadstep* cur_step() const { return mode == 2 ? &steps[l] : steps; }
};

static void req_residual(Task& t, const double* in, double* out) { t.want |= 1; t.rin = in; t.rout = out; }
static void req_multi(Task& t, int mode, const double* a, const double* b, const std::vector<const double*>& vs, int K2,
                      double* out) {
  MultiReq& m = t.mq[t.nmq];
  m.r = t.r; m.mode = mode; m.a = a; m.b = b; m.K = (int)vs.size(); m.K2 = K2; m.slot = t.nmq; m.out = out;
  for (int k = 0; k < m.K; ++k) m.v[k] = vs[k];
  t.nmq++;
  t.want |= 2;
}
// Issue a member's recorded vector ops directly, in order (before work of its own on the
// stream that reads or writes the same vectors, and when more ops are recorded than a
// round takes).
static dgx_status flush_ops(Task& t) {
  dgx_rve* r = t.r;
  for (const PreOp& op : t.ops) {
    if (op.kind == 0) {
      CK(cudaMemcpyAsync(op.z, op.x, sizeof(double) * op.n, cudaMemcpyDeviceToDevice, r->st));
    } else if (op.kind == 1) {
      launch_axpy(op.z, op.x, op.a, op.y, op.n, r->st);
      r->n_launch++;
    } else {
      VecList xl{};
      for (int i = 0; i < op.l; ++i) xl.v[i] = op.v[i];
      CK(h2d(r, r->d_beta, op.beta, sizeof(double) * op.l));
      launch_combine(op.z, op.x, xl, op.l, op.a, r->d_beta, op.n, r->nb_red, r->st);
      r->n_launch++;
    }
    // the combination's coefficients are read from host memory by the copy above
    // (pageable: staged before the call returns), so the record may go
    CK(cudaGetLastError());
  }
  t.ops.clear();
  return DGX_OK;
}
static dgx_status record_op(Task& t, const PreOp& op) {
  if ((int)t.ops.size() >= PREOP_LEVELS) TRY(flush_ops(t));
  t.ops.push_back(op);
  return DGX_OK;
}
static dgx_status op_copy(Task& t, double* dst, const double* src) {
  PreOp op{};
  op.kind = 0; op.n = 9 * t.r->N; op.z = dst; op.x = src;
  return record_op(t, op);
}
static dgx_status op_axpy(Task& t, double* z, const double* x, double a, const double* y) {
  PreOp op{};
  op.kind = 1; op.n = 9 * t.r->N; op.z = z; op.x = x; op.y = y; op.a = a;
  return record_op(t, op);
}
static dgx_status op_combine(Task& t, double* z, const double* x, double c0, const double* beta, int l) {
  if (l > PREOP_MAX_L) { set_err("NGMRES window above %d", PREOP_MAX_L); return DGX_ERR_ARG; }
  PreOp op{};
  op.kind = 2; op.n = 9 * t.r->N; op.z = z; op.x = x; op.a = c0; op.l = l;
  for (int i = 0; i < l; ++i) { op.beta[i] = beta[i]; op.v[i] = t.r->Xdot[i]; }
  return record_op(t, op);
}

// run the task's host logic until it parks a device request or finishes
static dgx_status advance(Task& t) {
  dgx_rve* r = t.r;
  for (;;) {
    // states that issue work of their own on the stream run after the recorded ops
    if (!t.ops.empty() && (t.pc == T_LC_BEGIN || t.pc == T_SUB_CHECK || t.pc == T_SOLVE_BEGIN ||
                           t.pc == T_SOLVE_END || t.pc == T_INC_END || t.pc == T_DONE))
      TRY(flush_ops(t));
    switch (t.pc) {
      case T_LC_BEGIN:
        t.l = 0; t.inc = 0; t.nrec = 0; t.total = 0;
        if (t.out.result) TRY(result_write_impl(t.out.result, r, 0, r->t));
        t.pc = t.nsteps > 0 ? T_INC_BEGIN : T_DONE;
        break;
      case T_INC_BEGIN: {
        const dgx_loadstep* ls = t.cur_step();
        if (t.l != r->cur_step) { r->cur_step = t.l; r->t_0 = r->t; r->guess = ls->estimate_rate && t.l > 0; }
        t.t0 = std::chrono::steady_clock::now();
        r->dt_prev = r->dt;
        r->dt = forward_time(ls, t.inc, 2, r->cut_back_level);
        t.step_fraction = 0; t.iters = 0; t.cutbacks = 0; t.ev0 = r->n_eval;
        t.pc = T_SUB_CHECK;
        break;
      }
      case T_SUB_CHECK: {
        const dgx_loadstep* ls = t.cur_step();
        if (t.step_fraction < (int)std::pow(2, r->cut_back_level)) {
          // forward needs the tangent of the converged state: requested from the next
          // round (computed there beside the other members' work) instead of a
          // synchronous launch of its own
          if (!r->cut_back && !r->tangent_fresh) { t.want |= 4; return DGX_OK; }
          double t_remaining = ls->t + r->t_0 - r->t;
          r->t += r->dt;
          t.step_fraction++;
          TRY(dgx_solver_forward(r, r->cut_back, r->guess, r->dt, r->dt_prev, t_remaining, ls));
          if (!r->cut_back) TRY(commit(r));
          t.pc = T_SOLVE_BEGIN;
        } else {
          t.pc = T_INC_END;
        }
        break;
      }
      case T_SOLVE_BEGIN:
        TRY(solve_prologue(r));
        t.X = r->X; t.F = r->R;
        r->total_iter = 0;
        t.tmp.assign(2 * 32 + 2, 0.0);
        t.tmpA.assign(2, 0.0);
        req_residual(t, t.X, t.F);
        req_multi(t, 0, t.F, nullptr, {t.F}, 0, t.tmp.data());      // |F|^2 in the same round
        t.pc = T_N_INIT2;
        return DGX_OK;
      case T_N_INIT2: {
        t.fnorm = std::sqrt(t.tmp[0]);
        if (!std::isfinite(t.fnorm)) { t.reason = -2; t.pc = T_SOLVE_END; break; }
        t.fminnorm = t.fnorm;
        t.reason = converged(r);
        if (t.reason) { t.pc = T_SOLVE_END; break; }
        t.k = 1;
        if (r->num.solver == 1) { t.pc = T_FP_ITER; break; }
        const int m = r->num.ngmres_m;
        t.qm.assign((size_t)m * m, 0.0); t.beta.assign(m, 0.0); t.xi.assign(m, 0.0);
        TRY(op_copy(t, r->Fdot[0], t.F)); TRY(op_copy(t, r->Xdot[0], t.X));
        t.k_restart = 1; t.lh = 1; t.ivec = 0; t.restart_count = 0;
        t.pc = T_N_ITER;
        break;
      }
      // ---- fixed point: X <- X - F
      case T_FP_ITER:
        if (t.k > r->num.snes_max_it) { t.reason = -1; t.pc = T_SOLVE_END; break; }
        TRY(op_axpy(t, t.X, t.X, -1.0, t.F));
        r->total_iter = t.k;
        req_residual(t, t.X, t.F);
        req_multi(t, 0, t.F, nullptr, {t.F}, 0, t.tmp.data());
        t.pc = T_FP_CHECK;
        return DGX_OK;
      case T_FP_CHECK: {
        double fn = std::sqrt(t.tmp[0]);
        if (!std::isfinite(fn)) { t.reason = -2; t.pc = T_SOLVE_END; break; }
        t.reason = converged(r);
        if (t.reason) { t.pc = T_SOLVE_END; break; }
        t.k++;
        t.pc = T_FP_ITER;
        break;
      }
      // ---- NGMRES iteration k
      case T_N_ITER:
        if (t.k > r->num.snes_max_it) { t.reason = 0; t.pc = T_SOLVE_END; break; }
        TRY(op_axpy(t, r->XM, t.X, -1.0, t.F));             // x^M = x - F(x) (basic line search)
        r->total_iter = t.k;
        req_residual(t, r->XM, r->FM);
        {
          // |FM|^2, <FM, Fdot_i>, <Fdot_ivec, Fdot_i> in one pass, after the residual
          std::vector<const double*> vs;
          for (int i = 0; i < t.lh; ++i) vs.push_back(r->Fdot[i]);
          vs.push_back(r->FM);
          req_multi(t, 0, r->FM, r->Fdot[t.ivec], vs, t.lh, t.tmp.data());
        }
        t.pc = T_N_LSQ;
        return DGX_OK;
      case T_N_LSQ: {
        const int m = r->num.ngmres_m, l = t.lh;
        t.fMnorm = std::sqrt(t.tmp[l]);
        if (!std::isfinite(t.fMnorm)) { t.reason = -2; t.pc = T_SOLVE_END; break; }
        double nu = t.fMnorm * t.fMnorm;
        for (int i = 0; i < l; ++i) { t.xi[i] = t.tmp[i]; t.beta[i] = t.tmp[l + 1 + i]; }
        for (int i = 0; i < l; ++i) { t.qm[i + m * t.ivec] = t.beta[i]; t.qm[t.ivec + m * i] = t.beta[i]; }
        for (int i = 0; i < l; ++i) t.beta[i] = nu - t.xi[i];
        std::vector<double> H((size_t)l * l);
        for (int j = 0; j < l; ++j)
          for (int i = 0; i < l; ++i) H[i + l * j] = t.qm[i + m * j] - t.xi[i] - t.xi[j] + nu;
        if (l == 1) t.beta[0] = H[0] != 0.0 ? t.beta[0] / H[0] : 0.0;
        else lsq_svd(l, H.data(), t.beta.data());
        for (int i = 0; i < l; ++i)
          if (!std::isfinite(t.beta[i])) { set_err("NGMRES: non-finite coefficient"); return DGX_ERR_STATE; }
        double alph = 0.0;
        for (int i = 0; i < l; ++i) alph += t.beta[i];
        TRY(op_combine(t, r->XA, r->XM, 1.0 - alph, t.beta.data(), l));
        if (t.fminnorm > t.fMnorm) t.fminnorm = t.fMnorm;
        req_residual(t, r->XA, r->FA);
        // |FA|^2 ; |XA - XM|^2, |XA - Xdot_i|^2 after the residual
        req_multi(t, 0, r->FA, nullptr, {r->FA}, 0, t.tmpA.data());
        std::vector<const double*> ds;
        ds.push_back(r->XM);
        for (int i = 0; i < t.lh; ++i) ds.push_back(r->Xdot[i]);
        req_multi(t, 1, r->XA, nullptr, ds, 0, t.tmp.data());
        t.pc = T_N_DECIDE;
        return DGX_OK;
      }
      case T_N_DECIDE: {
        const int m = r->num.ngmres_m, l = t.lh;
        double fAnorm = std::sqrt(t.tmpA[0]), dnorm = std::sqrt(t.tmp[0]), dminnorm = -1.0;
        for (int i = 0; i < l; ++i) { double d = std::sqrt(t.tmp[1 + i]); if (d < dminnorm || dminnorm < 0.0) dminnorm = d; }
        bool selectA = true;
        if (fAnorm >= 2.0 * t.fminnorm) selectA = false;
        if (!(0.1 * dnorm < dminnorm || std::sqrt(t.fnorm) < 0.9 * std::sqrt(t.fminnorm))) selectA = false;
        if (selectA) { t.fnorm = fAnorm; std::swap(t.F, r->FA); std::swap(t.X, r->XA); }
        else { t.fnorm = t.fMnorm; std::swap(t.F, r->FM); std::swap(t.X, r->XM); }
        t.ivec = t.k_restart % m;
        bool selectRestart = false;
        if (0.1 * dnorm > dminnorm && std::sqrt(fAnorm) > 0.9 * std::sqrt(t.fminnorm) && l > 0) selectRestart = true;
        if (std::sqrt(fAnorm) > 2.0 * std::sqrt(t.fminnorm)) selectRestart = true;
        t.restart_count = selectRestart ? t.restart_count + 1 : 0;
        if (t.restart_count >= 2) {
          t.restart_count = 0; t.k_restart = 1; t.lh = 1; t.ivec = 0;
          const double* srcF = selectA ? r->FM : t.F;    // the x^M pair, wherever it now lives
          const double* srcX = selectA ? r->XM : t.X;
          TRY(op_copy(t, r->Fdot[0], srcF)); TRY(op_copy(t, r->Xdot[0], srcX));
        } else {
          if (t.lh < m) t.lh++;
          t.k_restart++;
          if (t.fminnorm > t.fnorm) t.fminnorm = t.fnorm;
          TRY(op_copy(t, r->Fdot[t.ivec], t.F)); TRY(op_copy(t, r->Xdot[t.ivec], t.X));
        }
        t.reason = converged(r);
        if (t.reason) { t.pc = T_SOLVE_END; break; }
        t.k++;
        t.pc = T_N_ITER;
        break;
      }
      case T_SOLVE_END: {
        // buffers rotate between X/XM/XA and R/FM/FA; the three stay distinct
        r->X = t.X; r->R = t.F;
        solve_epilogue(r, t.reason ? t.reason : -1, &t.conv, &t.sit, &t.sill);
        t.pc = t.mode == 0 ? T_DONE : T_SUB_AFTER;
        break;
      }
      case T_SUB_AFTER:
        t.iters += t.sit;
        if (t.conv) {
          r->dt_prev = r->dt; r->cut_back = 0; r->guess = 1;
        } else if (r->cut_back_level < r->num.max_cut_back) {
          r->cut_back = 1; t.step_fraction = (t.step_fraction - 1) * 2; r->cut_back_level++;
          r->t -= r->dt; r->dt /= 2; t.cutbacks++;
        } else {
          set_err("no solution found for increment %d of load step %d", t.inc + 1, t.l + 1);
          return DGX_ERR_NOT_CONVERGED;
        }
        t.pc = T_SUB_CHECK;
        break;
      case T_INC_END: {
        r->cut_back_level = std::max(0, r->cut_back - 1);
        if (t.records && (t.mode == 1 || t.nrec < t.max_records)) {
          dgx_inc_record& rec = t.records[t.mode == 1 ? 0 : t.nrec];
          rec = dgx_inc_record{};
          rec.t = r->t; rec.dt = r->dt;
          memcpy(rec.P_av, r->P_av, sizeof(rec.P_av));
          memcpy(rec.F_aim, r->F_aim, sizeof(rec.F_aim));
          TRY(field_average(r, r->X, rec.F_av));
          rec.iterations = t.iters; rec.evaluations = (int32_t)(r->n_eval - t.ev0);
          rec.converged = 1; rec.cutbacks = t.cutbacks; rec.err_div = r->err_div; rec.err_BC = r->err_BC;
          rec.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t.t0).count();
        }
        t.nrec++;
        t.total++;
        if (t.mode == 2) {
          // DamaskGrid::loop_over_loadcase output (the Fortran grid solver's cadence,
          // 1-based increment within the step)
          const int f_out = std::max(1, (int)t.cur_step()->f_out);
          if (t.out.result && (t.inc + 1) % f_out == 0) TRY(result_write_impl(t.out.result, r, t.total, r->t));
          if (t.out.restart_every > 0 && t.total % t.out.restart_every == 0)
            TRY(restart_write_impl(r, t.out.restart_path));
        }
        if (t.mode == 1) { t.pc = T_DONE; break; }
        if (++t.inc >= t.steps[t.l].N) { t.l++; t.inc = 0; }
        t.pc = t.l < t.nsteps ? T_INC_BEGIN : T_DONE;
        break;
      }
      case T_DONE:
        return DGX_OK;
    }
  }
}

// one round: serve every parked request, then advance the tasks that were served.
// A task that fails is finished with its error; the others go on.
// cells x increments still to run (including the current one): the work left
static double remaining_work(const Task& t) {
  if (t.mode != 2) return (double)t.r->N;
  double inc = 0.0;
  for (int l = t.l; l < t.nsteps; ++l) inc += (l == t.l) ? (t.steps[l].N - t.inc) : t.steps[l].N;
  return (double)t.r->N * std::max(1.0, inc);
}

// One round: serve the parked requests (one host synchronisation), then advance the
// tasks that were served.  With a point budget, residual evaluations are served least
// remaining work first until the budget is filled (at least one per round); a task
// passed over gains priority each round it waits (its work counts half per skipped
// round), so none starves.  Requests of reductions alone are cheap and always served.
// A task that fails is finished with its error; the others go on.
static dgx_status serve_round(Executor* e, std::vector<Task*>& tasks, int64_t point_budget) {
  std::vector<Task*> res_tasks, served, tan_tasks;
  for (Task* t : tasks) {
    if (t->done() || t->want == 0) continue;
    if (t->want & 4) { tan_tasks.push_back(t); served.push_back(t); continue; }   // tangent only
    if (t->want & 1) res_tasks.push_back(t);
    else served.push_back(t);                         // reductions only
  }
  // the requested tangents go first on the round's stream; their averages are read
  // back with the round (pinned staging) and take effect after its synchronisation
  for (size_t i = 0; i < tan_tasks.size(); ++i) {
    dgx_rve* r = tan_tasks[i]->r;
    if (r->timing) CK(cudaEventRecord(r->ev[4], e->st));
    launch_tangent(r->mp, r->ps, r->tangent_dt, r->d_dPdF, r->N, r->d_tpart, e->st);
    if (r->timing) CK(cudaEventRecord(r->ev[5], e->st));
    launch_tangent_finish(r->d_tpart, r->nb_tan, r->wgt, r->d_Cvol, r->d_Cmm, e->st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e->h_tan + 162 * i, r->d_Cvol, 81 * sizeof(double), cudaMemcpyDeviceToHost, e->st));
    CK(cudaMemcpyAsync(e->h_tan + 162 * i + 81, r->d_Cmm, 81 * sizeof(double), cudaMemcpyDeviceToHost, e->st));
    r->n_launch += 2;
    r->bytes_d2h += 162 * sizeof(double);
  }
  int64_t total = 0;
  for (Task* t : res_tasks) total += t->r->N;
  if (point_budget > 0 && total > point_budget) {
    std::stable_sort(res_tasks.begin(), res_tasks.end(), [](const Task* a, const Task* b) {
      return std::ldexp(remaining_work(*a), -std::min(a->skips, 60)) <
             std::ldexp(remaining_work(*b), -std::min(b->skips, 60));
    });
    int64_t used = 0;
    size_t take = 0;
    while (take < res_tasks.size() && (take == 0 || used + res_tasks[take]->r->N <= point_budget))
      used += res_tasks[take++]->r->N;
    for (size_t k = take; k < res_tasks.size(); ++k) res_tasks[k]->skips++;
    res_tasks.resize(take);
  }
  std::vector<ResReq> rq;
  for (Task* t : res_tasks) { rq.push_back({t->r, t->rin, t->rout}); t->skips = 0; served.push_back(t); }
  std::vector<MultiReq> mq;
  for (Task* t : served) for (int i = 0; i < t->nmq; ++i) mq.push_back(t->mq[i]);
  // the served members' recorded vector ops, staged level by level (op k of every member
  // in one launch at the start of the round)
  int npre[PREOP_LEVELS] = {0, 0, 0, 0};
  int64_t maxn[PREOP_LEVELS] = {0, 0, 0, 0};
  {
    int off = 0;
    for (int k = 0; k < PREOP_LEVELS; ++k)
      for (Task* t : served)
        if ((int)t->ops.size() > k) {
          if (off >= PREOP_LEVELS * e->cap) { set_err("executor: vector ops exceed capacity"); return DGX_ERR_STATE; }
          e->h_preop[off++] = t->ops[k];
          npre[k]++;
          maxn[k] = std::max(maxn[k], t->ops[k].n);
        }
    for (Task* t : served) t->ops.clear();
  }
  TRY(ex_round(e, rq, mq, npre, maxn));
  if (!tan_tasks.empty()) {
    CK(cudaStreamSynchronize(e->st));
    for (size_t i = 0; i < tan_tasks.size(); ++i) {
      dgx_rve* r = tan_tasks[i]->r;
      memcpy(r->C_volAvg, e->h_tan + 162 * i, 81 * sizeof(double));
      memcpy(r->C_minMaxAvg, e->h_tan + 162 * i + 81, 81 * sizeof(double));
      r->n_tangent++;
      r->tangent_fresh = true;
      if (r->timing) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r->ev[4], r->ev[5]); r->t_ms[2] += ms; r->t_n[2]++;
      }
    }
  }
  const auto h0 = std::chrono::steady_clock::now();
  for (Task* t : served) {
    t->want = 0; t->nmq = 0;
    dgx_status s = advance(*t);
    if (s != DGX_OK) { t->err = s; t->pc = T_DONE; }
  }
  e->host_ms[3] += ms_since(h0);
  return DGX_OK;
}

static dgx_status ensure_executor(dgx_rve* r) {
  if (r->ex) return DGX_OK;
  return executor_create(1, r->st, r->d_cnt, r->cons_block_forced ? r->cons_block : 0, &r->ex);
}

// a solve (mode 0), one increment (mode 1) or a load case (mode 2) of one RVE as a batch of one
dgx_status run_single(dgx_rve* r, int mode, const dgx_loadstep* steps, int n_or_index, int inc,
                      dgx_inc_record* records, int max_records, int32_t* n_records, int32_t* conv, int32_t* iterations,
                      int32_t* ill, const Output* out) {
  TRY(ensure_executor(r));
  Task t;
  if (out) t.out = *out;
  t.r = r; t.mode = mode; t.steps = steps; t.records = records; t.max_records = max_records;
  if (mode == 0) t.pc = T_SOLVE_BEGIN;
  else if (mode == 1) { t.pc = T_INC_BEGIN; t.l = n_or_index; t.inc = inc; t.nsteps = 1; }
  else { t.pc = T_LC_BEGIN; t.nsteps = n_or_index; }
  std::vector<Task*> tasks{&t};
  dgx_status s = advance(t);
  while (s == DGX_OK && !t.done()) {
    s = serve_round(r->ex, tasks, 0);
    if (s == DGX_OK && t.err != DGX_OK) s = t.err;
  }
  if (s == DGX_OK) s = t.err;
  if (n_records) *n_records = std::min(t.nrec, max_records);
  if (mode == 0) { if (conv) *conv = t.conv; if (iterations) *iterations = t.sit; if (ill) *ill = t.sill; }
  return s;
}

}  // namespace dgx

// ------------------------------------------------------------------ batch C ABI
using namespace dgx;

struct dgx_batch {
  cudaStream_t st = nullptr;
  Executor* ex = nullptr;
  int cap = 0;
  struct Member { dgx_rve* r; Task* t; int active; };
  std::vector<Member> members;      // slot = index; removed members keep their slot (r = null)
  std::atomic<int64_t> round_points{0};   // residual points served per round (0: all)
};

extern "C" dgx_status dgx_batch_create(int32_t capacity, int32_t cons_block, dgx_batch** out) {
  if (!out || capacity < 1 || capacity > 65535) { set_err("dgx_batch_create: capacity in [1, 65535]"); return DGX_ERR_ARG; }
  dgx_batch* b = new dgx_batch();
  b->cap = capacity;
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
    set_err("dgx_batch_create: stream"); delete b; return DGX_ERR_CUDA;
  }
  dgx_status s = executor_create(capacity, b->st, nullptr, cons_block, &b->ex);
  if (s != DGX_OK) { cudaStreamDestroy(b->st); delete b; return s; }
  *out = b;
  return DGX_OK;
}

static void batch_detach(dgx_batch::Member& m) {
  if (!m.r) return;
  cudaStreamSynchronize(m.r->st);
  m.r->st = m.r->home_st;
  m.r->in_batch = 0;
  delete m.t;
  m.t = nullptr; m.r = nullptr; m.active = 0;
}

extern "C" void dgx_batch_destroy(dgx_batch* b) {
  if (!b) return;
  for (auto& m : b->members) batch_detach(m);
  executor_destroy(b->ex);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

extern "C" dgx_status dgx_batch_add(dgx_batch* b, dgx_rve* r, int32_t nsteps, const dgx_loadstep* steps,
                                    dgx_inc_record* records, int32_t max_records, int32_t* slot) {
  if (!b || !r || !steps || nsteps < 1) { set_err("dgx_batch_add: null argument"); return DGX_ERR_ARG; }
  if (r->in_batch) { set_err("dgx_batch_add: RVE already in a batch"); return DGX_ERR_STATE; }
  int active = 0;
  for (auto& m : b->members) active += m.active;
  if (active >= b->cap) { set_err("dgx_batch_add: batch full (%d members)", b->cap); return DGX_ERR_NOMEM; }
  CK(cudaStreamSynchronize(r->st));
  r->home_st = r->st;
  r->st = b->st;
  r->in_batch = 1;
  dgx_status s = dgx_solver_init(r);
  Task* t = new Task();
  t->r = r; t->mode = 2; t->steps = steps; t->nsteps = nsteps; t->records = records; t->max_records = max_records;
  t->pc = T_LC_BEGIN;
  if (s == DGX_OK) s = advance(*t);
  if (s != DGX_OK) { t->err = s; t->pc = T_DONE; }
  b->members.push_back({r, t, 1});
  if (slot) *slot = (int32_t)b->members.size() - 1;
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_step(dgx_batch* b, int32_t* n_active) {
  if (!b) return DGX_ERR_ARG;
  std::vector<Task*> tasks;
  for (auto& m : b->members) if (m.r && !m.t->done()) tasks.push_back(m.t);
  if (!tasks.empty()) TRY(serve_round(b->ex, tasks, b->round_points.load()));
  int n = 0;
  for (auto& m : b->members) {
    if (m.r && m.active && m.t->done()) m.active = 0;
    n += m.active;
  }
  if (n_active) *n_active = n;
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_run(dgx_batch* b) {
  if (!b) return DGX_ERR_ARG;
  int32_t n = 1;
  while (n > 0) TRY(dgx_batch_step(b, &n));
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_host_times(const dgx_batch* b, double ms[4]) {
  if (!b || !ms) return DGX_ERR_ARG;
  for (int k = 0; k < 4; ++k) ms[k] = b->ex->host_ms[k];
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_member(const dgx_batch* b, int32_t slot, int32_t* done, int32_t* n_records,
                                       int32_t* status) {
  if (!b || slot < 0 || slot >= (int32_t)b->members.size()) return DGX_ERR_ARG;
  const auto& m = b->members[slot];
  if (!m.r) { set_err("dgx_batch_member: slot %d was removed", slot); return DGX_ERR_STATE; }
  if (done) *done = m.t->done() ? 1 : 0;
  if (n_records) *n_records = std::min(m.t->nrec, m.t->max_records);
  if (status) *status = m.t->err;
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_remove(dgx_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int32_t)b->members.size()) return DGX_ERR_ARG;
  auto& m = b->members[slot];
  if (!m.r) return DGX_OK;
  if (!m.t->done()) { set_err("dgx_batch_remove: member %d still running", slot); return DGX_ERR_STATE; }
  batch_detach(m);
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_stats(const dgx_batch* b, double ms[3], int64_t out[10]) {
  if (!b) return DGX_ERR_ARG;
  const Executor* e = b->ex;
  if (ms) for (int i = 0; i < 3; ++i) ms[i] = e->t_ms[i];
  if (out) {
    ConsCounters c{};
    CK(cudaMemcpy(&c, e->cnt, sizeof(c), cudaMemcpyDeviceToHost));
    out[0] = e->point_evals; out[1] = (int64_t)c.state_iters; out[2] = (int64_t)c.lp_iters; out[3] = e->rounds;
    out[4] = e->launches; out[5] = (int64_t)c.jac_iters; out[6] = e->bytes_h2d; out[7] = e->bytes_d2h;
    out[8] = (int64_t)c.fpi_iters; out[9] = e->graph_rounds;
  }
  return DGX_OK;
}

extern "C" void* dgx_batch_stream(const dgx_batch* b) { return b ? (void*)b->st : nullptr; }

extern "C" dgx_status dgx_batch_set_round_points(dgx_batch* b, int64_t points) {
  if (!b || points < 0) return DGX_ERR_ARG;
  b->round_points = points;
  return DGX_OK;
}

extern "C" dgx_status dgx_batch_tuning(const dgx_batch* b, int32_t out[4]) {
  if (!b || !out) return DGX_ERR_ARG;
  const Executor* e = b->ex;
  out[0] = e->tune_cons ? 0 : cons_variant_bs(e->cons_variant);
  out[1] = (int32_t)e->spec_tuned.size();
  out[2] = e->tune_cons ? 0 : cons_variant_minb(e->cons_variant);
  out[3] = e->tune_spec ? 1 : 0;
  return DGX_OK;
}
