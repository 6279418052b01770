// rve.cuh -- the RVE object shared by the solver host code (solver.cu) and the
// batched executor (batch.cu), and the host helpers both use.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/dgx.h"
#include "dgx_internal.cuh"
#include "spectral.cuh"

namespace dgx { struct Executor; }

struct dgx_rve {
  int cells[3];
  int64_t N;
  double geom[3], scaled[3], wgt;
  dgx_material mat;
  dgx_numerics num;
  dgx::MatParams mp;
  cudaStream_t st = nullptr;
  bool owns_stream = false;
  // device memory
  std::vector<void*> allocs;
  int64_t bytes = 0;
  dgx::PointState ps{};
  double *X = nullptr, *R = nullptr, *XM = nullptr, *FM = nullptr, *XA = nullptr, *FA = nullptr;
  double *F_last_inc = nullptr, *F_dot = nullptr;
  std::vector<double*> Xdot, Fdot;
  void* spec = nullptr;
  double *d_Pav = nullptr, *d_Cvol = nullptr, *d_Cmm = nullptr, *d_Cref = nullptr, *d_aim = nullptr, *d_rms = nullptr;
  double *d_Ppart = nullptr, *d_divpart = nullptr, *d_redpart = nullptr, *d_redout = nullptr, *d_beta = nullptr;
  dgx::TangentPartial* d_tpart = nullptr;
  int* d_ill = nullptr;
  dgx::ConsCounters* d_cnt = nullptr;
  double *d_xi_x = nullptr, *d_xi_y = nullptr, *d_xi_z = nullptr;
  double* d_fw[3] = {nullptr, nullptr, nullptr};   // FWBW derivative: per-axis (D, E) factors
  double* d_gtab = nullptr;        // K^-1 of C_ref per frequency (gamma_table), rebuilt with C_ref
  double* d_dPdF = nullptr;        // optional (81 planes) for the boundary call
  double* d_aos = nullptr;         // optional: 12 N doubles, device-side AoS staging of field reads
                                   // (allocated on the first read; not part of the creation footprint)
  double *d_un = nullptr, *d_up = nullptr, *d_Favg = nullptr;   // optional: coordinate update
  // optional: library-owned fields in the reference layout (dgx_fields), allocated on
  // the first dgx_fields call: F0 (committed F), F (written by the caller), P, dPdF
  double *fx_F0 = nullptr, *fx_F = nullptr, *fx_P = nullptr, *fx_dPdF = nullptr;
  int32_t* fx_ill = nullptr;
  dgx::BcBlock* d_bc = nullptr;    // stress BC of the current solve (device copy)
  int32_t* d_mat = nullptr;
  double* d_Rm = nullptr;
  int n_materials = 0;
  std::vector<int32_t> h_mat;
  std::vector<double> h_orient;
  dgx::AxisHost ax[3];
  dgx::SpecLaunch sl{};
  int nb_cons = 0, nb_tan = 0, nb_red = 0;
  int cons_block = 128;            // direct (unbatched) constitutive launches
  bool cons_block_forced = false;  // DGX_CONS_BLOCK set: the executor keeps it (no autotuning)
  // host solver state (MechBase / MechSolverBasic members)
  double F_aim[9], F_aim_last_inc[9], F_aim_dot[9], P_aim[9], P_av[9];
  double C_volAvg[81], C_minMaxAvg[81], C_volAvgLastInc[81], C_minMaxAvgLastInc[81], C_ref[81], S[81];
  int stress_mask[9];
  double rot_q[4];
  double delta_t = 0.0;
  double err_div = 0.0, err_BC = 0.0;
  int terminally_ill = 0, total_iter = 0;
  bool tangent_fresh = false, initialized = false;
  double tangent_dt = 0.0;
  // load-case loop state (DamaskGrid::loop_over_loadcase)
  int cut_back = 0, cut_back_level = 0;
  double t = 0.0, dt = 1.0, dt_prev = 0.0, t_0 = 0.0;
  int guess = 0, cur_step = -1;
  // counters
  int64_t n_eval = 0, n_tangent = 0, n_launch = 0;
  int64_t evals_in_step = 0;   // constitutive evaluations since the last forward (commit or cut-back)
  // CUDA-event timers on the RVE stream: [0] constitutive kernel, [1] spectral chain, [2] tangent
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double t_ms[3] = {0, 0, 0};
  int64_t t_n[3] = {0, 0, 0};
  bool timing = true;
  int64_t bytes_h2d = 0, bytes_d2h = 0;
  // batched execution: the RVE's own executor (a batch of one) and, while it is a
  // member of a dgx_batch, the stream it had before joining
  dgx::Executor* ex = nullptr;
  cudaStream_t home_st = nullptr;
  int in_batch = 0;
  bool dry = false;           // size-only pass of the buffer allocation (footprint)
};

namespace dgx {

void set_err(const char* fmt, ...);

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) { ::dgx::set_err("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); return DGX_ERR_CUDA; } \
  } while (0)
#define TRY(x) do { dgx_status s_ = (x); if (s_ != DGX_OK) return s_; } while (0)

constexpr int RB = 256;  // threads per reduction block
inline int nblk(int64_t n, int b = 256) { return (int)((n + b - 1) / b); }

// counted host<->device copies on the RVE stream (bytes per direction)
inline cudaError_t h2d(dgx_rve* r, void* dst, const void* src, size_t bytes) {
  r->bytes_h2d += (int64_t)bytes;
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, r->st);
}
inline cudaError_t d2h(dgx_rve* r, void* dst, const void* src, size_t bytes) {
  r->bytes_d2h += (int64_t)bytes;
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, r->st);
}

struct VecList { const double* v[32]; };

// solver.cu: host steps of MechSolverBasic / DamaskGrid shared by every execution mode
void rotate2(const double* q, const double* T, double* out, bool active);
void qu2om(const double* q, double* om);
void lsq_svd(int l, const double* H, double* b);
int converged(dgx_rve* r);
double forward_time(const dgx_loadstep* ls, int inc, int sub_step_factor, int cut_back_level);
dgx_status commit(dgx_rve* r);
dgx_status ensure_tangent(dgx_rve* r);
// after the constitutive pass of a residual evaluation (P_av, ill on the host)
dgx_status post_constitutive(dgx_rve* r, int ill, bool want_tangent);
// MechSolverBasic::calculate_solution before and after SNESSolve; the prologue also
// uploads the solve's stress BC (BcBlock) to the device
dgx_status solve_prologue(dgx_rve* r);
void solve_epilogue(dgx_rve* r, int reason, int32_t* conv, int32_t* iterations, int32_t* ill_out);
// volume average of F (the record of an increment)
dgx_status field_average(dgx_rve* r, const double* X, double out[9]);
GammaArgs gamma_args(dgx_rve* r, bool gamma, bool div);
// upload r->C_ref (MechBase::update_gamma, mech_base.cpp:156-157) and rebuild the
// per-frequency K^-1 table of the Gamma operator from it, on the RVE's stream
dgx_status set_reference_stiffness(dgx_rve* r);
void launch_axpy(double* z, const double* x, double a, const double* y, int64_t n, cudaStream_t st);
void launch_combine(double* XA, const double* XM, const VecList& Xd, int l, double c0, const double* beta, int64_t n,
                    int nb, cudaStream_t st);


// batch.cu: the batched executor and the solver state machine
dgx_status executor_create(int cap, cudaStream_t st, ConsCounters* cnt, int cons_block, Executor** out);
void executor_destroy(Executor* e);
// adds the executor's timers (ms, launches per timer), launches and copied bytes
void executor_stats(const Executor* e, double ms[3], int64_t n[3], int64_t* launches, int64_t* h2d_b, int64_t* d2h_b,
                    int64_t* graph_rounds);
// a solve (mode 0), one increment (mode 1: steps = that step, n_or_index = its index)
// or a load case (mode 2: n_or_index = number of steps) of one RVE, as a batch of one
// result / restart output of a load case (increment 0 at the start, then every
// f_out-th increment of a step; a restart file every restart_every-th increment)
struct Output {
  dgx_result* result;
  const char* restart_path;
  int restart_every;
};
dgx_status run_single(dgx_rve* r, int mode, const dgx_loadstep* steps, int n_or_index, int inc,
                      dgx_inc_record* records, int max_records, int32_t* n_records, int32_t* conv, int32_t* iterations,
                      int32_t* ill, const Output* out = nullptr);
// the unguarded bodies of dgx_update_coords / dgx_result_write_increment / dgx_restart_write
dgx_status update_coords_impl(dgx_rve* r, double* u_n, double* u_p);
dgx_status result_write_impl(dgx_result* res, dgx_rve* r, int32_t inc, double t);
dgx_status restart_write_impl(dgx_rve* r, const char* path);

}  // namespace dgx
