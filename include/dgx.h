/*
 * dgx.h -- C ABI of the GB300 (sm_103a) DAMASK_grid spectral-basic solver.
 *
 * Plain C types only (pointers, sizes, int32/double); every call returns a
 * dgx_status.  All tensors at this boundary use the reference's layout:
 * column-major 3x3 (component i + 3*j), fields (3,3,N) with the cell index
 * cell = x + N0*(y + N1*z) slowest, i.e. value(i,j,cell) = a[(i + 3*j) + 9*cell],
 * and 3x3x3x3 tangents a[i + 3j + 9k + 27l] per cell.  Host pointers unless the
 * function name ends in _device.
 *
 * Each entry point names the reference interface it replaces (reference paths).
 */
#ifndef DGX_H
#define DGX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t dgx_status;
enum {
  DGX_OK = 0,
  DGX_ERR_ARG = -1,          /* invalid argument / size */
  DGX_ERR_CUDA = -2,         /* CUDA runtime error (message: dgx_last_error) */
  DGX_ERR_NOMEM = -3,        /* device allocation failed */
  DGX_ERR_UNSUPPORTED = -4,  /* option not implemented on this path */
  DGX_ERR_NOT_CONVERGED = -5,/* load case: no solution after max cut-backs */
  DGX_ERR_STATE = -6         /* call out of order (e.g. solve before init) */
};

/* phenopowerlaw cF phase + crystallite numerics.
 * Replaces material.yaml/numerics parsing of phase_mechanical_plastic_phenopowerlaw.f90:75-290,
 * phase_mechanical_elastic.f90:74-104 and phase_mechanical.f90:280-290. */
typedef struct dgx_material {
  double C11, C12, C44;
  double xi_0, xi_inf, h_0, n, dot_gamma_0, a, c_1, c_2;
  double h_sl_sl[7];
  double atol_xi, atol_gamma;
  double r_cutback_min, r_cutback, r_increase, eps_rel_state;
  int32_t N_iter_state_max, N_iter_Lp_max;
  double r_linesearch_Lp, eps_rel_Lp, eps_abs_Lp;
  int32_t f_update_jacobi_Lp;
} dgx_material;

/* grid solver numerics.  Replaces Config::Numerics (src/grid/config.h:50-78). */
typedef struct dgx_numerics {
  int32_t itmin, itmax, update_gamma;
  double eps_abs_div, eps_rel_div, eps_abs_P, eps_rel_P;
  int32_t divergence_correction;  /* 0 none, 1 size, 2 size+grid */
  int32_t derivative;             /* 0 continuous, 1 central_difference, 2 FWBW_difference */
  int32_t stag_iter_max, max_cut_back;
  int32_t solver;                 /* 0 NGMRES (PETSc SNESNGMRES defaults), 1 fixed point */
  int32_t ngmres_m, snes_max_it;
  int32_t precision;              /* 0 FP64 everywhere, 1 mixed: FP32 FFT/Gamma, FP32 Lp Jacobian,
                                     rates and state test around the FP64 Lp Newton */
  int32_t lazy_tangent;           /* 1: tangent only where C_volAvg/C_minMaxAvg are consumed */
} dgx_numerics;

void dgx_material_default(dgx_material* m);
void dgx_numerics_default(dgx_numerics* n);

/* One load step (Config::LoadStep, src/grid/config.h:86-97; parse_load config.cpp:247-358).
 * Masks are column-major, 1 where the load yaml has 'x'. */
typedef struct dgx_loadstep {
  int32_t def_type;   double def_values[9];    int32_t def_mask[9];    /* 0 F, 1 dot_F, 2 L */
  int32_t stress_type; double stress_values[9]; int32_t stress_mask[9]; /* 0 P, 1 dot_P */
  double rot_q[4];                                                     /* w, x, y, z */
  double t;  int32_t N;  double r;  int32_t estimate_rate;  int32_t f_out;
} dgx_loadstep;

typedef struct dgx_inc_record {
  double t, dt;
  double P_av[9], F_aim[9], F_av[9];
  int32_t iterations, evaluations, converged, cutbacks;
  double err_div, err_BC;
  double seconds;                 /* wall time of the increment */
} dgx_inc_record;

typedef struct dgx_rve dgx_rve;

/* Create an RVE on the current CUDA device: grid + material map + orientations.
 * Replaces f_materialpoint_initBase/initDamask (src/grid/main.cpp:9-13,
 * materialpoint.f90:68-156) and DiscretizationGrid::init (discretization_grid.cpp:8-84).
 * material_at: N0*N1*N2 0-based material indices; orientations: 4 doubles
 * (w,x,y,z) per material. */
dgx_status dgx_rve_create(const int32_t cells[3], const double size[3], const int32_t* material_at,
                          int32_t n_materials, const double* orientations, const dgx_material* mat,
                          const dgx_numerics* num, dgx_rve** out);
void dgx_rve_destroy(dgx_rve* rve);
const char* dgx_last_error(void);
/* Device bytes dgx_rve_create would allocate for this grid and numerics (admission
 * control).  No reference counterpart. */
dgx_status dgx_rve_footprint(const int32_t cells[3], const dgx_numerics* num, int32_t n_materials, int64_t* bytes);
int64_t dgx_rve_points(const dgx_rve* rve);
/* device bytes held by the RVE (fields, state, NGMRES history, scratch) */
int64_t dgx_rve_device_bytes(const dgx_rve* rve);

/* Per-cell constitutive response for cells [first, first+count) of F, with P and
 * (optionally) dPdF out; terminally_ill set if any cell failed.
 * Replaces f_homogenization_mechanical_response + f_homogenization_mechanical_response2
 * (src/grid/spectral.h:20-22; homogenization.f90:219-324).  The current
 * implementation evaluates whole RVEs: first must be 0 and count N. */
dgx_status dgx_constitutive_response(dgx_rve* rve, const double* F, double dt, int32_t first, int32_t count,
                                     double* P, double* dPdF, int32_t* terminally_ill);
/* Library-owned device fields in the reference layout, for a grid solver that keeps F,
 * P and dPdF on the device.  Replaces f_homogenization_fetch_tensor_pointers
 * (src/grid/spectral.h:17-19; homogenization.f90:491-510): F0 the committed deformation
 * gradient (3,3,N), refreshed by every commit; F the deformation gradient (3,3,N) the
 * caller writes before dgx_constitutive_response_fields; P (3,3,N) and dPdF
 * (3,3,3,3,N, a[i+3j+9k+27l + 81*cell]; null unless requested) written by it;
 * terminally_ill a device int32 (1: a cell failed), the reference's Fortran logical;
 * stream the cudaStream_t the library works on (order your kernels on it, or
 * synchronise).  All pointers are device pointers owned by the RVE (freed with it);
 * the first call allocates them (F0 and F start as the committed F). */
typedef struct dgx_field_ptrs {
  int64_t n;
  double* F0;
  double* F;
  double* P;
  double* dPdF;
  int32_t* terminally_ill;
  void* stream;
} dgx_field_ptrs;
dgx_status dgx_fields(dgx_rve* rve, int32_t with_dPdF, dgx_field_ptrs* out);
/* Constitutive response of the exported field F in place, no host copies of fields:
 * P (and dPdF if want_dPdF) written to the exported buffers, terminally_ill set; P_av
 * and the tangent averages available through dgx_averages.  Replaces
 * f_homogenization_mechanical_response + _response2 as Spectral::constitutive_response
 * calls them (src/grid/spectral.cpp:132-160).  Whole RVE only (first 0, count N);
 * returns after the results are on the device. */
dgx_status dgx_constitutive_response_fields(dgx_rve* rve, double dt, int32_t first, int32_t count, int32_t want_dPdF);
/* Volume averages of the last response: replaces the reductions of
 * Spectral::constitutive_response (src/grid/spectral.cpp:160-217). */
dgx_status dgx_averages(dgx_rve* rve, double P_av[9], double C_volAvg[81], double C_minMaxAvg[81]);
/* Commit the increment (state0 <- state).  Replaces f_materialpoint_forward
 * (src/grid/damask_grid.h:17; materialpoint.f90:208-215). */
dgx_status dgx_commit_increment(dgx_rve* rve);

/* Divergence RMS of a stress field.  Replaces MechBase::calculate_divergence_rms
 * (src/grid/mech_base.cpp:302-398). */
dgx_status dgx_divergence_rms(dgx_rve* rve, const double* P, double* rms);
/* In place Gamma convolution with zero frequency <- aim, using C_ref.
 * Replaces MechBase::gamma_convolution (src/grid/mech_base.cpp:400-477). */
dgx_status dgx_gamma_convolution(dgx_rve* rve, double* field, const double aim[9]);
/* Set the reference stiffness C_ref = C / wgt (MechBase::update_gamma, mech_base.cpp:156-157). */
dgx_status dgx_update_gamma(dgx_rve* rve, const double C[81]);
/* Forward FFT of a (3,3,N) field into the reference's transposed-out half spectrum
 * (3,3,N0/2+1,N2,N1) as interleaved (re,im) (FFT<5>::forward, src/grid/fft.h:37-47). */
dgx_status dgx_fft_forward(dgx_rve* rve, const double* field, double* spectrum);

/* Divergence RMS of a device-resident stress field (3,3,N) without any device
 * allocation.  No counterpart in the reference: it is for callers that cannot call
 * cudaMalloc (all device memory owned by their own pool or budget, or no
 * allocation allowed inside their time-critical loop); they pass input and output
 * buffers they already own.  Scratch is one file-scope device array of 10 MiB,
 * held by every GPU that loads the library until exit; at most 32768 cells
 * (larger grids return DGX_ERR_ARG).  All calls share that array and leave their
 * contents in it, so calls that overlap on the GPU race and must be serialised.
 * The first call on a device looks up the array's address (make it before any
 * stream capture).  divergence_correction 0 none, 1 size, 2 size+grid (else
 * DGX_ERR_ARG); derivative 0 continuous, 1 central difference.  A CUDA error left
 * pending by earlier work is reported (DGX_ERR_CUDA) and not cleared.
 * P_device: device (3,3,N) reference layout; rms_device: one device double;
 * stream: cudaStream_t (0 = default stream); the result is written asynchronously
 * on the stream (the small FFT tables are staged from host memory first). */
dgx_status dgx_divergence_rms_static(const int32_t cells[3], const double size[3], int32_t divergence_correction,
                                     int32_t derivative, const double* P_device, double* rms_device, void* stream);

/* ---- Geometry input: VTK ImageData (.vti) content held in memory (host only).
 * Replaces f_VTI_readCellsSizeOrigin (src/grid/discretization_grid.h:19-20): cells from
 * WholeExtent, size = cells x Spacing, origin from Origin. */
dgx_status dgx_vti_read_cells_size_origin(const char* content, int64_t length, int32_t cells[3], double size[3],
                                          double origin[3]);
/* Replaces f_VTI_readDataset_int (src/grid/discretization_grid.h:21-22): the integer
 * cell-data array `label` (DAMASK: "material"), x fastest, into dataset.  On entry
 * *dataset_size is the capacity of dataset, on return the number of values (N0*N1*N2);
 * too small a capacity returns DGX_ERR_ARG with *dataset_size set to the count needed.
 * ascii or inline base64 binary, raw or vtkZLibDataCompressor, UInt32/UInt64 headers,
 * any integer element type within int32 range. */
dgx_status dgx_vti_read_dataset_int(const char* content, int64_t length, const char* label, int32_t label_length,
                                    int32_t* dataset, int64_t* dataset_size);

/* Solver (MechSolverBasic + DamaskGrid, src/grid/mech_solver_basic.cpp, damask_grid.cpp) */
dgx_status dgx_solver_init(dgx_rve* rve);                                   /* MechSolverBasic::init :19-108 */
dgx_status dgx_solver_forward(dgx_rve* rve, int32_t cutback, int32_t guess, double dt, double dt_old,
                              double t_remaining, const dgx_loadstep* ls);  /* forward :163-220 */
dgx_status dgx_solver_solve(dgx_rve* rve, int32_t* converged, int32_t* iterations,
                            int32_t* terminally_ill);                      /* calculate_solution :110-161 */
/* DamaskGrid::loop_over_loadcase (damask_grid.cpp:82-196): runs all steps from
 * solver init; records[k] per increment (up to max_records). */
dgx_status dgx_run_loadcase(dgx_rve* rve, int32_t nsteps, const dgx_loadstep* steps,
                            dgx_inc_record* records, int32_t max_records, int32_t* n_records);
/* dgx_run_loadcase with output: result (may be null) receives increment 0 and every
 * f_out-th increment of each step (numbered by the increments completed so far); a
 * restart file is written to restart_path every restart_every increments (0: never). */
dgx_status dgx_run_loadcase_output(dgx_rve* rve, int32_t nsteps, const dgx_loadstep* steps,
                                   dgx_inc_record* records, int32_t max_records, int32_t* n_records,
                                   struct dgx_result* result, const char* restart_path, int32_t restart_every);
/* incremental variant: dgx_solver_init once, then one increment per call
 * (state carried on the device between calls) */
dgx_status dgx_run_increment(dgx_rve* rve, const dgx_loadstep* step, int32_t step_index, int32_t inc,
                             dgx_inc_record* record);

/* MechSolverBasic::update_coords (mech_solver_basic.cpp:222-238, mech_base.cpp:45-154):
 * displacements of the deformed grid from the current solution F, as written to the
 * results: u_n (3 per node, (N0+1)(N1+1)(N2+1) nodes) and u_p (3 per cell), x fastest;
 * either may be null. */
dgx_status dgx_update_coords(dgx_rve* rve, double* u_n, double* u_p);

/* ---- DADF5 results (f_materialpoint_result, damask_grid.h:18; result.f90:80-160).
 * open: file with root / geometry / cell_to / setup groups for the RVE's grid;
 * write_increment: group increment_<inc> (attribute t/s) with geometry/{u_n,u_p} and
 * phase/<phase>/mechanical/{F,F_e,F_p,L_p,O,P,xi_sl}; close: writes the metadata (the
 * file is valid after close).  phase / homogenization default to "phase" / "SX". */
typedef struct dgx_result dgx_result;
dgx_status dgx_result_open(const char* path, const dgx_rve* rve, const char* phase, const char* homogenization,
                           dgx_result** out);
/* an input file stored under /setup/<name> */
dgx_status dgx_result_add_setup(dgx_result* res, const char* name, const char* content, int64_t length);
dgx_status dgx_result_write_increment(dgx_result* res, dgx_rve* rve, int32_t inc, double t);
dgx_status dgx_result_close(dgx_result* res);
/* Restart (materialpoint.f90:163-202, phase_mechanical.f90:1264-1298): the RVE's
 * complete state after an increment; read into an RVE created with the same inputs,
 * the load case continues bitwise as if uninterrupted. */
dgx_status dgx_restart_write(dgx_rve* rve, const char* path);
dgx_status dgx_restart_read(dgx_rve* rve, const char* path);

/* Copy a per-point field out in the reference layout.  name: "F", "P", "Fp", "Lp",
 * "Fe", "S" (9 per cell), "xi", "gamma" (12 per cell), "dPdF" (81 per cell, last
 * response with dPdF), or averages "P_av", "F_aim", "C_volAvg", "C_minMaxAvg",
 * "C_ref", "S_compliance". */
dgx_status dgx_get(dgx_rve* rve, const char* name, double* out);

/* Work counters since creation: [0] residual evaluations, [1] constitutive state
 * integrations (sub-steps), [2] Lp Newton iterations, [3] tangent evaluations,
 * [4] kernel launches issued by the library, [5] Lp Jacobian factorisations,
 * [6] host-to-device bytes, [7] device-to-host bytes copied by the library,
 * [8] fixed-point state iterations, [9] rounds issued as CUDA graph replays. */
dgx_status dgx_counters(const dgx_rve* rve, int64_t out[10]);
/* FP64 flops per counted unit of the constitutive kernel (FMA = 2): [0] Lp iteration,
 * [1] Jacobian, [2] state integration, [3] fixed-point iteration.  No reference
 * counterpart; the numerator of the kernel's roofline. */
void dgx_flop_model(double out[4]);
/* The same for the mixed-precision constitutive form (numerics precision 1), split
 * into the FP64 flops (fp64) and the FP32 flops (fp32) per counted unit.  No reference
 * counterpart. */
void dgx_flop_model_mixed(double fp64[4], double fp32[4]);
/* CUDA-event time (ms, accumulated) and launch counts of [0] the constitutive
 * kernel, [1] the spectral chain (FFT + Gamma + div-RMS), [2] the tangent kernel,
 * measured on the RVE's stream. */
dgx_status dgx_timers(const dgx_rve* rve, double ms[3], int64_t launches[3]);
/* The CUDA stream (cudaStream_t) all work of the RVE is queued on. */
void* dgx_rve_stream(const dgx_rve* rve);
/* ---- Batched execution (no counterpart in the reference, which solves one RVE per
 * process).  A batch advances many RVEs of uneven size together on one stream: each
 * round serves the pending residual evaluations of all members with one persistent
 * constitutive launch over all their points and one launch per FFT pass for every
 * group of equal grids, and the pending fused reductions with one launch.  A member
 * computes exactly what dgx_run_loadcase computes for it alone (same kernels, same
 * reduction order), whatever else is in the batch.  Members may be added between
 * rounds (continuous batching); an RVE in a batch may not be driven by the
 * single-RVE calls until it is removed. */
typedef struct dgx_batch dgx_batch;
/* capacity: most members at once; cons_block: points per constitutive block (32,
 * 64, 128 or 256), or 0 to let the batch's autotuner pick it from the first rounds (it
 * also picks each grid's FFT tile shape; DGX_AUTOTUNE=0 turns both off).  Results do
 * not depend on these choices. */
dgx_status dgx_batch_create(int32_t capacity, int32_t cons_block, dgx_batch** out);
void dgx_batch_destroy(dgx_batch* batch);
/* Add an RVE that runs the load case steps[0..nsteps) from solver init (as
 * dgx_run_loadcase); records[k] is filled per increment (up to max_records).  steps
 * and records must stay valid until the member is done.  *slot identifies it. */
dgx_status dgx_batch_add(dgx_batch* batch, dgx_rve* rve, int32_t nsteps, const dgx_loadstep* steps,
                         dgx_inc_record* records, int32_t max_records, int32_t* slot);
/* One round; *n_active = members not yet done. */
dgx_status dgx_batch_step(dgx_batch* batch, int32_t* n_active);
/* Rounds until every member is done. */
dgx_status dgx_batch_run(dgx_batch* batch);
/* done: 1 when the member finished (status: its dgx_status), n_records written. */
dgx_status dgx_batch_member(const dgx_batch* batch, int32_t slot, int32_t* done, int32_t* n_records,
                            int32_t* status);
/* Detach a finished member: the RVE returns to its own stream and the single-RVE calls. */
dgx_status dgx_batch_remove(dgx_batch* batch, int32_t slot);
/* ms: CUDA-event time of [0] constitutive launches, [1] spectral chains, [2] the rounds'
 * device work (each round from its first copy to its last; wall time beyond it is host
 * work between rounds);
 * out: [0] point evaluations, [1] state integrations, [2] Lp iterations, [3] rounds,
 * [4] launches of the batched kernels, [5] Jacobian factorisations, [6] h2d bytes,
 * [7] d2h bytes of the executor, [8] fixed-point iterations, [9] rounds issued as a
 * CUDA graph replay (a round's launch sequence is captured once its launch parameters
 * repeat; DGX_GRAPHS=0 in the environment at creation launches every round directly). */
dgx_status dgx_batch_stats(const dgx_batch* batch, double ms[3], int64_t out[10]);
void* dgx_batch_stream(const dgx_batch* batch);
/* Host wall time of the batch's rounds (ms, accumulated): [0] planning and issuing,
 * [1] waiting for the device, [2] reading results after the wait, [3] advancing the
 * members' solver logic on the host.  No reference counterpart. */
dgx_status dgx_batch_host_times(const dgx_batch* batch, double ms[4]);
/* Cap the residual evaluations served per round at `points` cells (0: no cap).  Above
 * the cap, members with the least remaining work (cells x increments left) go first;
 * a member passed over gains priority every round it waits.  Lowers the latency of
 * small members without starving large ones; results are unchanged. */
dgx_status dgx_batch_set_round_points(dgx_batch* batch, int64_t points);
/* autotuner state: [0] constitutive points per block (0 while still tuning), [1] grids
 * with a chosen FFT tile shape, [2] blocks per SM the chosen constitutive variant's
 * register allocation targets (0 while still tuning), [3] tile tuning on */
dgx_status dgx_batch_tuning(const dgx_batch* batch, int32_t out[4]);

/* ---- Serving (no counterpart in the reference).  A server owns one worker thread, the
 * device and a dgx_batch.  Requests from any thread are queued; in arrival order a
 * request is admitted when a batch slot is free and its device footprint
 * (dgx_rve_footprint) fits the HBM budget beside the resident requests; its RVE is
 * created and joins the batch between two rounds, runs its load case with its state
 * resident on the device, and leaves (memory freed) when done.  Results equal those
 * of the same solve run alone. */
typedef struct dgx_server dgx_server;
typedef struct {
  int32_t cells[3];
  double size[3];
  const int32_t* material_at;      /* N0*N1*N2 0-based material indices (copied at submit) */
  int32_t n_materials;
  const double* orientations;      /* 4 per material, w,x,y,z (copied) */
  dgx_material material;
  dgx_numerics numerics;
  int32_t nsteps;
  const dgx_loadstep* steps;       /* copied */
} dgx_request;
typedef struct {
  int32_t state;                   /* 0 queued, 1 running, 2 done, 3 failed */
  int32_t status;                  /* dgx_status of the solve */
  int32_t n_records;               /* increments recorded */
  double t_submit, t_admit, t_done;   /* seconds since the server started */
  int64_t device_bytes, points;
  char error[160];
} dgx_request_status;
typedef struct {
  int32_t queued, running;
  int64_t completed, failed, rounds, budget_bytes, used_bytes;
  double now;                      /* seconds since the server started */
  int32_t status;                  /* DGX_OK unless a device error stopped the service */
} dgx_server_info;
/* hbm_budget_bytes <= 0: 85 % of the free device memory at creation */
dgx_status dgx_server_create(int64_t hbm_budget_bytes, int32_t max_active, int32_t cons_block, dgx_server** out);
/* stops the worker; queued and running requests end as failed ("server stopped") */
void dgx_server_destroy(dgx_server* server);
dgx_status dgx_server_submit(dgx_server* server, const dgx_request* request, int64_t* id);
/* status (waiting up to wait_s seconds for completion); records copied once done */
dgx_status dgx_server_poll(dgx_server* server, int64_t id, double wait_s, dgx_request_status* status,
                           dgx_inc_record* records, int32_t max_records);
/* forget a finished request */
dgx_status dgx_server_release(dgx_server* server, int64_t id);
dgx_status dgx_server_stats(dgx_server* server, dgx_server_info* info);
/* the server batch's per-round point cap (dgx_batch_set_round_points); default 1 M cells */
dgx_status dgx_server_set_round_points(dgx_server* server, int64_t points);

/* FP64 FMA throughput of the current device (TFLOP/s, best of 5), the
 * denominator of the constitutive kernel's roofline.  No reference counterpart. */
dgx_status dgx_measure_fp64_peak(double* tflops, double* ms);

/* The constitutive kernel's own device math on n host values (validation against the
 * CUDA library functions; no reference counterpart): fn 0 the Newton-Raphson
 * reciprocal 1/x, fn 1 x^(9/4) (slip-resistance saturation, a = 2.25), fn 2 x^19
 * (the power law's x^(n-1), n = 20), fn 3 the mixed form's FP64 -> FP32 -> FP64 round
 * trip on the integer pipe (FP32 rounded toward zero, subnormals flushed), fn 4 the
 * mixed form's FP32 tolerance scale of a state value (the high word's 20 mantissa bits,
 * below the FP32 normal range signed zero, above it or NaN signed infinity). */
dgx_status dgx_device_math(int32_t fn, int64_t n, const double* x, double* out);

#ifdef __cplusplus
}
#endif
#endif
