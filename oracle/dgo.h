/*
 * dgo.h -- CPU oracle for the DAMASK_grid spectral-basic + phenopowerlaw path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's algorithm, written to check the CUDA product path and to serve
 * as the timed CPU baseline.  Nothing in the product library links it; only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Storage conventions (same as the reference, Fortran column-major):
 *   3x3     A[i + 3*j]                      = A(i,j)
 *   3x3x3x3 T[i + 3*j + 9*k + 27*l]         = T(i,j,k,l)
 *   field   F[(i + 3*j) + 9*cell],  cell = a + N0*(b + N1*c)  (x fastest)
 *   spectrum  X[(l + 3*m) + 9*(i + N0r*(k + N2*j))]  = X(l,m,i,k,j)
 *             (transposed-out layout of src/grid/fft.cpp:100-125, N0r = N0/2+1)
 */
#ifndef DGO_H
#define DGO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- material */
typedef struct dgo_material {
  /* Hooke (phase_mechanical_elastic.f90:74-104), cubic */
  double C11, C12, C44;
  /* phenopowerlaw slip (phase_mechanical_plastic_phenopowerlaw.f90:75-290) */
  double xi_0, xi_inf, h_0, n, dot_gamma_0, a, c_1, c_2;
  double h_sl_sl[7];            /* interaction values by type (crystal.f90:613-646) */
  double atol_xi, atol_gamma;
  /* crystallite numerics (phase_mechanical.f90:280-290) */
  double r_cutback_min, r_cutback, r_increase, eps_rel_state;
  int    N_iter_state_max, N_iter_Lp_max;
  double r_linesearch_Lp, eps_rel_Lp, eps_abs_Lp;
  int    f_update_jacobi_Lp;
} dgo_material;

void dgo_material_default(dgo_material* m);

/* derived constant tables (Schmid matrices, interaction matrix, stiffness) */
typedef struct dgo_consts {
  double P_sl[12][9];
  double h[12][12];             /* h[reacting][acting] */
  double C66[36];               /* column-major 6x6 */
  double C[81];                 /* 3x3x3x3 stiffness */
} dgo_consts;

void dgo_consts_build(const dgo_material* m, dgo_consts* c);

/* ---------------------------------------------------------------- points */
typedef struct dgo_points {
  int64_t n;
  double *F, *F0, *Fp, *Fp0, *Fi, *Fi0, *Fe, *Lp, *Lp0, *Li, *Li0, *S, *S0, *P;
  double *xi, *xi0, *gamma, *gamma0;          /* 12 per point */
  double *dPdF;                               /* 81 per point */
  int32_t *status;                            /* 0 ok, 1 broken */
} dgo_points;

int  dgo_points_alloc(dgo_points* p, int64_t n);
void dgo_points_free(dgo_points* p);
/* orientations: 4 per point (w,x,y,z) */
void dgo_points_init(const dgo_material* m, dgo_points* p, const double* q);
/* materialpoint_forward: commit state (phase_mechanical.f90:992-1007) */
void dgo_points_commit(dgo_points* p);

/* per-cell loop of f_homogenization_mechanical_response(+2):
 * F (9n) in; writes P (9n) and, if want_dPdF, dPdF (81n).  Returns terminally_ill. */
int dgo_constitutive_response(const dgo_material* m, const dgo_consts* c, dgo_points* p,
                              const double* F, double dt, int want_dPdF, int nthreads);

/* Spectral::constitutive_response reductions (spectral.cpp:160-217) */
void dgo_averages(int64_t n, const double* P, const double* dPdF,
                  double P_av[9], double C_volAvg[81], double C_minMaxAvg[81]);

/* ---------------------------------------------------------------- math helpers */
void dgo_qu2om(const double q[4], double om[9]);
int  dgo_invert33(const double A[9], double inv[9], double* det);
int  dgo_invert(int n, const double* A, double* inv);            /* LU, column-major */
void dgo_rotate2(const double q[4], const double T[9], double out[9], int active);
void dgo_rotate4(const double q[4], const double T[81], double out[81], int active);
void dgo_3333to99(const double* m3333, double* m99);
void dgo_99to3333(const double* m99, double* m3333);

/* ---------------------------------------------------------------- FFT */
/* complex spectra are stored as interleaved (re, im) doubles */
void dgo_twiddle(long j, long n, double* c, double* s);
void dgo_fft_r2c(const int cells[3], int ncomp, const double* field, double* spec);
void dgo_fft_c2r(const int cells[3], int ncomp, const double* spec, double* field);

/* ---------------------------------------------------------------- spectral */
enum { DGO_DERIV_CONTINUOUS = 0, DGO_DERIV_CENTRAL = 1, DGO_DERIV_FWBW = 2 };
enum { DGO_DIVCORR_NONE = 0, DGO_DIVCORR_SIZE = 1, DGO_DIVCORR_SIZE_GRID = 2 };

/* xi1st, xi2nd: complex (3, N0r, N2, N1) */
void dgo_xi(const int cells[3], const double geom[3], int derivative, double* xi1st, double* xi2nd);
/* cell-centre (u_p, 3 per cell) and nodal (u_n, 3 per node) displacements of F */
void dgo_update_coords(const int cells[3], const double geom[3], int derivative, const double* F,
                       double* u_n, double* u_p);
/* orientation output: rotational part of F (closed form), quaternion of R^T */
void dgo_rotational_part(const double F[9], double R[9]);
void dgo_om2qu(const double om[9], double qu[4]);
void dgo_orientation_output(const double Fe[9], double qu[4]);
void dgo_scaled_geom(const int cells[3], const double geom[3], int divcorr, double out[3]);
double dgo_divergence_rms_spec(const int cells[3], const double geom[3], const double scaled[3],
                               const double* xi1st, const double* spec);
double dgo_divergence_rms(const int cells[3], const double geom[3], const double scaled[3],
                          const double* xi1st, const double* P);
/* in place: field <- Gamma(C_ref) * field, zero frequency <- aim */
void dgo_gamma_convolution(const int cells[3], const double* xi1st, const double C_ref[81],
                           const double aim[9], double* field);
void dgo_forward_field(int64_t n, double dt, const double* last, const double* rate,
                       const double* aim /* may be NULL */, double* out);
void dgo_calculate_rate(int64_t n, int heterogeneous, const double* field0, const double* field,
                        double dt, const double avRate[9], double* rate);
/* mask_stress: column-major, 1 = not prescribed ('x') */
int  dgo_masked_compliance(const double C[81], const double q[4], const int mask_stress[9],
                           double S[81]);
void dgo_mul3333xx33(const double A[81], const double B[9], double out[9]);

/* ---------------------------------------------------------------- solver */
enum { DGO_BC_F = 0, DGO_BC_DOT_F = 1, DGO_BC_L = 2 };
enum { DGO_BC_P = 0, DGO_BC_DOT_P = 1 };
enum { DGO_SOLVER_NGMRES = 0, DGO_SOLVER_FIXED_POINT = 1 };

typedef struct dgo_numerics {
  int    itmin, itmax, update_gamma;
  double eps_abs_div, eps_rel_div, eps_abs_P, eps_rel_P;
  int    divergence_correction, derivative;
  int    stag_iter_max, max_cut_back;
  int    solver, ngmres_m, snes_max_it;
} dgo_numerics;

void dgo_numerics_default(dgo_numerics* n);

typedef struct dgo_loadstep {
  int    def_type;   double def_values[9];    int def_mask[9];
  int    stress_type; double stress_values[9]; int stress_mask[9];
  double rot_q[4];
  double t;  int N;  double r;  int estimate_rate;  int f_out;
} dgo_loadstep;

typedef struct dgo_solver dgo_solver;

/* material_at: n ints (0-based material index); orientations: 4 per material */
dgo_solver* dgo_solver_create(const int cells[3], const double geom[3], const int32_t* material_at,
                              int n_materials, const double* orientations,
                              const dgo_material* mat, const dgo_numerics* num, int nthreads);
void dgo_solver_free(dgo_solver* s);

/* per-increment record filled by dgo_solver_run */
typedef struct dgo_inc_record {
  double t, dt;
  double P_av[9], F_aim[9], F_av[9];
  int    iterations, evaluations, converged, cutbacks;
  double err_div, err_BC;
  double seconds;               /* wall time of the increment */
} dgo_inc_record;

/* runs all load steps; returns number of increments recorded (<0 on error) */
int dgo_solver_run(dgo_solver* s, int nsteps, const dgo_loadstep* steps,
                   dgo_inc_record* records, int max_records);
/* run a single increment inside a previously started load case (bench sample) */
int64_t dgo_solver_total_evaluations(const dgo_solver* s);

/* field access (copies out, reference layout) */
void dgo_solver_get(const dgo_solver* s, const char* name, double* out);
const dgo_points* dgo_solver_points(const dgo_solver* s);

/* lower-level steps for known-answer tests */
void dgo_solver_init_state(dgo_solver* s);            /* MechSolverBasic::init */
int  dgo_solver_forward(dgo_solver* s, int cutback, int guess, double dt, double dt_old,
                        double t_remaining, const dgo_loadstep* ls);
int  dgo_solver_solve(dgo_solver* s, int* iterations, int* terminally_ill);

/* form_residual BC part (mech_solver_basic.cpp:321-334) exposed for the
 * TestFormResidual known answer: updates F_aim in place, returns err_BC and the
 * rotated delta_F_aim */
double dgo_form_residual_bc(const double S[81], const double P_av[9], const double P_aim[9],
                            const int stress_mask[9], const double q[4], double F_aim[9],
                            double rotated[9]);

/* op counters: constitutive kernel work (state iterations, Lp iterations) */
void dgo_counters(int64_t out[4]);
void dgo_counters_reset(void);

#ifdef __cplusplus
}
#endif
#endif
