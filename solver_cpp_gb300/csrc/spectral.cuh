// spectral.cuh -- host interface of the spectral kernels (spectral.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

namespace dgx {

// FFT plan for one axis length (device constant data passed by value)
struct AxisPlan {
  int n, nstages;
  int radix[16];
  const double2* tw;      // exp(-2 pi i j / n), j < n  (FP64 table)
  const float2* twf;      // same in FP32
};

struct AxisHost {
  AxisPlan plan;
  double2* d_tw = nullptr;
  float2* d_twf = nullptr;
};

struct SpecGeom {
  int N0, N1, N2, N0r;
  long long N, Nh;        // real points, half-spectrum points (per component)
};

// launch configuration shared by the spectral kernels
struct SpecLaunch {
  SpecGeom g;
  int LX, TIy, TIz;       // x lines per block; x-frequencies per y / z block
  size_t smx, smy, smz;
  int nbx, nby, nbz;
  int ndiv;               // divergence partials: one per (x-frequency, y) line = N0r * N1
};

struct GammaArgs {
  const double* xi_x;     // N0r  (imaginary part of xi1st along x; continuous/central)
  const double* xi_y;     // N1
  const double* xi_z;     // N2
  // forward/backward difference (FWBW): per axis and FFT index the complex factors
  // D = e^(i theta) - 1 and E = e^(i theta) + 1 (4 doubles: D.re, D.im, E.re, E.im),
  // xi_p = D_p E_q E_r / (4 h_p) with q, r the other two axes; null otherwise
  const double* fw[3];
  double fw_h4[3];        // 4 h_p = 4 size_p / cells_p
  double resc[3];         // geom / scaled_geom
  const double* C_ref;    // 81, device (gamma_table input)
  const void* gtab;       // per-frequency K^-1 table of C_ref (gamma_table), spectrum precision
  const double* aim;      // 9, device (zero-frequency value), may be null when !gamma
  int do_gamma, do_div;
  int store_fwd;          // without gamma: write the z transform back (forward, or inverse if zsign > 0)
  int zsign;              // with store_fwd: -1 forward (default 0 means forward), +1 inverse
  double* div_part;       // N0r * N1 partials of the divergence sum, one per frequency line (FP64)
};

// one RVE of a size-grouped batched convolution (selected by blockIdx.y)
struct SpecItem {
  const double* in;       // 9 real planes, ld = N
  double* out;            // 9 real planes, ld = N (Gamma * in)
  void* spec;             // 9 Nh complex (FP64 or FP32)
  const void* gtab;       // the RVE's K^-1 table (gamma_table)
  const double* aim;      // 9, zero-frequency value
  double* div_part;       // ndiv partials of the divergence sum
  double* rms;            // divergence RMS out
};

// The Gamma operator depends on the frequency only through K^-1(xi) of the reference
// stiffness, which stays fixed between reference-stiffness updates: gamma_table
// evaluates it once per frequency (layout: entry planes of Nh, frequency index
// (y N0r + x) N2 + z) into gtab, of gamma_table_bytes.  FP64 spectra: the 9 entries of
// the real K^-1 (continuous / central difference) or of the complex (K^*)^-1 (FWBW, 18
// reals); FP32 spectra: the same in FP32, the real one as its 6 symmetric entries.
size_t gamma_table_bytes(const SpecGeom& g, bool fp32, bool fwbw);
void gamma_table(const SpecGeom& g, bool fp32, const GammaArgs& ga, void* gtab, cudaStream_t st);

// cos/sin of 2 pi j / n with the argument reduced to the first octant
void twiddle(long j, long n, double* c, double* s);
// radix factorisation (4, 2, then odd primes in increasing order); number of stages or -1
int factorize(int n, int* rad);
// twiddle tables exp(-2 pi i j / n), j < n, in FP64 and FP32
void axis_tables(int n, std::vector<double2>& tw, std::vector<float2>& twf);
// plan of one axis without tables (tw / twf null); false if n has more than 16 factors
bool axis_plan(int n, AxisPlan* p);
bool axis_create(AxisHost* ax, int n);
// MechBase::base_init divergence correction: scaled geometry for 0 none, 1 size, 2 size+grid
void scaled_geometry(const int cells[3], const double size[3], int divergence_correction, double out[3]);
// imaginary parts of xi1st along one axis (continuous 0 / central difference 1)
void xi_axis(int axis, const int cells[3], const double size[3], int derivative, std::vector<double>& v);
// opt-in dynamic shared memory per block of the current device
size_t smem_optin_limit();
void axis_destroy(AxisHost* ax);
SpecLaunch spec_launch(int N0, int N1, int N2, size_t csize);
// explicit tile shape (autotuner); spec_launch_fits: shared memory within the limit
SpecLaunch spec_launch_tiles(int N0, int N1, int N2, size_t csize, int LX, int TIy, int TIz);
bool spec_launch_fits(const SpecLaunch& L);
// raise the kernels' dynamic shared-memory limits on the current device for L; false if
// L does not fit the device or the attribute could not be set
bool spec_prepare(const SpecLaunch& L, bool fp32);
void spec_convolve(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                   const double* in, double* field, long long ld, void* spec, const GammaArgs& ga, cudaStream_t st);
// Displacements of the deformed grid from the deformation gradient planes F (ld):
// u_p (3 per cell) and u_n (3 per node, (N0+1)(N1+1)(N2+1)), AoS, x fastest.
// scratch: 9 real planes (ld); Favg: 9 doubles out (device).
void spec_update_coords(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                        const double* F, long long ld, void* spec, double* scratch, const double size[3],
                        int derivative, const GammaArgs& xi, double wgt, double* Favg, double* u_n, double* u_p,
                        cudaStream_t st);
// host table of the FWBW factors (D, E) of one axis in FFT index order (4 doubles each)
void fw_axis(int axis, const int cells[3], std::vector<double>& v);
// nitems RVEs of the same grid (and precision) in one launch per pass; items in device memory
void spec_convolve_batch(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                         const SpecItem* items, int nitems, const GammaArgs& ga, cudaStream_t st);
void spec_div_finish_batch(const SpecItem* items, int nitems, int nb, double wgt, int N0, cudaStream_t st);
void spec_div_finish(const double* part, int nb, double wgt, int N0, double* out, cudaStream_t st);

}  // namespace dgx
