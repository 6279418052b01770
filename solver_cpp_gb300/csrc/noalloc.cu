// noalloc.cu -- divergence RMS of a stress field without any device allocation.
//
// For callers that cannot call cudaMalloc: code that owns all device memory
// through its own pool (a serving process with a fixed device budget, a host
// framework whose allocator must not be bypassed), or code that must not pay
// allocation latency inside a time-critical loop.  Those callers hand in the
// input and output buffers they already own; the scratch this computation needs
// (planar copy of the field, half spectrum, FFT twiddles, frequency tables,
// block partials) lives in one file-scope device array of fixed size.
//
// Limits and rules:
//  * at most DGX_STATIC_MAX_CELLS = 32768 cells (e.g. 32^3); larger grids are
//    rejected with DGX_ERR_ARG; the array is 10 MiB and every GPU that loads the
//    library holds it until the process exits;
//  * every call shares the array and leaves the last call's contents in it;
//    calls that overlap on the GPU (different streams, or host threads issuing
//    calls concurrently) race on it and must be serialised by the caller;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture on the device.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/dgx.h"
#include "spectral.cuh"

namespace {

constexpr long long MAXC = 32768;                     // DGX_STATIC_MAX_CELLS
// layout of the scratch array, in doubles
constexpr long long OFF_PLANAR = 0;                   // 9 * MAXC real planes
constexpr long long OFF_SPEC = OFF_PLANAR + 9 * MAXC; // <= 9 * MAXC complex
constexpr long long OFF_TW = OFF_SPEC + 18 * MAXC;    // twiddles: 2 doubles + 1 float2 per entry
constexpr long long TW_LEN = MAXC + 64;               // per-axis capacity (entries)
constexpr long long OFF_XI = OFF_TW + 3 * 3 * TW_LEN; // xi_x, xi_y, xi_z
constexpr long long OFF_PART = OFF_XI + 3 * TW_LEN;   // divergence partials, N0r * N1 <= MAXC
constexpr long long SCRATCH_DOUBLES = OFF_PART + MAXC + 64;

static __device__ __align__(256) double g_scratch[SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
static double* g_scratch_ptr[MAX_DEVICES] = {nullptr};

// twiddles exp(-2 pi i j / n) (FP64 and FP32) with the octant reduction used by
// the host tables, and the xi1st frequency table (imaginary parts) of one axis
__global__ void k_axis_tables(int n, int nxi, int axis_is_x, double size, int derivative, double2* tw, float2* twf,
                              double* xi) {
  const double TAU = 6.283185307179586476925286766559;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n || j < nxi; j += gridDim.x * blockDim.x) {
    if (j < n) {
      long q = (4L * j) / n, r = 4L * j - q * n;
      double c0, s0;
      if (r == 0) { c0 = 1.0; s0 = 0.0; }
      else if (2 * r <= n) { double a = (TAU / 4.0) * ((double)r / (double)n); c0 = cos(a); s0 = sin(a); }
      else { double a = (TAU / 4.0) * ((double)(n - r) / (double)n); c0 = sin(a); s0 = cos(a); }
      double c, s;
      switch (q) {
        case 0: c = c0; s = s0; break;
        case 1: c = -s0; s = c0; break;
        case 2: c = -c0; s = -s0; break;
        default: c = s0; s = -c0; break;
      }
      tw[j] = make_double2(c, -s);
      twf[j] = make_float2((float)c, (float)-s);
    }
    if (j < nxi) {
      int k = axis_is_x ? j : (j > n / 2 ? j - n : j);
      double val = derivative == 0 ? TAU * k / size : sin(TAU * k / n) / (2.0 * size / n);
      bool nyq = (n % 2 == 0) && (j == n / 2) && derivative == 0;
      xi[j] = nyq ? 0.0 : val;
    }
  }
}

// reference layout (3,3,N) interleaved -> 9 planes
__global__ void k_interleaved_to_planes(const double* __restrict__ a, long long n, double* __restrict__ p) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 9 * n) return;
  long long e = t / 9;
  int c = (int)(t - e * 9);
  p[c * n + e] = a[t];
}

}  // namespace

extern "C" dgx_status dgx_divergence_rms_static(const int32_t cells[3], const double size[3],
                                                int32_t divergence_correction, int32_t derivative,
                                                const double* P_device, double* rms_device, void* stream) {
  if (!cells || !size || !P_device || !rms_device) return DGX_ERR_ARG;
  for (int i = 0; i < 3; ++i)
    if (cells[i] < 1 || !(size[i] > 0.0)) return DGX_ERR_ARG;
  const long long N = (long long)cells[0] * cells[1] * cells[2];
  if (N > MAXC) return DGX_ERR_ARG;                    // beyond the static scratch
  if (derivative != 0 && derivative != 1) return DGX_ERR_UNSUPPORTED;
  dgx::AxisPlan plan[3];
  for (int i = 0; i < 3; ++i) {
    plan[i].n = cells[i];
    plan[i].nstages = dgx::factorize(cells[i], plan[i].radix);
    if (plan[i].nstages < 0) return DGX_ERR_UNSUPPORTED;
    for (int k = 0; k < plan[i].nstages; ++k)
      if (plan[i].radix[k] > 16) return DGX_ERR_UNSUPPORTED;
  }
  dgx::SpecLaunch L = dgx::spec_launch(cells[0], cells[1], cells[2], sizeof(double2));
  const size_t SMEM_MAX = 227 * 1024;                  // one line tile per pass must fit shared memory
  if (L.smx > SMEM_MAX || L.smy > SMEM_MAX || L.smz > SMEM_MAX) return DGX_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return DGX_ERR_CUDA;
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_scratch) != cudaSuccess || !p) return DGX_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  double* base = g_scratch_ptr[dev];
  cudaStream_t st = (cudaStream_t)stream;
  // divergence correction of the reference (MechBase::base_init)
  double scaled[3];
  {
    int idx[3] = {0, 1, 2};
    if (divergence_correction == 1 || divergence_correction == 2) {
      double key[3];
      for (int i = 0; i < 3; ++i) key[i] = divergence_correction == 1 ? size[i] : size[i] / (double)cells[i];
      for (int a = 1; a < 3; ++a)
        for (int b = a; b > 0 && key[idx[b]] < key[idx[b - 1]]; --b) { int t = idx[b]; idx[b] = idx[b - 1]; idx[b - 1] = t; }
      for (int j = 0; j < 3; ++j)
        scaled[j] = divergence_correction == 1 ? size[j] / size[idx[1]] : size[j] / size[idx[1]] * cells[idx[1]];
    } else {
      for (int j = 0; j < 3; ++j) scaled[j] = size[j];
    }
  }
  double* planes = base + OFF_PLANAR;
  double* spec = base + OFF_SPEC;
  double* xi[3];
  for (int i = 0; i < 3; ++i) {
    double2* tw = reinterpret_cast<double2*>(base + OFF_TW + 3 * TW_LEN * i);
    float2* twf = reinterpret_cast<float2*>(base + OFF_TW + 3 * TW_LEN * i + 2 * TW_LEN);
    xi[i] = base + OFF_XI + TW_LEN * i;
    int nxi = i == 0 ? cells[0] / 2 + 1 : cells[i];
    k_axis_tables<<<64, 256, 0, st>>>(cells[i], nxi, i == 0, size[i], derivative, tw, twf, xi[i]);
    plan[i].tw = tw;
    plan[i].twf = twf;
  }
  k_interleaved_to_planes<<<(int)((9 * N + 255) / 256), 256, 0, st>>>(P_device, N, planes);
  dgx::spec_prepare(L, false);
  dgx::GammaArgs ga{};
  ga.xi_x = xi[0]; ga.xi_y = xi[1]; ga.xi_z = xi[2];
  for (int i = 0; i < 3; ++i) ga.resc[i] = size[i] / scaled[i];
  ga.do_gamma = 0; ga.do_div = 1; ga.store_fwd = 0;
  ga.div_part = base + OFF_PART;
  dgx::spec_convolve(L, false, plan[0], plan[1], plan[2], planes, planes, N, spec, ga, st);
  dgx::spec_div_finish(ga.div_part, L.ndiv, std::pow((double)N, -1.0), cells[0], rms_device, st);
  return cudaGetLastError() == cudaSuccess ? DGX_OK : DGX_ERR_CUDA;
}
