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
//    before any stream capture on the device;
//  * the FFT twiddles and frequency tables are built on the host by the same code
//    as the regular entry point and copied into the array on every call
//    (cudaMemcpyAsync from pageable host memory: the call returns once the host
//    data is staged), so both entry points use identical tables.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/dgx.h"
#include "spectral.cuh"

namespace dgx { void set_err(const char* fmt, ...); }

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

// device address of g_scratch per device, looked up once per device (host threads may
// call concurrently: the lookup runs under a lock, readers see a published pointer)
constexpr int MAX_DEVICES = 64;
static std::atomic<double*> g_scratch_ptr[MAX_DEVICES];
static std::mutex g_scratch_mu;

double* scratch_address(int dev) {
  double* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (p) return p;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  p = g_scratch_ptr[dev].load(std::memory_order_relaxed);
  if (p) return p;
  if (cudaGetSymbolAddress((void**)&p, g_scratch) != cudaSuccess || !p) return nullptr;
  g_scratch_ptr[dev].store(p, std::memory_order_release);
  return p;
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
  using dgx::set_err;
  if (!cells || !size || !P_device || !rms_device) { set_err("dgx_divergence_rms_static: null argument"); return DGX_ERR_ARG; }
  for (int i = 0; i < 3; ++i)
    if (cells[i] < 1 || !(size[i] > 0.0)) { set_err("dgx_divergence_rms_static: bad cells / size"); return DGX_ERR_ARG; }
  if (divergence_correction < 0 || divergence_correction > 2) {
    set_err("dgx_divergence_rms_static: divergence_correction must be 0, 1 or 2"); return DGX_ERR_ARG;
  }
  if (derivative == 2) { set_err("dgx_divergence_rms_static: FWBW derivative not supported here"); return DGX_ERR_UNSUPPORTED; }
  if (derivative != 0 && derivative != 1) { set_err("dgx_divergence_rms_static: derivative must be 0 or 1"); return DGX_ERR_ARG; }
  const long long N = (long long)cells[0] * cells[1] * cells[2];
  if (N > MAXC) { set_err("dgx_divergence_rms_static: %lld cells exceed the static limit of %lld", N, MAXC); return DGX_ERR_ARG; }
  dgx::AxisPlan plan[3];
  for (int i = 0; i < 3; ++i)
    if (!dgx::axis_plan(cells[i], &plan[i])) { set_err("dgx_divergence_rms_static: no FFT plan for %d", cells[i]); return DGX_ERR_UNSUPPORTED; }
  // an error left pending by earlier work on this thread is reported as such, and
  // left in place, rather than attributed to this call
  cudaError_t pend = cudaPeekAtLastError();
  if (pend != cudaSuccess) {
    set_err("dgx_divergence_rms_static: CUDA error pending from earlier work: %s", cudaGetErrorString(pend));
    return DGX_ERR_CUDA;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) { set_err("dgx_divergence_rms_static: no device"); return DGX_ERR_CUDA; }
  dgx::SpecLaunch L = dgx::spec_launch(cells[0], cells[1], cells[2], sizeof(double2));
  if (!dgx::spec_prepare(L, false)) { set_err("dgx_divergence_rms_static: FFT line tiles exceed shared memory"); return DGX_ERR_UNSUPPORTED; }
  double* base = scratch_address(dev);
  if (!base) { set_err("dgx_divergence_rms_static: cudaGetSymbolAddress failed"); return DGX_ERR_CUDA; }
  cudaStream_t st = (cudaStream_t)stream;
  double scaled[3];
  dgx::scaled_geometry(cells, size, divergence_correction, scaled);
  double* planes = base + OFF_PLANAR;
  double* spec = base + OFF_SPEC;
  double* xi[3];
  // twiddle and frequency tables: the same host tables as the regular entry point,
  // copied from host memory into the static array (no device allocation)
  for (int i = 0; i < 3; ++i) {
    double2* tw = reinterpret_cast<double2*>(base + OFF_TW + 3 * TW_LEN * i);
    float2* twf = reinterpret_cast<float2*>(base + OFF_TW + 3 * TW_LEN * i + 2 * TW_LEN);
    xi[i] = base + OFF_XI + TW_LEN * i;
    std::vector<double2> h_tw;
    std::vector<float2> h_twf;
    std::vector<double> h_xi;
    dgx::axis_tables(cells[i], h_tw, h_twf);
    dgx::xi_axis(i, cells, size, derivative, h_xi);
    if (cudaMemcpyAsync(tw, h_tw.data(), sizeof(double2) * h_tw.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(twf, h_twf.data(), sizeof(float2) * h_twf.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(xi[i], h_xi.data(), sizeof(double) * h_xi.size(), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      set_err("dgx_divergence_rms_static: table upload: %s", cudaGetErrorString(cudaGetLastError()));
      return DGX_ERR_CUDA;
    }
    plan[i].tw = tw;
    plan[i].twf = twf;
  }
  k_interleaved_to_planes<<<(int)((9 * N + 255) / 256), 256, 0, st>>>(P_device, N, planes);
  dgx::GammaArgs ga{};
  ga.xi_x = xi[0]; ga.xi_y = xi[1]; ga.xi_z = xi[2];
  for (int i = 0; i < 3; ++i) ga.resc[i] = size[i] / scaled[i];
  ga.do_gamma = 0; ga.do_div = 1; ga.store_fwd = 0;
  ga.div_part = base + OFF_PART;
  dgx::spec_convolve(L, false, plan[0], plan[1], plan[2], planes, planes, N, spec, ga, st);
  dgx::spec_div_finish(ga.div_part, L.ndiv, std::pow((double)N, -1.0), cells[0], rms_device, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_err("dgx_divergence_rms_static: launch: %s", cudaGetErrorString(e)); return DGX_ERR_CUDA; }
  return DGX_OK;
}
