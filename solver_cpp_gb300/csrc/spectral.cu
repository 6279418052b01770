// spectral.cu -- 3-D real FFTs of the 9-component tensor field on sm_103a, fused
// with the Fourier-space Gamma convolution and the divergence-RMS reduction.
//
// Reference behaviour (reference paths):
//   src/grid/fft.h:37-60, fft.cpp:9-78   unnormalised r2c / c2r of (3,3,N0,N1,N2) fields
//   src/grid/spectral.cpp:53-130         xi1st (continuous / central difference), Nyquist zeroing
//   src/grid/mech_base.cpp:302-398       divergence RMS with half-spectrum weights
//   src/grid/mech_base.cpp:156-205, 400-477  Gamma_hat(xi; C_ref) : P_hat, zero frequency <- aim
// Pipeline of one convolution (all FP64 in the plain form, FP32 spectrum in the
// mixed form), spectrum stored component-planar, x-frequency fastest:
//   x-pass  r2c of each x line               (real planes -> half spectrum)
//   y-pass  complex FFT along y              (tile of x-frequencies, coalesced)
//   z-pass  forward FFT along z, per-frequency div-RMS + Gamma, inverse FFT along z
//           (all 9 components of a pencil tile resident in shared memory)
//   y-pass  inverse
//   x-pass  c2r (Hermitian extension), real planes out
// Line FFTs are Stockham autosort (radix 4/2 butterflies with exact +-i, other
// radices by a direct DFT) in shared memory with twiddles from a host table.
#include <cuda_runtime.h>
#include <cstdint>

#include "dgx_internal.cuh"
#include "spectral.cuh"

namespace dgx {

template <typename T> struct cpx;
template <> struct cpx<double> { typedef double2 t; };
template <> struct cpx<float> { typedef float2 t; };

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}


// twiddle exp(sign 2 pi i j / n) for 0 <= j < n
template <typename R> __device__ __forceinline__ typename cpx<R>::t twid(const AxisPlan& p, int j, int sign) {
  typename cpx<R>::t w;
  if constexpr (sizeof(R) == 8) { double2 t = p.tw[j]; w.x = t.x; w.y = sign > 0 ? -t.y : t.y; }
  else { float2 t = p.twf[j]; w.x = t.x; w.y = sign > 0 ? -t.y : t.y; }
  return w;
}

__device__ __forceinline__ int ilog2_or_neg(int v) { return (v & (v - 1)) == 0 ? __ffs(v) - 1 : -1; }

// Stockham FFT of `nl` lines of length p.n, stored contiguously (line l at a + l*n).
// Returns the buffer that holds the result (a or b).  sign -1 forward, +1 inverse.
// Index arithmetic uses shifts when the stage sizes are powers of two; the first stage
// (all twiddles 1) skips the twiddle products, which leaves the results unchanged.
template <typename R>
__device__ typename cpx<R>::t* block_fft(typename cpx<R>::t* a, typename cpx<R>::t* b, int nl, const AxisPlan& p, int sign) {
  typedef typename cpx<R>::t C;
  const int n = p.n;
  int Ls = 1;
  for (int s = 0; s < p.nstages; ++s) {
    const int r = p.radix[s], m = n / r;
    const int tot = nl * m;
    const int mlog = ilog2_or_neg(m), llog = ilog2_or_neg(Ls);
    const int tws = n / (Ls * r);
    const bool first = Ls == 1;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
      int line, j, k, jl;
      if (mlog >= 0) { line = t >> mlog; j = t & (m - 1); }
      else { line = t / m; j = t - line * m; }
      if (llog >= 0) { k = j & (Ls - 1); jl = j >> llog; }
      else { jl = j / Ls; k = j - jl * Ls; }
      const C* in = a + (long)line * n;
      C* out = b + (long)line * n;
      const int od = jl * Ls * r + k;
      const int twstep = tws * k;
      if (r == 2) {
        C v0 = in[j], v1 = first ? in[j + m] : cmul(in[j + m], twid<R>(p, twstep, sign));
        C y0, y1; y0.x = v0.x + v1.x; y0.y = v0.y + v1.y; y1.x = v0.x - v1.x; y1.y = v0.y - v1.y;
        out[od] = y0; out[od + Ls] = y1;
      } else if (r == 4) {
        C v0 = in[j], v1, v2, v3;
        if (first) { v1 = in[j + m]; v2 = in[j + 2 * m]; v3 = in[j + 3 * m]; }
        else {
          v1 = cmul(in[j + m], twid<R>(p, twstep, sign));
          v2 = cmul(in[j + 2 * m], twid<R>(p, 2 * twstep, sign));
          v3 = cmul(in[j + 3 * m], twid<R>(p, 3 * twstep, sign));
        }
        C s02, d02, s13, d13;
        s02.x = v0.x + v2.x; s02.y = v0.y + v2.y; d02.x = v0.x - v2.x; d02.y = v0.y - v2.y;
        s13.x = v1.x + v3.x; s13.y = v1.y + v3.y; d13.x = v1.x - v3.x; d13.y = v1.y - v3.y;
        // (v1 - v3) * (-i) forward, * (+i) inverse
        C rot; if (sign < 0) { rot.x = d13.y; rot.y = -d13.x; } else { rot.x = -d13.y; rot.y = d13.x; }
        C y0, y1, y2, y3;
        y0.x = s02.x + s13.x; y0.y = s02.y + s13.y;
        y2.x = s02.x - s13.x; y2.y = s02.y - s13.y;
        y1.x = d02.x + rot.x; y1.y = d02.y + rot.y;
        y3.x = d02.x - rot.x; y3.y = d02.y - rot.y;
        out[od] = y0; out[od + Ls] = y1; out[od + 2 * Ls] = y2; out[od + 3 * Ls] = y3;
      } else if (r > 16) {
        // a prime factor above 16: each of the r outputs is a direct DFT sum over the
        // r inputs, read from shared memory (no per-thread array)
        for (int s2 = 0; s2 < r; ++s2) {
          C acc = in[j];
          for (int q = 1; q < r; ++q) {
            const C vq = cmul(in[j + q * m], twid<R>(p, q * twstep, sign));
            const C t2 = cmul(vq, twid<R>(p, (int)(((long)q * s2 * m) % n), sign));
            acc.x += t2.x; acc.y += t2.y;
          }
          out[od + s2 * Ls] = acc;
        }
      } else {
        C v[16];
        for (int q = 0; q < r; ++q) v[q] = cmul(in[j + q * m], twid<R>(p, q * twstep, sign));
        for (int s2 = 0; s2 < r; ++s2) {
          C acc; acc.x = v[0].x; acc.y = v[0].y;
          for (int q = 1; q < r; ++q) {
            C w = twid<R>(p, (int)(((long)q * s2 * m) % n), sign);
            C t2 = cmul(v[q], w);
            acc.x += t2.x; acc.y += t2.y;
          }
          out[od + s2 * Ls] = acc;
        }
      }
    }
    __syncthreads();
    C* tmp = a; a = b; b = tmp;
    Ls *= r;
  }
  return a;
}


// ---------------------------------------------------------------- x pass
// forward: real planes (ld_in) -> spectrum planes (stride Nh); one block = LX lines
template <typename R, typename Rin>
__global__ void k_xfwd(SpecGeom g, AxisPlan px, const Rin* __restrict__ field, long long ld_in,
                       typename cpx<R>::t* __restrict__ spec, int LX, const SpecItem* __restrict__ items) {
  typedef typename cpx<R>::t C;
  if (items) { field = (const Rin*)items[blockIdx.y].in; spec = (C*)items[blockIdx.y].spec; }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long nlines = 9LL * g.N1 * g.N2;
  const long long l0 = (long long)blockIdx.x * LX;
  const int nl = (int)min((long long)LX, nlines - l0);
  const int np = (nl + 1) >> 1;          // complex lines: real lines 2j and 2j+1 as z = a + i b (LX even)
  C* a = reinterpret_cast<C*>(smem_raw);
  C* b = a + (long)np * g.N0;
  const long long nyz = (long long)g.N1 * g.N2;
  for (int t = threadIdx.x; t < np * g.N0; t += blockDim.x) {
    const int j = t / g.N0, x = t - j * g.N0;
    const long long L = l0 + 2 * j;
    const long long c = L / nyz, yz = L - c * nyz;
    C v;
    v.x = (R)field[c * ld_in + yz * g.N0 + x];
    if (2 * j + 1 < nl) {
      const long long L1 = L + 1, c1 = L1 / nyz, yz1 = L1 - c1 * nyz;
      v.y = (R)field[c1 * ld_in + yz1 * g.N0 + x];
    } else {
      v.y = 0;
    }
    a[t] = v;
  }
  __syncthreads();
  C* res = block_fft<R>(a, b, np, px, -1);
  // separate the two real lines' spectra: with Z = FFT(a + i b) and W_i = Z_(N0-i),
  // A_i = (Z_i + conj W_i) / 2, B_i = (Z_i - conj W_i) / 2i
  for (int t = threadIdx.x; t < nl * g.N0r; t += blockDim.x) {
    const int l = t / g.N0r, i = t - l * g.N0r;
    const int j = l >> 1;
    const C z = res[(long)j * g.N0 + i], w = res[(long)j * g.N0 + (i == 0 ? 0 : g.N0 - i)];
    C v;
    if ((l & 1) == 0) { v.x = (R)0.5 * (z.x + w.x); v.y = (R)0.5 * (z.y - w.y); }
    else { v.x = (R)0.5 * (z.y + w.y); v.y = (R)0.5 * (w.x - z.x); }
    const long long L = l0 + l;
    const long long c = L / nyz, yz = L - c * nyz;
    spec[c * g.Nh + yz * g.N0r + i] = v;
  }
}

// inverse: spectrum -> real planes (ld_out), c2r by Hermitian extension; the half
// spectra A, B of real lines 2j, 2j+1 are transformed together as z = A + i B (both
// Hermitian-extended), whose inverse is a + i b.
template <typename R, typename Rout>
__global__ void k_xinv(SpecGeom g, AxisPlan px, const typename cpx<R>::t* __restrict__ spec, Rout* __restrict__ field,
                       long long ld_out, int LX, const SpecItem* __restrict__ items) {
  typedef typename cpx<R>::t C;
  if (items) { spec = (const C*)items[blockIdx.y].spec; field = (Rout*)items[blockIdx.y].out; }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long nlines = 9LL * g.N1 * g.N2;
  const long long l0 = (long long)blockIdx.x * LX;
  const int nl = (int)min((long long)LX, nlines - l0);
  const int np = (nl + 1) >> 1;
  C* a = reinterpret_cast<C*>(smem_raw);
  C* b = a + (long)np * g.N0;
  C* hs = b + (long)np * g.N0;           // the nl half spectra (2 np N0 + nl N0r <= 2 LX N0)
  const long long nyz = (long long)g.N1 * g.N2;
  for (int t = threadIdx.x; t < nl * g.N0r; t += blockDim.x) {
    const int l = t / g.N0r, i = t - l * g.N0r;
    const long long L = l0 + l;
    const long long c = L / nyz, yz = L - c * nyz;
    hs[t] = spec[c * g.Nh + yz * g.N0r + i];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < np * g.N0; t += blockDim.x) {
    const int j = t / g.N0, k = t - j * g.N0;
    const bool hi = k >= g.N0r;
    const int kk = hi ? g.N0 - k : k;
    C A = hs[(long)(2 * j) * g.N0r + kk], B;
    if (2 * j + 1 < nl) B = hs[(long)(2 * j + 1) * g.N0r + kk];
    else { B.x = 0; B.y = 0; }
    if (hi) { A.y = -A.y; B.y = -B.y; }
    C v;
    v.x = A.x - B.y; v.y = A.y + B.x;
    a[t] = v;
  }
  __syncthreads();
  C* res = block_fft<R>(a, b, np, px, +1);
  for (int t = threadIdx.x; t < nl * g.N0; t += blockDim.x) {
    const int l = t / g.N0, x = t - l * g.N0;
    const C v = res[(long)(l >> 1) * g.N0 + x];
    const long long L = l0 + l;
    const long long c = L / nyz, yz = L - c * nyz;
    field[c * ld_out + yz * g.N0 + x] = (Rout)((l & 1) ? v.y : v.x);
  }
}

// ---------------------------------------------------------------- y pass
// block = (tile of TI x-frequencies) x (component, z); lines along y, stride N0r
template <typename R>
__global__ void k_ypass(SpecGeom g, AxisPlan py, typename cpx<R>::t* __restrict__ spec, int TI, int sign,
                        const SpecItem* __restrict__ items) {
  typedef typename cpx<R>::t C;
  if (items) spec = (C*)items[blockIdx.y].spec;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* a = reinterpret_cast<C*>(smem_raw);
  C* b = a + (long)TI * g.N1;
  const int ntile = (g.N0r + TI - 1) / TI;
  const int tile = blockIdx.x % ntile;
  const long long cz = blockIdx.x / ntile;           // c * N2 + z
  const long long c = cz / g.N2, z = cz - c * g.N2;
  const int i0 = tile * TI;
  const int ti = min(TI, g.N0r - i0);
  C* base = spec + c * g.Nh + z * (long long)g.N1 * g.N0r;
  for (int t = threadIdx.x; t < ti * g.N1; t += blockDim.x) {
    int y = t / ti, i = t - y * ti;
    a[(long)i * g.N1 + y] = base[(long long)y * g.N0r + i0 + i];
  }
  __syncthreads();
  C* res = block_fft<R>(a, b, ti, py, sign);
  for (int t = threadIdx.x; t < ti * g.N1; t += blockDim.x) {
    int y = t / ti, i = t - y * ti;
    base[(long long)y * g.N0r + i0 + i] = res[(long)i * g.N1 + y];
  }
}

// ---------------------------------------------------------------- z pass + Gamma + div

// xi of one frequency for the forward/backward difference: xi_p = D_p E_q E_r / (4 h_p)
// (q, r the next two axes, cyclically), the complex factors from the per-axis tables
__device__ __forceinline__ void fw_xi(const GammaArgs& ga, int ix, int y, int z, double2 xi[3]) {
  const double* t[3] = {ga.fw[0] + 4 * ix, ga.fw[1] + 4 * y, ga.fw[2] + 4 * z};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const double* a = t[p];
    const double* b = t[(p + 1) % 3];
    const double* c = t[(p + 2) % 3];
    const double abr = a[0] * b[2] - a[1] * b[3], abi = a[0] * b[3] + a[1] * b[2];
    const double xr = abr * c[2] - abi * c[3], xim = abr * c[3] + abi * c[2];
    xi[p] = make_double2(xr / ga.fw_h4[p], xim / ga.fw_h4[p]);
  }
}

// Number of entries per frequency of the Gamma table.
__host__ __device__ constexpr int gtab_entries(bool fp32, bool fw) { return fw ? 18 : (fp32 ? 6 : 9); }

// K^-1(xi) per half-spectrum frequency (the spectral operator's only dependence on the
// reference stiffness), evaluated once per reference-stiffness update.  Continuous and
// central derivative: xi = i a (a real), K_lm = -sum_no C_ref(l,n,m,o) a_n a_o real;
// |det K| <= 1e-16 (and xi = 0) gives a zero operator.  FWBW: K_lm = sum_no
// C_ref(l,n,m,o) conj(-xi_n) xi_o (Hermitian), the determinant test on Re K, and the
// operator uses the inverse of conj(K), as the real 6x6 form [[Re K, Im K],
// [-Im K, Re K]] of the reference's update_gamma (mech_base.cpp:164-205) inverts it.
template <typename R, bool FW>
__global__ void k_gamma_table(SpecGeom g, GammaArgs ga, R* __restrict__ tab) {
  __shared__ double s_C[81];
  for (int k = threadIdx.x; k < 81; k += blockDim.x) s_C[k] = ga.C_ref[k];
  __syncthreads();                      // every thread of the block reaches this barrier
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (f >= g.Nh) return;
  const int z = (int)(f % g.N2);
  const long long xy = f / g.N2;
  const int ix = (int)(xy % g.N0r), y = (int)(xy / g.N0r);
  constexpr int NE = gtab_entries(sizeof(R) == 4, FW);
  R out[NE];
#pragma unroll
  for (int k = 0; k < NE; ++k) out[k] = R(0);
  if constexpr (!FW) {
    const double av[3] = {ga.xi_x[ix], ga.xi_y[y], ga.xi_z[z]};
    double K[9];
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        double s = 0.0;
#pragma unroll
        for (int nn = 0; nn < 3; ++nn)
#pragma unroll
          for (int o = 0; o < 3; ++o) s = fma(s_C[l + 3 * nn + 9 * m + 27 * o], av[nn] * av[o], s);
        K[l + 3 * m] = -s;
      }
    double c0 = K[4] * K[8] - K[7] * K[5], c1 = -K[1] * K[8] + K[7] * K[2], c2 = K[1] * K[5] - K[4] * K[2];
    double det = K[0] * c0 + K[3] * c1 + K[6] * c2;
    if (f != 0 && fabs(det) > 1e-16) {
      double r = 1.0 / det;
      double Ki[9] = {c0 * r, c1 * r, c2 * r,
                      (-K[3] * K[8] + K[6] * K[5]) * r, (K[0] * K[8] - K[6] * K[2]) * r, (-K[0] * K[5] + K[3] * K[2]) * r,
                      (K[3] * K[7] - K[6] * K[4]) * r, (-K[0] * K[7] + K[6] * K[1]) * r, (K[0] * K[4] - K[3] * K[1]) * r};
      if constexpr (sizeof(R) == 8) {
#pragma unroll
        for (int k = 0; k < 9; ++k) out[k] = Ki[k];
      } else {
        // symmetric: 00 11 22 01 02 12
        out[0] = (R)Ki[0]; out[1] = (R)Ki[4]; out[2] = (R)Ki[8];
        out[3] = (R)Ki[3]; out[4] = (R)Ki[6]; out[5] = (R)Ki[7];
      }
    }
  } else {
    double2 xi[3];
    fw_xi(ga, ix, y, z, xi);
    // dyad(n, o) = conj(-xi_n) xi_o
    double dr[9], di[9];
#pragma unroll
    for (int nn = 0; nn < 3; ++nn)
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        const double ar = -xi[nn].x, ai = xi[nn].y;     // conj(-xi_n)
        dr[nn + 3 * o] = ar * xi[o].x - ai * xi[o].y;
        di[nn + 3 * o] = ar * xi[o].y + ai * xi[o].x;
      }
    double Kr[9], Kim[9];
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        double sr = 0.0, si = 0.0;
#pragma unroll
        for (int nn = 0; nn < 3; ++nn)
#pragma unroll
          for (int o = 0; o < 3; ++o) {
            const double c = s_C[l + 3 * nn + 9 * m + 27 * o];
            sr = fma(c, dr[nn + 3 * o], sr);
            si = fma(c, di[nn + 3 * o], si);
          }
        Kr[l + 3 * m] = sr; Kim[l + 3 * m] = si;
      }
    const double detr = Kr[0] * (Kr[4] * Kr[8] - Kr[7] * Kr[5]) - Kr[3] * (Kr[1] * Kr[8] - Kr[7] * Kr[2]) +
                        Kr[6] * (Kr[1] * Kr[5] - Kr[4] * Kr[2]);
    if (f != 0 && fabs(detr) > 1e-16) {
      // M = conj(K): complex adjugate over the complex determinant
      double Mr[9], Mi[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) { Mr[k] = Kr[k]; Mi[k] = -Kim[k]; }
      auto cm = [](double ar, double ai, double br, double bi, double& r, double& i) { r = ar * br - ai * bi; i = ar * bi + ai * br; };
      // cofactor C(i,j) of M, stored as adj(j,i)
      double Ar[9], Ai[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
          double pr, pi, qr, qi;
          cm(Mr[i1 + 3 * j1], Mi[i1 + 3 * j1], Mr[i2 + 3 * j2], Mi[i2 + 3 * j2], pr, pi);
          cm(Mr[i1 + 3 * j2], Mi[i1 + 3 * j2], Mr[i2 + 3 * j1], Mi[i2 + 3 * j1], qr, qi);
          Ar[j + 3 * i] = pr - qr; Ai[j + 3 * i] = pi - qi;
        }
      double dr_ = 0.0, di_ = 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {       // det = sum_j M(0,j) C(0,j) = sum_j M(0,j) adj(j,0)
        double pr, pi;
        cm(Mr[3 * j], Mi[3 * j], Ar[j], Ai[j], pr, pi);
        dr_ += pr; di_ += pi;
      }
      const double n2 = dr_ * dr_ + di_ * di_;
      const double ir = dr_ / n2, ii = -di_ / n2;          // 1 / det
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        double r, i;
        cm(Ar[k], Ai[k], ir, ii, r, i);
        out[2 * k] = (R)r; out[2 * k + 1] = (R)i;
      }
    }
  }
  const long long gi = ((long long)y * g.N0r + ix) * g.N2 + z;
#pragma unroll
  for (int k = 0; k < NE; ++k) tab[k * g.Nh + gi] = out[k];
}

// 2 blocks of 256 threads per SM (register cap 128)
template <typename R, bool FW>
__global__ void __launch_bounds__(256, 2) k_zpass(SpecGeom g, AxisPlan pz, typename cpx<R>::t* __restrict__ spec, int TI, GammaArgs ga,
                        const SpecItem* __restrict__ items) {
  typedef typename cpx<R>::t C;
  if (items) {
    const SpecItem& it = items[blockIdx.y];
    spec = (C*)it.spec; ga.gtab = it.gtab; ga.aim = it.aim; ga.div_part = it.div_part;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int per = TI * g.N2;                       // lines x length per component
  C* a = reinterpret_cast<C*>(smem_raw);
  C* b = a + 9L * per;
  double* s_val = reinterpret_cast<double*>(b + 9L * per);   // weighted |div|^2 per frequency of the tile
  const int ntile = (g.N0r + TI - 1) / TI;
  const int tile = blockIdx.x % ntile;
  const int y = blockIdx.x / ntile;
  const int i0 = tile * TI;
  const int ti = min(TI, g.N0r - i0);
  const long long zs = (long long)g.N1 * g.N0r;
  // load: line (c, i) at a + (c*ti + i) * N2
  for (int t = threadIdx.x; t < 9 * ti * g.N2; t += blockDim.x) {
    int c = t / (ti * g.N2), rem = t - c * ti * g.N2;
    int z = rem / ti, i = rem - z * ti;
    a[((long)c * ti + i) * g.N2 + z] = spec[c * g.Nh + z * zs + (long long)y * g.N0r + i0 + i];
  }
  __syncthreads();
  C* res = block_fft<R>(a, b, 9 * ti, pz, (ga.store_fwd && !ga.do_gamma && ga.zsign > 0) ? +1 : -1);
  C* other = (res == a) ? b : a;
  const R* gt = reinterpret_cast<const R*>(ga.gtab);
  for (int t = threadIdx.x; (ga.do_div || ga.do_gamma) && t < ti * g.N2; t += blockDim.x) {
    int i = t / g.N2, z = t - i * g.N2;
    int ix = i0 + i;
    C Ph[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) Ph[c] = res[((long)c * ti + i) * g.N2 + z];
    double ax = 0.0, ay = 0.0, az = 0.0;
    double2 xi[3];
    if constexpr (FW) fw_xi(ga, ix, y, z, xi);
    else { ax = ga.xi_x[ix]; ay = ga.xi_y[y]; az = ga.xi_z[z]; }
    if (ga.do_div) {
      double wgt = (ix == 0 ? 1.0 : 0.0) + (ix == g.N0r - 1 ? 1.0 : 0.0) + ((ix > 0 && ix < g.N0r - 1) ? 2.0 : 0.0);
      double s = 0.0;
      if constexpr (!FW) {
        double bx = ax * ga.resc[0], by = ay * ga.resc[1], bz = az * ga.resc[2];
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          double ur = (double)Ph[l].x * bx + (double)Ph[l + 3].x * by + (double)Ph[l + 6].x * bz;
          double ui = (double)Ph[l].y * bx + (double)Ph[l + 3].y * by + (double)Ph[l + 6].y * bz;
          s += ur * ur + ui * ui;
        }
      } else {
        // prod_l = sum_n P(l, n) conj(-xi_n) resc_n
        double vr[3], vi[3];
#pragma unroll
        for (int nn = 0; nn < 3; ++nn) { vr[nn] = -xi[nn].x * ga.resc[nn]; vi[nn] = xi[nn].y * ga.resc[nn]; }
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          double pr = 0.0, pi = 0.0;
#pragma unroll
          for (int nn = 0; nn < 3; ++nn) {
            const double xr = (double)Ph[l + 3 * nn].x, xim = (double)Ph[l + 3 * nn].y;
            pr += xr * vr[nn] - xim * vi[nn];
            pi += xr * vi[nn] + xim * vr[nn];
          }
          s += pr * pr + pi * pi;
        }
      }
      s_val[t] = wgt * s;
    }
    if (ga.do_gamma) {
      C out[9];
      const long long gi = ((long long)y * g.N0r + ix) * g.N2 + z;
      if (ix == 0 && y == 0 && z == 0) {
#pragma unroll
        for (int c = 0; c < 9; ++c) { out[c].x = (R)ga.aim[c]; out[c].y = 0; }
      } else if constexpr (!FW) {
        // Gamma:P with K^-1 from the table, in the spectrum's precision:
        // v(n) = sum_o a_o P(n,o); w(l) = sum_n Kinv(l,n) v(n); out(l,m) = -a_m w(l)
        R Ki[9];
        if constexpr (sizeof(R) == 8) {
#pragma unroll
          for (int k = 0; k < 9; ++k) Ki[k] = gt[k * g.Nh + gi];
        } else {
          const R k00 = gt[gi], k11 = gt[g.Nh + gi], k22 = gt[2 * g.Nh + gi];
          const R k01 = gt[3 * g.Nh + gi], k02 = gt[4 * g.Nh + gi], k12 = gt[5 * g.Nh + gi];
          Ki[0] = k00; Ki[4] = k11; Ki[8] = k22; Ki[1] = Ki[3] = k01; Ki[2] = Ki[6] = k02; Ki[5] = Ki[7] = k12;
        }
        const R av[3] = {(R)ax, (R)ay, (R)az};
        R vr[3], vi[3];
#pragma unroll
        for (int nn = 0; nn < 3; ++nn) {
          vr[nn] = av[0] * Ph[nn].x + av[1] * Ph[nn + 3].x + av[2] * Ph[nn + 6].x;
          vi[nn] = av[0] * Ph[nn].y + av[1] * Ph[nn + 3].y + av[2] * Ph[nn + 6].y;
        }
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          R wr = Ki[l] * vr[0] + Ki[l + 3] * vr[1] + Ki[l + 6] * vr[2];
          R wi = Ki[l] * vi[0] + Ki[l + 3] * vi[1] + Ki[l + 6] * vi[2];
#pragma unroll
          for (int m = 0; m < 3; ++m) { out[l + 3 * m].x = -av[m] * wr; out[l + 3 * m].y = -av[m] * wi; }
        }
      } else {
        // complex: v(n) = sum_o conj(-xi_o) P(n,o); w(l) = sum_n N(l,n) v(n); out(l,m) = xi_m w(l)
        R vr[3], vi[3];
#pragma unroll
        for (int nn = 0; nn < 3; ++nn) {
          R sr = 0, si = 0;
#pragma unroll
          for (int o = 0; o < 3; ++o) {
            const R cr = (R)(-xi[o].x), ci = (R)xi[o].y;          // conj(-xi_o)
            sr += cr * Ph[nn + 3 * o].x - ci * Ph[nn + 3 * o].y;
            si += cr * Ph[nn + 3 * o].y + ci * Ph[nn + 3 * o].x;
          }
          vr[nn] = sr; vi[nn] = si;
        }
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          R wr = 0, wi = 0;
#pragma unroll
          for (int nn = 0; nn < 3; ++nn) {
            const R nr = gt[(2 * (l + 3 * nn)) * g.Nh + gi], ni = gt[(2 * (l + 3 * nn) + 1) * g.Nh + gi];
            wr += nr * vr[nn] - ni * vi[nn];
            wi += nr * vi[nn] + ni * vr[nn];
          }
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const R xr = (R)xi[m].x, xim = (R)xi[m].y;
            out[l + 3 * m].x = xr * wr - xim * wi;
            out[l + 3 * m].y = xr * wi + xim * wr;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 9; ++c) other[((long)c * ti + i) * g.N2 + z] = out[c];
    }
  }
  if (ga.do_div) {
    // one partial per frequency line (x-frequency i, y): the z sum in a fixed order that
    // does not depend on the tile shape, so tile choices never change the result
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int line = threadIdx.x >> 5; line < ti; line += nw) {
      double v = 0.0;
      for (int z = lane; z < g.N2; z += 32) v += s_val[line * g.N2 + z];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) ga.div_part[(long long)y * g.N0r + i0 + line] = v;
    }
  }
  if (!ga.do_gamma) {
    if (ga.store_fwd)
      for (int t = threadIdx.x; t < 9 * ti * g.N2; t += blockDim.x) {
        int c = t / (ti * g.N2), rem = t - c * ti * g.N2;
        int z = rem / ti, i = rem - z * ti;
        spec[c * g.Nh + z * zs + (long long)y * g.N0r + i0 + i] = res[((long)c * ti + i) * g.N2 + z];
      }
    return;
  }
  __syncthreads();
  C* res2 = block_fft<R>(other, res, 9 * ti, pz, +1);
  for (int t = threadIdx.x; t < 9 * ti * g.N2; t += blockDim.x) {
    int c = t / (ti * g.N2), rem = t - c * ti * g.N2;
    int z = rem / ti, i = rem - z * ti;
    spec[c * g.Nh + z * zs + (long long)y * g.N0r + i0 + i] = res2[((long)c * ti + i) * g.N2 + z];
  }
}

// ---------------------------------------------------------------- coordinates
// per half-spectrum frequency: u^ = F^ xi2nd / sum conj(-xi2nd) xi2nd, zero at the zero
// frequency (whose real part gives Favg) and where xi2nd = 0; components 3..8 cleared.
// Continuous and central derivative: xi2nd = i a purely imaginary, u^_l = -i (F^ a)_l / |a|^2;
// FWBW: xi2nd complex from the per-axis factor tables (ga.fw), u^_l = -(F^ xi)_l / |xi|^2.
template <typename R>
__global__ void k_coords_freq(SpecGeom g, typename cpx<R>::t* __restrict__ spec, double s0, double s1, double s2,
                              int derivative, GammaArgs ga, double wgt, double* __restrict__ Favg) {
  typedef typename cpx<R>::t C;
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (f >= g.Nh) return;
  const double TAU = 6.283185307179586476925286766559;
  const int i = (int)(f % g.N0r);
  const long long yz = f / g.N0r;
  const int y = (int)(yz % g.N1), z = (int)(yz / g.N1);
  C Fh[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) Fh[c] = spec[c * g.Nh + f];
  if (f == 0) {
#pragma unroll
    for (int c = 0; c < 9; ++c) Favg[c] = (double)Fh[c].x * wgt;
  }
  C out[3];
  if (derivative == 2) {
    double2 xi[3];
    fw_xi(ga, i, y, z, xi);
    const double a2 = xi[0].x * xi[0].x + xi[0].y * xi[0].y + xi[1].x * xi[1].x + xi[1].y * xi[1].y +
                      xi[2].x * xi[2].x + xi[2].y * xi[2].y;
    const bool zero = (f == 0) || !(a2 > 0.0);
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double nr = 0.0, ni = 0.0;
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const double fr = (double)Fh[l + 3 * m].x, fi = (double)Fh[l + 3 * m].y;
        nr += fr * xi[m].x - fi * xi[m].y;
        ni += fr * xi[m].y + fi * xi[m].x;
      }
      out[l].x = zero ? (R)0 : (R)(-nr / a2);
      out[l].y = zero ? (R)0 : (R)(-ni / a2);
    }
  } else {
    const int k[3] = {i, y > g.N1 / 2 ? y - g.N1 : y, z > g.N2 / 2 ? z - g.N2 : z};
    const int n[3] = {g.N0, g.N1, g.N2};
    const double sz[3] = {s0, s1, s2};
    double a[3], a2 = 0.0;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      a[p] = derivative == 0 ? TAU * k[p] / sz[p] : sin(TAU * k[p] / n[p]) / (2.0 * sz[p] / n[p]);
      a2 += a[p] * a[p];
    }
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double nr = 0.0, ni = 0.0;
#pragma unroll
      for (int m = 0; m < 3; ++m) { nr += (double)Fh[l + 3 * m].x * a[m]; ni += (double)Fh[l + 3 * m].y * a[m]; }
      // -i (nr + i ni) / a2 = (ni - i nr) / a2
      bool zero = (f == 0) || !(a2 > 0.0);
      out[l].x = zero ? (R)0 : (R)(ni / a2);
      out[l].y = zero ? (R)0 : (R)(-nr / a2);
    }
  }
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    C v; v.x = 0; v.y = 0;
    if (c < 3) v = out[c];
    spec[c * g.Nh + f] = v;
  }
}

// cell-centre and nodal displacements from the fluctuation planes ut (wgt applied here)
__global__ void k_coords_out(SpecGeom g, const double* __restrict__ ut, long long ld, double wgt, const double* Favg,
                             double st0, double st1, double st2, double* __restrict__ u_n, double* __restrict__ u_p) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long Nn = (long long)(g.N0 + 1) * (g.N1 + 1) * (g.N2 + 1);
  double F[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) F[c] = Favg[c];
  const double step[3] = {st0, st1, st2};
  if (t < g.N) {
    const int x = (int)(t % g.N0);
    const long long yz = t / g.N0;
    const int y = (int)(yz % g.N1), z = (int)(yz / g.N1);
    const double pos[3] = {(x + 0.5) * step[0], (y + 0.5) * step[1], (z + 0.5) * step[2]};
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double v = ut[l * ld + t] * wgt;
#pragma unroll
      for (int m = 0; m < 3; ++m) v += F[l + 3 * m] * pos[m];
      u_p[3 * t + l] = v - pos[l];
    }
  }
  if (t < Nn) {
    const int x = (int)(t % (g.N0 + 1));
    const long long yz = t / (g.N0 + 1);
    const int y = (int)(yz % (g.N1 + 1)), z = (int)(yz / (g.N1 + 1));
    const double pos[3] = {x * step[0], y * step[1], z * step[2]};
    double v[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      v[l] = 0.0;
#pragma unroll
      for (int m = 0; m < 3; ++m) v[l] += F[l + 3 * m] * pos[m];
    }
    for (int dz = 0; dz < 2; ++dz)
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const int cx = (x + dx - 1 + g.N0) % g.N0, cy = (y + dy - 1 + g.N1) % g.N1, cz = (z + dz - 1 + g.N2) % g.N2;
          const long long e = cx + (long long)g.N0 * (cy + (long long)g.N1 * cz);
#pragma unroll
          for (int l = 0; l < 3; ++l) v[l] += ut[l * ld + e] * wgt * 0.125;
        }
#pragma unroll
    for (int l = 0; l < 3; ++l) u_n[3 * t + l] = v[l] - pos[l];
  }
}

__global__ void k_div_finish(const double* __restrict__ part, int nb, double wgt, int N0, double* out,
                             const SpecItem* __restrict__ items) {
  if (items) { part = items[blockIdx.x].div_part; out = items[blockIdx.x].rms; }
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) s += part[b];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) {
    double r = sqrt(s) * wgt;
    if (N0 == 1) r = r / 2.0;
    *out = r;
  }
}

}  // namespace dgx

// ------------------------------------------------------------------ host side
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace dgx {

void twiddle(long j, long n, double* c, double* s) {
  // cos/sin of 2 pi j / n, argument reduced to the first octant (quarter turns exact)
  const double TAU = 6.283185307179586476925286766559;
  j %= n; if (j < 0) j += n;
  long q = (4 * j) / n, r = 4 * j - q * n;
  double c0, s0;
  if (r == 0) { c0 = 1.0; s0 = 0.0; }
  else if (2 * r <= n) { double a = (TAU / 4.0) * ((double)r / (double)n); c0 = std::cos(a); s0 = std::sin(a); }
  else { double a = (TAU / 4.0) * ((double)(n - r) / (double)n); c0 = std::sin(a); s0 = std::cos(a); }
  switch (q) {
    case 0: *c = c0; *s = s0; break;
    case 1: *c = -s0; *s = c0; break;
    case 2: *c = -c0; *s = -s0; break;
    default: *c = s0; *s = -c0; break;
  }
}


int factorize(int n, int* rad) {
  int ns = 0, m = n;
  while (m % 4 == 0 && ns < 16) { rad[ns++] = 4; m /= 4; }
  while (m % 2 == 0 && ns < 16) { rad[ns++] = 2; m /= 2; }
  for (int r = 3; m > 1 && ns < 16; r += 2)
    while (m % r == 0 && ns < 16) { rad[ns++] = r; m /= r; }
  return m == 1 ? ns : -1;
}

void axis_tables(int n, std::vector<double2>& tw, std::vector<float2>& twf) {
  tw.resize(n);
  twf.resize(n);
  for (int j = 0; j < n; ++j) {
    double c, s;
    twiddle(j, n, &c, &s);
    tw[j] = make_double2(c, -s);
    twf[j] = make_float2((float)c, (float)-s);
  }
}

bool axis_plan(int n, AxisPlan* p) {
  p->n = n;
  p->nstages = factorize(n, p->radix);
  p->tw = nullptr;
  p->twf = nullptr;
  return p->nstages >= 0;
}

bool axis_create(AxisHost* ax, int n) {
  if (!axis_plan(n, &ax->plan)) return false;
  std::vector<double2> tw;
  std::vector<float2> twf;
  axis_tables(n, tw, twf);
  if (cudaMalloc(&ax->d_tw, sizeof(double2) * n) != cudaSuccess) return false;
  if (cudaMalloc(&ax->d_twf, sizeof(float2) * n) != cudaSuccess) return false;
  if (cudaMemcpy(ax->d_tw, tw.data(), sizeof(double2) * n, cudaMemcpyHostToDevice) != cudaSuccess) return false;
  if (cudaMemcpy(ax->d_twf, twf.data(), sizeof(float2) * n, cudaMemcpyHostToDevice) != cudaSuccess) return false;
  ax->plan.tw = ax->d_tw;
  ax->plan.twf = ax->d_twf;
  return true;
}

void scaled_geometry(const int cells[3], const double size[3], int divergence_correction, double out[3]) {
  // MechBase::base_init (mech_base.cpp:11-43): 1 size, 2 size + grid, else none
  int idx[3] = {0, 1, 2};
  const int dc = divergence_correction;
  if (dc == 1 || dc == 2) {
    double key[3];
    for (int i = 0; i < 3; ++i) key[i] = dc == 1 ? size[i] : size[i] / (double)cells[i];
    for (int a = 1; a < 3; ++a)
      for (int b = a; b > 0 && key[idx[b]] < key[idx[b - 1]]; --b) std::swap(idx[b], idx[b - 1]);
    for (int j = 0; j < 3; ++j) out[j] = dc == 1 ? size[j] / size[idx[1]] : size[j] / size[idx[1]] * cells[idx[1]];
  } else {
    for (int j = 0; j < 3; ++j) out[j] = size[j];
  }
}

void xi_axis(int axis, const int cells[3], const double size[3], int derivative, std::vector<double>& v) {
  // imaginary part of xi1st along one axis (Spectral::init / get_freq_derivative,
  // spectral.cpp:53-130): continuous 2 pi k / size with the Nyquist frequency zeroed
  // (per component), central difference sin(2 pi k / n) / (2 size / n); x holds the
  // N0/2+1 non-negative frequencies, y and z all n in FFT order
  const double TAU = 6.283185307179586476925286766559;
  const int n = cells[axis];
  const int len = axis == 0 ? n / 2 + 1 : n;
  v.resize(len);
  for (int i = 0; i < len; ++i) {
    const int k = axis == 0 ? i : (i > n / 2 ? i - n : i);
    const double val = derivative == 0 ? TAU * k / size[axis] : std::sin(TAU * k / n) / (2.0 * size[axis] / n);
    const bool nyq = (n % 2 == 0) && (i == n / 2) && derivative == 0;
    v[i] = nyq ? 0.0 : val;
  }
}

void axis_destroy(AxisHost* ax) {
  if (ax->d_tw) cudaFree(ax->d_tw);
  if (ax->d_twf) cudaFree(ax->d_twf);
  ax->d_tw = nullptr; ax->d_twf = nullptr;
}


SpecLaunch spec_launch_tiles(int N0, int N1, int N2, size_t csize, int LX, int TIy, int TIz) {
  SpecLaunch L;
  L.g.N0 = N0; L.g.N1 = N1; L.g.N2 = N2; L.g.N0r = N0 / 2 + 1;
  L.g.N = (long long)N0 * N1 * N2;
  L.g.Nh = (long long)L.g.N0r * N1 * N2;
  // x lines are transformed in pairs (2m, 2m + 1) of the global line index; an even
  // number of lines per block keeps every pair inside one block for any tile choice, so
  // the results do not depend on LX
  L.LX = std::max(2, LX + (LX & 1));
  L.TIy = std::max(1, std::min(TIy, L.g.N0r));
  L.TIz = std::max(1, std::min(TIz, L.g.N0r));
  // x passes: two real lines per complex line (np = ceil(LX / 2)): ping-pong buffers of
  // np lines, plus the inverse pass's staging of the LX half spectra
  L.smx = (2 * (size_t)((L.LX + 1) / 2) * N0 + (size_t)L.LX * L.g.N0r) * csize;
  L.smy = 2 * (size_t)L.TIy * N1 * csize;
  L.smz = 2 * 9 * (size_t)L.TIz * N2 * csize + (size_t)L.TIz * N2 * sizeof(double);
  long long nlines = 9LL * N1 * N2;
  L.nbx = (int)((nlines + L.LX - 1) / L.LX);
  L.nby = ((L.g.N0r + L.TIy - 1) / L.TIy) * 9 * N2;
  L.nbz = ((L.g.N0r + L.TIz - 1) / L.TIz) * N1;
  L.ndiv = L.g.N0r * N1;
  return L;
}

// opt-in shared memory per block of the current device (queried once per device)
static std::mutex g_dev_mu;
static std::map<int, size_t> g_smem_optin;

size_t smem_optin_limit() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 48 * 1024;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  auto it = g_smem_optin.find(dev);
  if (it != g_smem_optin.end()) return it->second;
  int v = 0;
  size_t lim = 48 * 1024;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && v > 0) lim = (size_t)v;
  g_smem_optin[dev] = lim;
  return lim;
}

bool spec_launch_fits(const SpecLaunch& L) {
  const size_t mx = smem_optin_limit();
  return L.smx <= mx && L.smy <= mx && L.smz <= mx;
}

SpecLaunch spec_launch(int N0, int N1, int N2, size_t csize) {
  int LX = N0 >= 256 ? 1 : 256 / N0;
  int TIy = N1 >= 256 ? 1 : 256 / N1;
  int TIz = N2 >= 256 ? 1 : 256 / N2;
  TIz = std::min(TIz, N0 / 2 + 1);
  // keep the z-pass tile within 200 KB of shared memory (9 components x 2 buffers)
  while (TIz > 1 && (2 * 9 * (size_t)TIz * N2 * csize + (size_t)TIz * N2 * 8) > 200 * 1024) TIz /= 2;
  return spec_launch_tiles(N0, N1, N2, csize, LX, TIy, TIz);
}

// The dynamic shared-memory limit is a property of the kernel on one device, shared by
// every RVE on that device: raise it to the largest request seen so far on the current
// device (never lower it, or an RVE created earlier with a larger grid could no longer
// launch).  Limits are kept per device and per precision, under a lock (RVEs may be
// created from several host threads).
template <typename R>
static bool set_smem_limits(const SpecLaunch& L) {
  static std::map<int, std::array<size_t, 3>> lim;   // device -> x, y, z pass limits
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  std::array<size_t, 3>& m = lim[dev];
  bool ok = true;
  if (L.smz > m[2]) {
    ok &= cudaFuncSetAttribute(k_zpass<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smz) == cudaSuccess;
    ok &= cudaFuncSetAttribute(k_zpass<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smz) == cudaSuccess;
    if (ok) m[2] = L.smz;
  }
  if (L.smy > m[1]) {
    ok &= cudaFuncSetAttribute(k_ypass<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smy) == cudaSuccess;
    if (ok) m[1] = L.smy;
  }
  if (L.smx > m[0]) {
    ok &= cudaFuncSetAttribute(k_xfwd<R, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smx) == cudaSuccess;
    ok &= cudaFuncSetAttribute(k_xinv<R, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smx) == cudaSuccess;
    if (ok) m[0] = L.smx;
  }
  return ok;
}

bool spec_prepare(const SpecLaunch& L, bool fp32) {
  if (!spec_launch_fits(L)) return false;
  return fp32 ? set_smem_limits<float>(L) : set_smem_limits<double>(L);
}

// full convolution of 9 real planes: forward x, y, z passes, div-RMS partials and
// Gamma in the z pass, inverse y and x passes.  items == null: one RVE (in, field,
// spec, ga as given); otherwise nitems RVEs of the same grid, one per blockIdx.y.
template <typename R>
static void convolve_impl(const SpecLaunch& L, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                          const double* in, double* field, long long ld, void* spec, const GammaArgs& ga,
                          const SpecItem* items, int nitems, cudaStream_t st) {
  typedef typename cpx<R>::t C;
  const unsigned ny = items ? (unsigned)nitems : 1u;
  k_xfwd<R, double><<<dim3(L.nbx, ny), 256, L.smx, st>>>(L.g, px, in, ld, (C*)spec, L.LX, items);
  k_ypass<R><<<dim3(L.nby, ny), 256, L.smy, st>>>(L.g, py, (C*)spec, L.TIy, -1, items);
  if (ga.fw[0]) k_zpass<R, true><<<dim3(L.nbz, ny), 256, L.smz, st>>>(L.g, pz, (C*)spec, L.TIz, ga, items);
  else k_zpass<R, false><<<dim3(L.nbz, ny), 256, L.smz, st>>>(L.g, pz, (C*)spec, L.TIz, ga, items);
  if (ga.do_gamma) {
    k_ypass<R><<<dim3(L.nby, ny), 256, L.smy, st>>>(L.g, py, (C*)spec, L.TIy, +1, items);
    k_xinv<R, double><<<dim3(L.nbx, ny), 256, L.smx, st>>>(L.g, px, (const C*)spec, field, ld, L.LX, items);
  }
}

void spec_convolve(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                   const double* in, double* field, long long ld, void* spec, const GammaArgs& ga, cudaStream_t st) {
  if (fp32) convolve_impl<float>(L, px, py, pz, in, field, ld, spec, ga, nullptr, 1, st);
  else convolve_impl<double>(L, px, py, pz, in, field, ld, spec, ga, nullptr, 1, st);
}

void spec_convolve_batch(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                         const SpecItem* items, int nitems, const GammaArgs& ga, cudaStream_t st) {
  if (fp32) convolve_impl<float>(L, px, py, pz, nullptr, nullptr, L.g.N, nullptr, ga, items, nitems, st);
  else convolve_impl<double>(L, px, py, pz, nullptr, nullptr, L.g.N, nullptr, ga, items, nitems, st);
}

void spec_update_coords(const SpecLaunch& L, bool fp32, const AxisPlan& px, const AxisPlan& py, const AxisPlan& pz,
                        const double* F, long long ld, void* spec, double* scratch, const double size[3],
                        int derivative, const GammaArgs& xi, double wgt, double* Favg, double* u_n, double* u_p,
                        cudaStream_t st) {
  GammaArgs ga{};
  ga.store_fwd = 1; ga.zsign = -1;
  const SpecGeom& g = L.g;
  const long long Nn = (long long)(g.N0 + 1) * (g.N1 + 1) * (g.N2 + 1);
  const int nbf = (int)((g.Nh + 255) / 256), nbo = (int)((std::max(g.N, Nn) + 255) / 256);
  if (fp32) {
    typedef float2 C;
    convolve_impl<float>(L, px, py, pz, F, nullptr, ld, spec, ga, nullptr, 1, st);
    k_coords_freq<float><<<nbf, 256, 0, st>>>(g, (C*)spec, size[0], size[1], size[2], derivative, xi, wgt, Favg);
    ga.zsign = +1;
    k_zpass<float, false><<<L.nbz, 256, L.smz, st>>>(g, pz, (C*)spec, L.TIz, ga, nullptr);
    k_ypass<float><<<L.nby, 256, L.smy, st>>>(g, py, (C*)spec, L.TIy, +1, nullptr);
    k_xinv<float, double><<<L.nbx, 256, L.smx, st>>>(g, px, (const C*)spec, scratch, ld, L.LX, nullptr);
  } else {
    typedef double2 C;
    convolve_impl<double>(L, px, py, pz, F, nullptr, ld, spec, ga, nullptr, 1, st);
    k_coords_freq<double><<<nbf, 256, 0, st>>>(g, (C*)spec, size[0], size[1], size[2], derivative, xi, wgt, Favg);
    ga.zsign = +1;
    k_zpass<double, false><<<L.nbz, 256, L.smz, st>>>(g, pz, (C*)spec, L.TIz, ga, nullptr);
    k_ypass<double><<<L.nby, 256, L.smy, st>>>(g, py, (C*)spec, L.TIy, +1, nullptr);
    k_xinv<double, double><<<L.nbx, 256, L.smx, st>>>(g, px, (const C*)spec, scratch, ld, L.LX, nullptr);
  }
  k_coords_out<<<nbo, 256, 0, st>>>(g, scratch, ld, wgt, Favg, size[0] / g.N0, size[1] / g.N1, size[2] / g.N2, u_n,
                                    u_p);
}

size_t gamma_table_bytes(const SpecGeom& g, bool fp32, bool fwbw) {
  return (size_t)gtab_entries(fp32, fwbw) * (size_t)g.Nh * (fp32 ? sizeof(float) : sizeof(double));
}

void gamma_table(const SpecGeom& g, bool fp32, const GammaArgs& ga, void* gtab, cudaStream_t st) {
  const int nb = (int)((g.Nh + 255) / 256);
  const bool fw = ga.fw[0] != nullptr;
  if (fp32) {
    if (fw) k_gamma_table<float, true><<<nb, 256, 0, st>>>(g, ga, (float*)gtab);
    else k_gamma_table<float, false><<<nb, 256, 0, st>>>(g, ga, (float*)gtab);
  } else {
    if (fw) k_gamma_table<double, true><<<nb, 256, 0, st>>>(g, ga, (double*)gtab);
    else k_gamma_table<double, false><<<nb, 256, 0, st>>>(g, ga, (double*)gtab);
  }
}

void fw_axis(int axis, const int cells[3], std::vector<double>& v) {
  // D = e^(i theta) - 1, E = e^(i theta) + 1, theta = 2 pi k / n (k in FFT order), the
  // factors of the reference's forward/backward difference (spectral.cpp:115-124);
  // cos / sin exact at quarter turns, where D or E vanishes (and xi with it)
  const double TAU = 6.283185307179586476925286766559;
  const int n = cells[axis];
  const int len = axis == 0 ? n / 2 + 1 : n;
  v.assign(4 * (size_t)len, 0.0);
  for (int i = 0; i < len; ++i) {
    const int k = axis == 0 ? i : (i > n / 2 ? i - n : i);
    double c, s;
    if ((4L * k) % n == 0) {
      long quarter = ((4L * k) / n) % 4;
      if (quarter < 0) quarter += 4;
      const double cc[4] = {1.0, 0.0, -1.0, 0.0}, ss[4] = {0.0, 1.0, 0.0, -1.0};
      c = cc[quarter]; s = ss[quarter];
    } else {
      c = std::cos(TAU * k / n);
      s = std::sin(TAU * k / n);
    }
    v[4 * i] = c - 1.0; v[4 * i + 1] = s; v[4 * i + 2] = c + 1.0; v[4 * i + 3] = s;
  }
}

void spec_div_finish_batch(const SpecItem* items, int nitems, int nb, double wgt, int N0, cudaStream_t st) {
  k_div_finish<<<nitems, 32, 0, st>>>(nullptr, nb, wgt, N0, nullptr, items);
}

void spec_div_finish(const double* part, int nb, double wgt, int N0, double* out, cudaStream_t st) {
  k_div_finish<<<1, 32, 0, st>>>(part, nb, wgt, N0, out, nullptr);
}

}  // namespace dgx
