/*
 * dgo_spec.c -- oracle: FFT and spectral operators.
 * TEST INFRASTRUCTURE ONLY (see dgo.h).
 *
 * Follows (reference paths):
 *   src/grid/fft.cpp:17-78, fft.h:37-60   unnormalised r2c/c2r, transposed-out layout
 *   src/grid/spectral.cpp:53-130          xi1st/xi2nd (Nyquist zeroing per component, as
 *                                          src/grid/test/test_spectral.cpp:23-46 expects)
 *   src/grid/mech_base.cpp:11-43          divergence-correction scaled geometry
 *   src/grid/mech_base.cpp:302-398        divergence RMS (Hermitian half-spectrum weights)
 *   src/grid/mech_base.cpp:400-477 + 156-205  Gamma convolution (full operator; the
 *                                          C++ memory-efficient branch is a stub)
 *   src/grid/mech_base.cpp:213-300, 479-497   forward_field, masked compliance, rate
 *   src/grid/mech_solver_basic.cpp:321-334    residual BC part
 * The FFT is a plain mixed-radix Cooley-Tukey (radix 2,3,4,5 butterflies, any other
 * prime by a direct DFT), evaluated in FP64 with twiddles from cos/sin.
 */
#include "dgo.h"
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TAU 6.283185307179586476925286766559

typedef double complex cplx;

/* ------------------------------------------------------------------ 1-D FFT */
/* cos/sin of 2*pi*j/n with the argument reduced to the first octant, so that
 * quarter-turn multiples are exact (0, +-1) and cos/sin are mirror-consistent */
void dgo_twiddle(long j, long n, double* c, double* s) {
  j %= n; if (j < 0) j += n;
  long q = (4 * j) / n, r = 4 * j - q * n;       /* angle = (q + r/n) * pi/2 */
  double c0, s0;
  if (r == 0) { c0 = 1.0; s0 = 0.0; }
  else if (2 * r <= n) { double a = (TAU / 4.0) * ((double)r / (double)n); c0 = cos(a); s0 = sin(a); }
  else { double a = (TAU / 4.0) * ((double)(n - r) / (double)n); c0 = sin(a); s0 = cos(a); }
  switch (q) {
    case 0: *c = c0; *s = s0; break;
    case 1: *c = -s0; *s = c0; break;
    case 2: *c = -c0; *s = -s0; break;
    default: *c = s0; *s = -c0; break;
  }
}

typedef struct plan1 { int n; int nf; int f[32]; cplx* tw; } plan1;

static void plan_make(plan1* p, int n, int sign) {
  p->n = n; p->nf = 0;
  int m = n;
  while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
  for (int r = 3; m > 1; r += 2) while (m % r == 0) { p->f[p->nf++] = r; m /= r; }
  p->tw = (cplx*)malloc(sizeof(cplx) * (n > 0 ? n : 1));
  for (int j = 0; j < n; ++j) {
    double c, s;
    dgo_twiddle(j, n, &c, &s);
    p->tw[j] = c + sign * I * s;
  }
}
static void plan_free(plan1* p) { free(p->tw); }

/* y[k] = sum_j x[j*stride] w^(jk), w = tw[1] */
static void fft_rec(const plan1* p, int n, int level, const cplx* x, int stride, cplx* y, int twstep) {
  if (n == 1) { y[0] = x[0]; return; }
  int r = p->f[level], m = n / r;
  for (int q = 0; q < r; ++q) fft_rec(p, m, level + 1, x + q * stride, stride * r, y + q * m, twstep * r);
  cplx tbuf[64];
  cplx* t = r <= 64 ? tbuf : (cplx*)malloc(sizeof(cplx) * r);
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < r; ++q) t[q] = y[q * m + k] * p->tw[((long)q * k * twstep) % p->n];
    for (int s = 0; s < r; ++s) {
      cplx acc = 0;
      for (int q = 0; q < r; ++q) acc += t[q] * p->tw[((long)q * s * m * twstep) % p->n];
      y[s * m + k] = acc;
    }
  }
  if (t != tbuf) free(t);
}
static void fft_line(const plan1* p, cplx* line, cplx* work) {
  if (p->n <= 1) return;
  fft_rec(p, p->n, 0, line, 1, work, 1);
  memcpy(line, work, sizeof(cplx) * p->n);
}

/* ------------------------------------------------------------------ 3-D r2c / c2r */
void dgo_fft_r2c(const int cells[3], int ncomp, const double* field, double* spec_) {
  int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  cplx* spec = (cplx*)spec_;
  plan1 px, py, pz;
  plan_make(&px, N0, -1); plan_make(&py, N1, -1); plan_make(&pz, N2, -1);
  int L = N0 > N1 ? N0 : N1; if (N2 > L) L = N2;
  cplx* line = (cplx*)malloc(sizeof(cplx) * L);
  cplx* work = (cplx*)malloc(sizeof(cplx) * L);
  cplx* T = (cplx*)malloc(sizeof(cplx) * (size_t)N0r * N1 * N2);
  for (int c = 0; c < ncomp; ++c) {
    for (int z = 0; z < N2; ++z)
      for (int y = 0; y < N1; ++y) {
        for (int x = 0; x < N0; ++x) line[x] = field[c + ncomp * ((size_t)x + N0 * (y + (size_t)N1 * z))];
        fft_line(&px, line, work);
        for (int i = 0; i < N0r; ++i) T[i + (size_t)N0r * (y + (size_t)N1 * z)] = line[i];
      }
    for (int z = 0; z < N2; ++z)
      for (int i = 0; i < N0r; ++i) {
        for (int y = 0; y < N1; ++y) line[y] = T[i + (size_t)N0r * (y + (size_t)N1 * z)];
        fft_line(&py, line, work);
        for (int y = 0; y < N1; ++y) T[i + (size_t)N0r * (y + (size_t)N1 * z)] = line[y];
      }
    for (int y = 0; y < N1; ++y)
      for (int i = 0; i < N0r; ++i) {
        for (int z = 0; z < N2; ++z) line[z] = T[i + (size_t)N0r * (y + (size_t)N1 * z)];
        fft_line(&pz, line, work);
        for (int z = 0; z < N2; ++z) spec[c + ncomp * ((size_t)i + N0r * (z + (size_t)N2 * y))] = line[z];
      }
  }
  free(line); free(work); free(T);
  plan_free(&px); plan_free(&py); plan_free(&pz);
}

void dgo_fft_c2r(const int cells[3], int ncomp, const double* spec_, double* field) {
  int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  const cplx* spec = (const cplx*)spec_;
  plan1 px, py, pz;
  plan_make(&px, N0, +1); plan_make(&py, N1, +1); plan_make(&pz, N2, +1);
  int L = N0 > N1 ? N0 : N1; if (N2 > L) L = N2;
  cplx* line = (cplx*)malloc(sizeof(cplx) * L);
  cplx* work = (cplx*)malloc(sizeof(cplx) * L);
  cplx* T = (cplx*)malloc(sizeof(cplx) * (size_t)N0r * N1 * N2);
  for (int c = 0; c < ncomp; ++c) {
    for (int y = 0; y < N1; ++y)
      for (int i = 0; i < N0r; ++i) {
        for (int z = 0; z < N2; ++z) line[z] = spec[c + ncomp * ((size_t)i + N0r * (z + (size_t)N2 * y))];
        fft_line(&pz, line, work);
        for (int z = 0; z < N2; ++z) T[i + (size_t)N0r * (y + (size_t)N1 * z)] = line[z];
      }
    for (int z = 0; z < N2; ++z)
      for (int i = 0; i < N0r; ++i) {
        for (int y = 0; y < N1; ++y) line[y] = T[i + (size_t)N0r * (y + (size_t)N1 * z)];
        fft_line(&py, line, work);
        for (int y = 0; y < N1; ++y) T[i + (size_t)N0r * (y + (size_t)N1 * z)] = line[y];
      }
    for (int z = 0; z < N2; ++z)
      for (int y = 0; y < N1; ++y) {
        for (int i = 0; i < N0r; ++i) line[i] = T[i + (size_t)N0r * (y + (size_t)N1 * z)];
        for (int i = N0r; i < N0; ++i) line[i] = conj(line[N0 - i]);
        fft_line(&px, line, work);
        for (int x = 0; x < N0; ++x) field[c + ncomp * ((size_t)x + N0 * (y + (size_t)N1 * z))] = creal(line[x]);
      }
  }
  free(line); free(work); free(T);
  plan_free(&px); plan_free(&py); plan_free(&pz);
}

/* ------------------------------------------------------------------ xi */
/* cos/sin of 2 pi k / n for the forward/backward difference: exact at quarter turns
 * (k / n a multiple of 1/4), where the factors e^(i theta) +- 1 vanish and xi with them;
 * cos(2 pi k / n), sin(2 pi k / n) otherwise */
static void fw_trig(int k, int n, double* c, double* s) {
  long q4 = (4L * k) % n;
  if (q4 == 0) {
    long quarter = ((4L * k) / n) % 4;
    if (quarter < 0) quarter += 4;
    const double cc[4] = {1.0, 0.0, -1.0, 0.0}, ss[4] = {0.0, 1.0, 0.0, -1.0};
    *c = cc[quarter]; *s = ss[quarter];
    return;
  }
  *c = cos(TAU * k / n);
  *s = sin(TAU * k / n);
}

static void freq_derivative(int derivative, const int cells[3], const double geom[3], const int ks[3], cplx out[3]) {
  for (int i = 0; i < 3; ++i) {
    switch (derivative) {
      case DGO_DERIV_CONTINUOUS:
        out[i] = I * (TAU * ks[i] / geom[i]);
        break;
      case DGO_DERIV_CENTRAL:
        out[i] = (I * sin(TAU * ks[i] / cells[i])) / (2.0 * geom[i] / cells[i]);
        break;
      default: {  /* forward/backward difference (spectral.cpp:115-124 spells the factors out; as
                     written there the statement ends in a comma operator and yields zero) */
        int j = (i + 1) % 3, k = (i + 2) % 3;
        double ci, si, cj, sj, ck, sk;
        fw_trig(ks[i], cells[i], &ci, &si);
        fw_trig(ks[j], cells[j], &cj, &sj);
        fw_trig(ks[k], cells[k], &ck, &sk);
        cplx a = (ci - 1.0) + I * si;
        cplx b = (cj + 1.0) + I * sj;
        cplx c = (ck + 1.0) + I * sk;
        out[i] = a * b * c / (4.0 * geom[i] / cells[i]);
      }
    }
  }
}

void dgo_xi(const int cells[3], const double geom[3], int derivative, double* xi1st_, double* xi2nd_) {
  int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  cplx* xi1st = (cplx*)xi1st_;
  cplx* xi2nd = (cplx*)xi2nd_;
  for (int j = 0; j < N1; ++j) {
    int ky = j > N1 / 2 ? j - N1 : j;
    for (int k = 0; k < N2; ++k) {
      int kz = k > N2 / 2 ? k - N2 : k;
      for (int i = 0; i < N0r; ++i) {
        int ks[3] = {i, ky, kz};
        cplx fd[3];
        freq_derivative(derivative, cells, geom, ks, fd);
        size_t base = 3 * ((size_t)i + N0r * (k + (size_t)N2 * j));
        int idx[3] = {i, j, k};
        for (int p = 0; p < 3; ++p) {
          if (xi2nd) xi2nd[base + p] = fd[p];
          int nyq = (cells[p] % 2 == 0) && (idx[p] == cells[p] / 2) && derivative == DGO_DERIV_CONTINUOUS;
          xi1st[base + p] = nyq ? 0.0 : fd[p];
        }
      }
    }
  }
}

void dgo_scaled_geom(const int cells[3], const double geom[3], int divcorr, double out[3]) {
  int idx[3] = {0, 1, 2};
  if (divcorr == DGO_DIVCORR_SIZE || divcorr == DGO_DIVCORR_SIZE_GRID) {
    double key[3];
    for (int i = 0; i < 3; ++i) key[i] = divcorr == DGO_DIVCORR_SIZE ? geom[i] : geom[i] / (double)cells[i];
    /* stable insertion sort by key */
    for (int a = 1; a < 3; ++a)
      for (int b = a; b > 0 && key[idx[b]] < key[idx[b - 1]]; --b) { int t = idx[b]; idx[b] = idx[b - 1]; idx[b - 1] = t; }
    for (int j = 0; j < 3; ++j)
      out[j] = divcorr == DGO_DIVCORR_SIZE ? geom[j] / geom[idx[1]]
                                           : geom[j] / geom[idx[1]] * cells[idx[1]];
  } else {
    for (int j = 0; j < 3; ++j) out[j] = geom[j];
  }
}

double dgo_divergence_rms_spec(const int cells[3], const double geom[3], const double scaled[3],
                               const double* xi1st_, const double* spec_) {
  int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  const cplx* xi1st = (const cplx*)xi1st_;
  const cplx* spec = (const cplx*)spec_;
  double resc[3];
  for (int i = 0; i < 3; ++i) resc[i] = geom[i] / scaled[i];
  double rms = 0.0;
  for (int j = 0; j < N1; ++j)
    for (int k = 0; k < N2; ++k) {
      /* interior x frequencies (weight 2), then i = 0 and i = N0r-1 (weight 1) */
      for (int pass = 0; pass < 3; ++pass) {
        int ilo = pass == 0 ? 1 : (pass == 1 ? 0 : N0r - 1);
        int ihi = pass == 0 ? N0r - 1 : ilo + 1;
        for (int i = ilo; i < ihi; ++i) {
          size_t f = (size_t)i + N0r * (k + (size_t)N2 * j);
          cplx v[3];
          for (int n = 0; n < 3; ++n) v[n] = conj(-xi1st[3 * f + n]) * resc[n];
          double s = 0.0;
          for (int l = 0; l < 3; ++l) {
            cplx prod = 0;
            for (int n = 0; n < 3; ++n) prod += spec[9 * f + l + 3 * n] * v[n];
            s += creal(prod) * creal(prod) + cimag(prod) * cimag(prod);
          }
          rms += pass == 0 ? 2.0 * s : s;
        }
      }
    }
  double wgt = 1.0 / ((double)N0 * N1 * N2);
  rms = sqrt(rms) * wgt;
  if (N0 == 1) rms = rms / 2.0;
  return rms;
}

double dgo_divergence_rms(const int cells[3], const double geom[3], const double scaled[3],
                          const double* xi1st, const double* P) {
  size_t nh = (size_t)(cells[0] / 2 + 1) * cells[1] * cells[2];
  double* spec = (double*)malloc(sizeof(double) * 2 * 9 * nh);
  dgo_fft_r2c(cells, 9, P, spec);
  double r = dgo_divergence_rms_spec(cells, geom, scaled, xi1st, spec);
  free(spec);
  return r;
}

void dgo_gamma_convolution(const int cells[3], const double* xi1st_, const double C_ref[81],
                           const double aim[9], double* field) {
  int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  const cplx* xi1st = (const cplx*)xi1st_;
  size_t nh = (size_t)N0r * N1 * N2;
  cplx* spec = (cplx*)malloc(sizeof(cplx) * 9 * nh);
  dgo_fft_r2c(cells, 9, field, (double*)spec);
  for (size_t f = 0; f < nh; ++f) {
    if (f == 0) continue;                               /* singular point xi = 0 */
    const cplx* xi = xi1st + 3 * f;
    cplx dyad[9], K[9];
    for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) dyad[l + 3 * m] = conj(-xi[l]) * xi[m];
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < 3; ++m) {
        cplx s = 0;
        for (int n = 0; n < 3; ++n)
          for (int o = 0; o < 3; ++o) s += C_ref[l + 3 * n + 9 * m + 27 * o] * dyad[n + 3 * o];
        K[l + 3 * m] = s;
      }
    double A[36];
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < 3; ++m) {
        A[l + 6 * m] = creal(K[l + 3 * m]);
        A[(l + 3) + 6 * (m + 3)] = creal(K[l + 3 * m]);
        A[l + 6 * (m + 3)] = cimag(K[l + 3 * m]);
        A[(l + 3) + 6 * m] = -cimag(K[l + 3 * m]);
      }
    double Are[9];
    for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) Are[l + 3 * m] = A[l + 6 * m];
    double det = Are[0] * (Are[4] * Are[8] - Are[7] * Are[5]) - Are[3] * (Are[1] * Are[8] - Are[7] * Are[2])
               + Are[6] * (Are[1] * Are[5] - Are[4] * Are[2]);
    cplx out[9];
    if (fabs(det) > 1e-16) {
      double Ainv[36];
      dgo_invert(6, A, Ainv);
      cplx Kinv[9];
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) Kinv[l + 3 * m] = Ainv[l + 6 * m] + I * Ainv[(l + 3) + 6 * m];
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) {
          cplx s = 0;
          for (int n = 0; n < 3; ++n)
            for (int o = 0; o < 3; ++o) s += (Kinv[l + 3 * n] * dyad[o + 3 * m]) * spec[9 * f + n + 3 * o];
          out[l + 3 * m] = s;
        }
    } else {
      for (int k = 0; k < 9; ++k) out[k] = 0;
    }
    for (int k = 0; k < 9; ++k) spec[9 * f + k] = out[k];
  }
  for (int k = 0; k < 9; ++k) spec[k] = aim[k];
  dgo_fft_c2r(cells, 9, (const double*)spec, field);
  free(spec);
}

void dgo_forward_field(int64_t n, double dt, const double* last, const double* rate,
                       const double* aim, double* out) {
  for (int64_t e = 0; e < 9 * n; ++e) out[e] = last[e] + rate[e] * dt;
  if (aim) {
    double diff[9];
    for (int k = 0; k < 9; ++k) {
      double s = 0.0;
      for (int64_t e = 0; e < n; ++e) s += out[9 * e + k];
      diff[k] = s * (1.0 / (double)n) - aim[k];
    }
    for (int64_t e = 0; e < n; ++e)
      for (int k = 0; k < 9; ++k) out[9 * e + k] -= diff[k];
  }
}

void dgo_calculate_rate(int64_t n, int heterogeneous, const double* field0, const double* field,
                        double dt, const double avRate[9], double* rate) {
  for (int64_t e = 0; e < n; ++e)
    for (int k = 0; k < 9; ++k)
      rate[9 * e + k] = heterogeneous ? (field[9 * e + k] - field0[9 * e + k]) / dt : avRate[k];
}

/* mask_stress: column-major, 1 = not prescribed; the 9-vector follows the
 * row-major MAPPLAIN order of the 9x9 stiffness (Fortran: reshape(transpose(mask))) */
int dgo_masked_compliance(const double C[81], const double q[4], const int mask_stress[9], double S[81]) {
  int act[9], nred = 0;
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) { act[3 * a + b] = !mask_stress[a + 3 * b]; nred += act[3 * a + b]; }
  double t99[81];
  memset(t99, 0, sizeof(t99));
  int err = 0;
  if (nred > 0) {
    double rot[81], c99[81], cred[81], sred[81];
    dgo_rotate4(q, C, rot, 0);
    dgo_3333to99(rot, c99);
    int idx = 0;
    for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
      if (act[i] && act[j]) { cred[(idx / nred) + nred * (idx % nred)] = c99[i + 9 * j]; ++idx; }
    err = dgo_invert(nred, cred, sred);
    idx = 0;
    for (int i = 0; i < 9; ++i) for (int j = 0; j < 9; ++j)
      if (act[i] && act[j]) { t99[i + 9 * j] = sred[(idx / nred) + nred * (idx % nred)]; ++idx; }
  }
  dgo_99to3333(t99, S);
  return err;
}

double dgo_form_residual_bc(const double S[81], const double P_av[9], const double P_aim[9],
                            const int stress_mask[9], const double q[4], double F_aim[9], double rotated[9]) {
  double dF[9];
  dgo_mul3333xx33(S, P_av, dF);
  for (int k = 0; k < 9; ++k) F_aim[k] -= dF[k];
  double err = 0.0;
  for (int k = 0; k < 9; ++k) {
    double e = stress_mask[k] ? 0.0 : fabs(P_av[k] - P_aim[k]);
    if (e > err) err = e;
  }
  dgo_rotate2(q, dF, rotated, 1);
  return err;
}

/* ------------------------------------------------------------------ coordinates
 * Cell-centre and nodal displacements of the deformed grid (the grid solver's
 * coordinate update; reference src/grid/mech_base.cpp:45-154, with the cell-centre
 * positions x_p = u~ + Favg (i + 1/2) step of the Fortran grid solver that wrote the
 * reference's DADF5 results).  F: 9 per cell (column-major 3x3), cells x fastest.
 * u_p[3*cell + k] = x_p - (i + 1/2) step ; u_n[3*node + k] = x_n - i step, nodes
 * (N0+1)(N1+1)(N2+1) x fastest.  Fluctuation: u~^(xi) = F^(xi) xi / sum conj(-xi) xi
 * with xi = xi2nd, zero at xi = 0, backward FFT times wgt. */
void dgo_update_coords(const int cells[3], const double geom[3], int derivative, const double* F,
                       double* u_n, double* u_p) {
  const int N0 = cells[0], N1 = cells[1], N2 = cells[2], N0r = N0 / 2 + 1;
  const size_t N = (size_t)N0 * N1 * N2, Nh = (size_t)N0r * N1 * N2;
  const double wgt = pow((double)N, -1.0);
  cplx* Fh = (cplx*)malloc(sizeof(cplx) * 9 * Nh);
  cplx* uh = (cplx*)malloc(sizeof(cplx) * 3 * Nh);
  cplx* x1 = (cplx*)malloc(sizeof(cplx) * 3 * Nh);
  cplx* x2 = (cplx*)malloc(sizeof(cplx) * 3 * Nh);
  double* ut = (double*)malloc(sizeof(double) * 3 * N);
  dgo_fft_r2c(cells, 9, F, (double*)Fh);
  dgo_xi(cells, geom, derivative, (double*)x1, (double*)x2);
  double Favg[9];
  for (int c = 0; c < 9; ++c) Favg[c] = creal(Fh[c]) * wgt;          /* zero frequency, (i,z,y) = 0 */
  for (size_t f = 0; f < Nh; ++f) {
    const cplx* xi = x2 + 3 * f;
    if (f == 0) { uh[0] = uh[1] = uh[2] = 0.0; continue; }
    cplx den = 0.0;
    for (int m = 0; m < 3; ++m) den += conj(-xi[m]) * xi[m];
    if (den == 0.0) { uh[3 * f] = uh[3 * f + 1] = uh[3 * f + 2] = 0.0; continue; }   /* xi = 0: no fluctuation */
    for (int l = 0; l < 3; ++l) {
      cplx s = 0.0;
      for (int m = 0; m < 3; ++m) s += Fh[9 * f + l + 3 * m] * xi[m];
      uh[3 * f + l] = s / den;
    }
  }
  dgo_fft_c2r(cells, 3, (const double*)uh, ut);
  for (size_t k = 0; k < 3 * N; ++k) ut[k] *= wgt;
  const double step[3] = {geom[0] / N0, geom[1] / N1, geom[2] / N2};
  for (int z = 0; z < N2; ++z)
    for (int y = 0; y < N1; ++y)
      for (int x = 0; x < N0; ++x) {
        size_t e = (size_t)x + N0 * ((size_t)y + N1 * z);
        double pos[3] = {(x + 0.5) * step[0], (y + 0.5) * step[1], (z + 0.5) * step[2]};
        for (int l = 0; l < 3; ++l) {
          double v = ut[3 * e + l];
          for (int m = 0; m < 3; ++m) v += Favg[l + 3 * m] * pos[m];
          u_p[3 * e + l] = v - pos[l];
        }
      }
  for (int z = 0; z <= N2; ++z)
    for (int y = 0; y <= N1; ++y)
      for (int x = 0; x <= N0; ++x) {
        size_t nd = (size_t)x + (N0 + 1) * ((size_t)y + (N1 + 1) * z);
        double pos[3] = {x * step[0], y * step[1], z * step[2]};
        double v[3];
        for (int l = 0; l < 3; ++l) {
          v[l] = 0.0;
          for (int m = 0; m < 3; ++m) v[l] += Favg[l + 3 * m] * pos[m];
        }
        for (int dz = 0; dz < 2; ++dz)
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
              int cx = (x + dx - 1 + N0) % N0, cy = (y + dy - 1 + N1) % N1, cz = (z + dz - 1 + N2) % N2;
              size_t e = (size_t)cx + N0 * ((size_t)cy + N1 * cz);
              for (int l = 0; l < 3; ++l) v[l] += ut[3 * e + l] * 0.125;
            }
        for (int l = 0; l < 3; ++l) u_n[3 * nd + l] = v[l] - pos[l];
      }
  free(Fh); free(uh); free(x1); free(x2); free(ut);
}
