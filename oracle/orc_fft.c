/*
 * Oracle FFTs (test infrastructure only).
 *
 * Restates the transforms the reference obtains from FFTW-MPI
 * (src/wrappers.c:26-96: fftw_mpi_plan_dft_r2c_3d / _c2r_3d on a
 * [N][N][2(N/2+1)] padded grid, unnormalised).  Written from the textbook
 * Cooley-Tukey radix-2 algorithm; lengths that are not powers of two go
 * through Bluestein's chirp-z identity on power-of-two sub-transforms.
 *
 * c2r semantics: complex inverse transforms along x and y for every kz in
 * [0, N/2], then a half-complex-to-real transform along z that uses only the
 * real parts of the kz = 0 and kz = N/2 entries.  This is the behaviour of a
 * real-output inverse DFT on data that is not exactly Hermitian.
 */
#include "orc.h"
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

typedef struct {
  int n, pow2, m;        /* m: Bluestein convolution length (pow2) */
  cplx *tw;              /* e^{-2 pi i k / L}, k < L/2, L = n (pow2) or m */
  int *rev;
  cplx *chirp;           /* Bluestein: w_k = e^{-i pi k^2 / n} */
  cplx *bfft;            /* FFT of the conjugate chirp, length m */
} plan1d;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static void make_radix2(int L, cplx **tw, int **rev) {
  *tw = malloc(sizeof(cplx) * (L / 2 > 0 ? L / 2 : 1));
  for (int k = 0; k < L / 2; k++) (*tw)[k] = cexp(-2.0 * M_PI * I * (double)k / (double)L);
  *rev = malloc(sizeof(int) * L);
  int bits = 0;
  while ((1 << bits) < L) bits++;
  for (int i = 0; i < L; i++) {
    int r = 0;
    for (int b = 0; b < bits; b++) if (i & (1 << b)) r |= 1 << (bits - 1 - b);
    (*rev)[i] = r;
  }
}

/* In-place radix-2 DIT, sign -1 uses tw, sign +1 uses conj(tw). */
static void radix2(cplx *a, int L, const cplx *tw, const int *rev, int sign) {
  for (int i = 0; i < L; i++) {
    int r = rev[i];
    if (r > i) { cplx t = a[i]; a[i] = a[r]; a[r] = t; }
  }
  for (int len = 2; len <= L; len <<= 1) {
    int half = len >> 1, step = L / len;
    for (int s = 0; s < L; s += len) {
      for (int k = 0; k < half; k++) {
        cplx w = tw[k * step];
        if (sign > 0) w = conj(w);
        cplx u = a[s + k], v = a[s + k + half] * w;
        a[s + k] = u + v;
        a[s + k + half] = u - v;
      }
    }
  }
}

static plan1d *plan_create(int n) {
  plan1d *p = calloc(1, sizeof(plan1d));
  p->n = n;
  p->pow2 = is_pow2(n);
  if (p->pow2) {
    make_radix2(n, &p->tw, &p->rev);
  } else {
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    p->m = m;
    make_radix2(m, &p->tw, &p->rev);
    p->chirp = malloc(sizeof(cplx) * n);
    for (int k = 0; k < n; k++) {
      /* k^2 mod 2n keeps the argument small */
      long kk = ((long)k * (long)k) % (2L * n);
      p->chirp[k] = cexp(-M_PI * I * (double)kk / (double)n);
    }
    p->bfft = calloc(m, sizeof(cplx));
    p->bfft[0] = conj(p->chirp[0]);
    for (int k = 1; k < n; k++) p->bfft[k] = p->bfft[m - k] = conj(p->chirp[k]);
    radix2(p->bfft, m, p->tw, p->rev, -1);
  }
  return p;
}

static void plan_free(plan1d *p) {
  if (!p) return;
  free(p->tw); free(p->rev); free(p->chirp); free(p->bfft); free(p);
}

/* work must hold p->m entries for Bluestein plans. */
static void exec1d(const plan1d *p, cplx *a, int sign, cplx *work) {
  if (p->pow2) { radix2(a, p->n, p->tw, p->rev, sign); return; }
  int n = p->n, m = p->m;
  /* sign +1 is the conjugate of the sign -1 transform of the conjugate. */
  for (int k = 0; k < n; k++) {
    cplx x = sign > 0 ? conj(a[k]) : a[k];
    work[k] = x * p->chirp[k];
  }
  for (int k = n; k < m; k++) work[k] = 0;
  radix2(work, m, p->tw, p->rev, -1);
  for (int k = 0; k < m; k++) work[k] *= p->bfft[k];
  radix2(work, m, p->tw, p->rev, +1);
  for (int k = 0; k < n; k++) {
    cplx y = work[k] / (double)m * p->chirp[k];
    a[k] = sign > 0 ? conj(y) : y;
  }
}

void orc_fft1d(int n, double *data, int sign) {
  plan1d *p = plan_create(n);
  cplx *work = malloc(sizeof(cplx) * (p->m > 0 ? p->m : 1));
  exec1d(p, (cplx *)data, sign, work);
  free(work);
  plan_free(p);
}

#define KB 16 /* kz block for the strided passes */

/* Complex passes along y then x (sign), on the [N][N][N/2+1] complex view. */
static void complex_xy_passes(int N, cplx *c, int sign, const plan1d *p, int order_y_first) {
  const int NH = N / 2 + 1;
  for (int pass = 0; pass < 2; pass++) {
    int along_y = order_y_first ? (pass == 0) : (pass == 1);
    if (along_y) {
#pragma omp parallel
      {
        cplx *buf = malloc(sizeof(cplx) * (size_t)N * KB);
        cplx *work = malloc(sizeof(cplx) * (p->m > 0 ? p->m : 1));
#pragma omp for schedule(static)
        for (int x = 0; x < N; x++) {
          for (int k0 = 0; k0 < NH; k0 += KB) {
            int nb = NH - k0 < KB ? NH - k0 : KB;
            for (int y = 0; y < N; y++)
              for (int b = 0; b < nb; b++) buf[(size_t)b * N + y] = c[((size_t)x * N + y) * NH + k0 + b];
            for (int b = 0; b < nb; b++) exec1d(p, buf + (size_t)b * N, sign, work);
            for (int y = 0; y < N; y++)
              for (int b = 0; b < nb; b++) c[((size_t)x * N + y) * NH + k0 + b] = buf[(size_t)b * N + y];
          }
        }
        free(buf); free(work);
      }
    } else {
#pragma omp parallel
      {
        cplx *buf = malloc(sizeof(cplx) * (size_t)N * KB);
        cplx *work = malloc(sizeof(cplx) * (p->m > 0 ? p->m : 1));
#pragma omp for schedule(static)
        for (int y = 0; y < N; y++) {
          for (int k0 = 0; k0 < NH; k0 += KB) {
            int nb = NH - k0 < KB ? NH - k0 : KB;
            for (int x = 0; x < N; x++)
              for (int b = 0; b < nb; b++) buf[(size_t)b * N + x] = c[((size_t)x * N + y) * NH + k0 + b];
            for (int b = 0; b < nb; b++) exec1d(p, buf + (size_t)b * N, sign, work);
            for (int x = 0; x < N; x++)
              for (int b = 0; b < nb; b++) c[((size_t)x * N + y) * NH + k0 + b] = buf[(size_t)b * N + x];
          }
        }
        free(buf); free(work);
      }
    }
  }
}

void orc_fft_r2c(int N, double *grid) {
  const int NH = N / 2 + 1;
  const size_t P = 2 * (size_t)NH;
  plan1d *p = plan_create(N);
  /* rows along z: real -> first N/2+1 complex outputs */
#pragma omp parallel
  {
    cplx *row = malloc(sizeof(cplx) * N);
    cplx *work = malloc(sizeof(cplx) * (p->m > 0 ? p->m : 1));
#pragma omp for schedule(static)
    for (long r = 0; r < (long)N * N; r++) {
      double *g = grid + (size_t)r * P;
      for (int z = 0; z < N; z++) row[z] = g[z];
      exec1d(p, row, -1, work);
      for (int k = 0; k < NH; k++) { g[2 * k] = creal(row[k]); g[2 * k + 1] = cimag(row[k]); }
    }
    free(row); free(work);
  }
  complex_xy_passes(N, (cplx *)grid, -1, p, 1);
  plan_free(p);
}

void orc_fft_c2r(int N, double *grid) {
  const int NH = N / 2 + 1;
  const size_t P = 2 * (size_t)NH;
  plan1d *p = plan_create(N);
  complex_xy_passes(N, (cplx *)grid, +1, p, 0);
#pragma omp parallel
  {
    cplx *row = malloc(sizeof(cplx) * N);
    cplx *work = malloc(sizeof(cplx) * (p->m > 0 ? p->m : 1));
#pragma omp for schedule(static)
    for (long r = 0; r < (long)N * N; r++) {
      double *g = grid + (size_t)r * P;
      row[0] = g[0];
      for (int k = 1; k < NH; k++) {
        cplx h = g[2 * k] + I * g[2 * k + 1];
        if (2 * k == N) { row[k] = creal(h); continue; }
        row[k] = h;
        row[N - k] = conj(h);
      }
      exec1d(p, row, +1, work);
      for (int z = 0; z < N; z++) g[z] = creal(row[z]);
      for (size_t z = N; z < P; z++) g[z] = 0.0;
    }
    free(row); free(work);
  }
  plan_free(p);
}
