/*
 * Oracle 2LPT initial conditions (test infrastructure only):
 * displacement_fields() Gaussian branch and 2LPT part, src/2LPT.c:185-495 and
 * 1209-1519, in double precision for a single task.
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846

/* Seed table, src/2LPT.c:262-271: one sequential stream seeded by Seed. */
void orc_seedtable(int N, uint32_t seed, uint32_t *t) {
  uint64_t n = 0;
#define DRAW ((uint32_t)(0x7fffffff * orc_stream_uniform(seed, n++)))
  for (int i = 0; i < N / 2; i++) {
    for (int j = 0; j < i; j++) t[i * N + j] = DRAW;
    for (int j = 0; j < i + 1; j++) t[j * N + i] = DRAW;
    for (int j = 0; j < i; j++) t[(N - 1 - i) * N + j] = DRAW;
    for (int j = 0; j < i + 1; j++) t[(N - 1 - j) * N + i] = DRAW;
    for (int j = 0; j < i; j++) t[i * N + (N - 1 - j)] = DRAW;
    for (int j = 0; j < i + 1; j++) t[j * N + (N - 1 - i)] = DRAW;
    for (int j = 0; j < i; j++) t[(N - 1 - i) * N + (N - 1 - j)] = DRAW;
    for (int j = 0; j < i + 1; j++) t[(N - 1 - j) * N + (N - 1 - i)] = DRAW;
  }
#undef DRAW
}

/* kvec component exactly as written at 2LPT.c:359-375 */
static double kcomp(int i, int N, double box) {
  if (i < N / 2) return i * 2 * PI / box;
  return -(N - i) * 2 * PI / box;
}

static void cset(double *c, size_t idx, double re, double im) { c[2 * idx] = re; c[2 * idx + 1] = im; }

static void lpt_from_cdisp(const orc_ic_params *ip, double *cdisp[3], double *D1, double *D2,
                           double *source2k_out);

void orc_ic_2lpt(const orc_ic_params *ip, const orc_power *pw, double *D1, double *D2,
                 double *deltak_out, double *source2k_out) {
  const int N = ip->N, Ns = ip->Ns, NH = N / 2 + 1;
  const double Box = ip->box;
  const size_t tot = (size_t)N * N * NH;
  uint32_t *seedtable = malloc(sizeof(uint32_t) * (size_t)N * N);
  orc_seedtable(N, ip->seed, seedtable);
  double *cdisp[3], *cdelta = calloc(2 * tot, 8);
  for (int a = 0; a < 3; a++) cdisp[a] = calloc(2 * tot, 8);

  for (int i = 0; i < N; i++) {
    for (int j = 0; j < N; j++) {
      uint32_t s = seedtable[i * N + j];
      uint64_t n = 0;
      for (int k = 0; k < N / 2; k++) {
        double phase = orc_stream_uniform(s, n++) * 2 * PI, ampl = 0.0;
        if (!ip->fixed_amplitude) {
          do { ampl = orc_stream_uniform(s, n++); } while (ampl == 0);
        }
        if (i == N / 2 || j == N / 2 || k == N / 2) continue;
        if (i == 0 && j == 0 && k == 0) continue;
        double kvec[3] = {kcomp(i, N, Box), kcomp(j, N, Box), kcomp(k, N, Box)};
        double kmag2 = kvec[0] * kvec[0] + kvec[1] * kvec[1] + kvec[2] * kvec[2];
        double kmag = sqrt(kmag2);
        if (ip->sphere_mode == 1) {
          if (kmag * Box / (2 * PI) > Ns / 2) continue;
        } else {
          if (fabs(kvec[0]) * Box / (2 * PI) > Ns / 2) continue;
          if (fabs(kvec[1]) * Box / (2 * PI) > Ns / 2) continue;
          if (fabs(kvec[2]) * Box / (2 * PI) > Ns / 2) continue;
        }
        double p_of_k = orc_power_spec(pw, kmag);
        if (!ip->fixed_amplitude) p_of_k *= -log(ampl);
        p_of_k *= ip->pofk_rescale;
        double delta = pow(Box, -1.5) * sqrt(p_of_k);
        if (ip->inverted) delta *= -1.0;
        double re = delta * cos(phase), im = delta * sin(phase);
        if (k > 0) {
          size_t c = ((size_t)i * N + j) * NH + k;
          for (int a = 0; a < 3; a++) cset(cdisp[a], c, -kvec[a] / kmag2 * im, kvec[a] / kmag2 * re);
          cset(cdelta, c, re, im);
        } else if (i == 0) {
          if (j >= N / 2) continue;
          int jj = N - j;
          size_t c = ((size_t)i * N + j) * NH + k, c2 = ((size_t)i * N + jj) * NH + k;
          for (int a = 0; a < 3; a++) {
            cset(cdisp[a], c, -kvec[a] / kmag2 * im, kvec[a] / kmag2 * re);
            cset(cdisp[a], c2, -kvec[a] / kmag2 * im, -kvec[a] / kmag2 * re);
          }
          cset(cdelta, c, re, im);
          cset(cdelta, c2, re, -im);
        } else {
          if (i >= N / 2) continue;
          int ii = N - i, jj = N - j;
          if (ii == N) ii = 0;
          if (jj == N) jj = 0;
          size_t c = ((size_t)i * N + j) * NH + k, c2 = ((size_t)ii * N + jj) * NH + k;
          for (int a = 0; a < 3; a++) {
            cset(cdisp[a], c, -kvec[a] / kmag2 * im, kvec[a] / kmag2 * re);
            cset(cdisp[a], c2, -kvec[a] / kmag2 * im, -kvec[a] / kmag2 * re);
          }
          cset(cdelta, c, re, im);
          cset(cdelta, c2, re, -im);
        }
      }
    }
  }
  free(seedtable);
  if (deltak_out) memcpy(deltak_out, cdelta, sizeof(double) * 2 * tot);
  free(cdelta);
  lpt_from_cdisp(ip, cdisp, D1, D2, source2k_out);
}

/* The 2LPT part shared by both IC sources (2LPT.c:1209-1519): gradients of
 * the ZA displacements, second-order source, both displacement fields and
 * the read-out to the lattice.  Frees cdisp. */
static void lpt_from_cdisp(const orc_ic_params *ip, double *cdisp[3], double *D1, double *D2,
                           double *source2k_out) {
  const int N = ip->N, Ns = ip->Ns, NH = N / 2 + 1;
  const double Box = ip->box;
  const size_t tot = (size_t)N * N * NH;
  /* displacement gradients, 2LPT.c:1224-1270 */
  double *dg[6];
  for (int g = 0; g < 6; g++) dg[g] = malloc(sizeof(double) * 2 * tot);
  const int src_a[6] = {0, 0, 0, 1, 1, 2}, der_b[6] = {0, 1, 2, 1, 2, 2};
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t c = ((size_t)i * N + j) * NH + k;
        double kvec[3] = {kcomp(i, N, Box), kcomp(j, N, Box), kcomp(k, N, Box)};
        for (int g = 0; g < 6; g++) {
          const double *cd = cdisp[src_a[g]];
          dg[g][2 * c] = -cd[2 * c + 1] * kvec[der_b[g]];
          dg[g][2 * c + 1] = cd[2 * c] * kvec[der_b[g]];
        }
      }
  for (int g = 0; g < 6; g++) orc_fft_c2r(N, dg[g]);
  /* second-order source, 2LPT.c:1282-1290 */
  const size_t P = 2 * (size_t)NH;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < N; k++) {
        size_t c = ((size_t)i * N + j) * P + k;
        dg[3][c] = dg[0][c] * (dg[3][c] + dg[5][c]) + dg[3][c] * dg[5][c] - dg[1][c] * dg[1][c] -
                   dg[2][c] * dg[2][c] - dg[4][c] * dg[4][c];
      }
  orc_fft_r2c(N, dg[3]);
  if (source2k_out) {
    /* cdelta_cdm2 = -source(k), zero at k = 0 (2LPT.c:1334-1341) */
    for (size_t c = 0; c < tot; c++) { source2k_out[2 * c] = -dg[3][2 * c]; source2k_out[2 * c + 1] = -dg[3][2 * c + 1]; }
    source2k_out[0] = source2k_out[1] = 0.0;
  }
  /* 2nd order displacements, 2LPT.c:1311-1355 */
  double *cdisp2[3] = {dg[0], dg[1], dg[2]};
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t c = ((size_t)i * N + j) * NH + k;
        double kvec[3] = {kcomp(i, N, Box), kcomp(j, N, Box), kcomp(k, N, Box)};
        double kmag2 = kvec[0] * kvec[0] + kvec[1] * kvec[1] + kvec[2] * kvec[2];
        for (int a = 0; a < 3; a++) {
          if (kmag2 > 0.0) {
            cdisp2[a][2 * c] = dg[3][2 * c + 1] * kvec[a] / kmag2;
            cdisp2[a][2 * c + 1] = -dg[3][2 * c] * kvec[a] / kmag2;
          } else {
            cdisp2[a][2 * c] = cdisp2[a][2 * c + 1] = 0.0;
          }
        }
      }
  free(dg[3]); free(dg[4]); free(dg[5]);
  for (int a = 0; a < 3; a++) { orc_fft_c2r(N, cdisp[a]); orc_fft_c2r(N, cdisp2[a]); }

  /* read-out to the particle lattice, 2LPT.c:1424-1491 */
  const double nmesh3 = (double)N * (double)N * (double)N;
  double sum1[3] = {0, 0, 0}, sum2[3] = {0, 0, 0};
  const long np = (long)Ns * Ns * Ns;
  for (int nn = 0; nn < Ns; nn++)
    for (int m = 0; m < Ns; m++)
      for (int p = 0; p < Ns; p++) {
        long coord = ((long)nn * Ns + m) * Ns + p;
        double u = (double)(nn * N) / (double)Ns, v = (double)(m * N) / (double)Ns, w = (double)(p * N) / (double)Ns;
        int i = (int)u, j = (int)v, k = (int)w;
        if (i == N) i = N - 1;
        if (j == N) j = N - 1;
        if (k == N) k = N - 1;
        u -= i; v -= j; w -= k;
        int ii = i + 1, jj = j + 1, kk = k + 1;
        if (ii >= N) ii -= N; /* ghost slice = slice 0 for one task */
        if (jj >= N) jj -= N;
        if (kk >= N) kk -= N;
        double f[8] = {(1 - u) * (1 - v) * (1 - w), (1 - u) * (1 - v) * (w), (1 - u) * (v) * (1 - w), (1 - u) * (v) * (w),
                       (u) * (1 - v) * (1 - w),     (u) * (1 - v) * (w),     (u) * (v) * (1 - w),     (u) * (v) * (w)};
        size_t id[8] = {((size_t)i * N + j) * P + k,  ((size_t)i * N + j) * P + kk,  ((size_t)i * N + jj) * P + k,
                        ((size_t)i * N + jj) * P + kk, ((size_t)ii * N + j) * P + k, ((size_t)ii * N + j) * P + kk,
                        ((size_t)ii * N + jj) * P + k, ((size_t)ii * N + jj) * P + kk};
        for (int a = 0; a < 3; a++) {
          double dis = 0, dis2 = 0;
          for (int t = 0; t < 8; t++) { dis += cdisp[a][id[t]] * f[t]; dis2 += cdisp2[a][id[t]] * f[t]; }
          dis2 /= nmesh3;
          D1[3 * coord + a] = dis;
          D2[3 * coord + a] = -3. / 7. * dis2;
          sum1[a] += dis;
          sum2[a] += -3. / 7. * dis2;
        }
      }
  for (int a = 0; a < 3; a++) { sum1[a] /= (double)np; sum2[a] /= (double)np; }
  for (long q = 0; q < np; q++)
    for (int a = 0; a < 3; a++) { D1[3 * q + a] -= sum1[a]; D2[3 * q + a] -= sum2[a]; }
  for (int a = 0; a < 3; a++) { free(cdisp[a]); free(cdisp2[a]); }
}

/* ReadFilesMakeDisplacementField + AssignDisplacementField
 * (src/readICfromfile.c:133-219, 533-777): particles (positions in [0,1) of
 * the box, [n][3]) CIC-deposited as ProcessParticlesSingleFile does (density
 * starts at -1, weight (N/Ns)^3 folded into the y factors), R2C, times
 * normfac = D_LCDM(1) / D_LCDM(a_i) / N^3, modes with |d| > Ns/2 zeroed when
 * N > Ns; then cdisp = i k / k^2 delta(k) * grid_corr * rescale with
 * grid_corr = 1 / prod_{d != 0} sinc(pi d / N)^2 and rescale[|d|^2] given by
 * the caller (sqrt(mg_pofk_ratio(k, 1)), divided by the sigma8 enhancement
 * when the input sigma8 is not for LCDM).  With N <= Ns the three Nyquist
 * planes of delta(k) are zeroed (the reference uses +N/2 there for the
 * displacement and -N/2 for its gradients).  Then the shared 2LPT part. */
void orc_ic_2lpt_from_particles(const orc_ic_params *ip, const double *pos01, long n, double normfac,
                                const double *rescale_rk, double *D1, double *D2, double *deltak_out,
                                double *source2k_out) {
  const int N = ip->N, Ns = ip->Ns, NH = N / 2 + 1;
  const size_t P = 2 * (size_t)NH, tot = (size_t)N * N * NH;
  const double Box = ip->box;
  double *rho = malloc(sizeof(double) * (size_t)N * N * P);
  for (size_t q = 0; q < (size_t)N * N * P; q++) rho[q] = -1.0;
  const double wpar = pow((double)N / (double)Ns, 3);
  for (long q = 0; q < n; q++) {
    double X = pos01[3 * q] * N, Y = pos01[3 * q + 1] * N, Z = pos01[3 * q + 2] * N;
    unsigned IX = (unsigned)X, IY = (unsigned)Y, IZ = (unsigned)Z;
    double DX = X - IX, DY = Y - IY, DZ = Z - IZ, TX = 1 - DX, TY = 1 - DY, TZ = 1 - DZ;
    DY *= wpar;
    TY *= wpar;
    if (IX >= (unsigned)N) IX = 0;
    if (IY >= (unsigned)N) IY = 0;
    if (IZ >= (unsigned)N) IZ = 0;
    unsigned IXn = IX + 1 >= (unsigned)N ? 0 : IX + 1, IYn = IY + 1 >= (unsigned)N ? 0 : IY + 1,
             IZn = IZ + 1 >= (unsigned)N ? 0 : IZ + 1; /* the ghost x-slice is slice 0 for one task */
    rho[((size_t)IX * N + IY) * P + IZ] += TX * TY * TZ;
    rho[((size_t)IX * N + IY) * P + IZn] += TX * TY * DZ;
    rho[((size_t)IX * N + IYn) * P + IZ] += TX * DY * TZ;
    rho[((size_t)IX * N + IYn) * P + IZn] += TX * DY * DZ;
    rho[((size_t)IXn * N + IY) * P + IZ] += DX * TY * TZ;
    rho[((size_t)IXn * N + IY) * P + IZn] += DX * TY * DZ;
    rho[((size_t)IXn * N + IYn) * P + IZ] += DX * DY * TZ;
    rho[((size_t)IXn * N + IYn) * P + IZn] += DX * DY * DZ;
  }
  orc_fft_r2c(N, rho);
  double *dk = rho; /* complex [N][N][NH] in place */
  for (size_t c = 0; c < 2 * tot; c++) dk[c] *= normfac;
  double *cdisp[3], *cdelta = calloc(2 * tot, 8);
  for (int a = 0; a < 3; a++) cdisp[a] = calloc(2 * tot, 8);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        const size_t c = ((size_t)i * N + j) * NH + k;
        const int d[3] = {i > N / 2 ? i - N : i, j > N / 2 ? j - N : j, k};
        const long d2 = (long)d[0] * d[0] + (long)d[1] * d[1] + (long)d[2] * d[2];
        if (d2 == 0) continue;
        if (N > Ns && sqrt((double)d2) > Ns / 2) continue;
        if (N <= Ns && (i == N / 2 || j == N / 2 || k == N / 2)) continue;
        double gc = 1.0;
        for (int a = 0; a < 3; a++)
          if (d[a] != 0) gc *= sin(PI * d[a] / (double)N) / (PI * d[a] / (double)N);
        const double f = 1.0 / (gc * gc) * rescale_rk[d2];
        const double re = dk[2 * c] * f, im = dk[2 * c + 1] * f;
        double kvec[3], kmag2 = 0.0;
        for (int a = 0; a < 3; a++) {
          kvec[a] = d[a] * 2 * PI / Box;
          kmag2 += kvec[a] * kvec[a];
        }
        for (int a = 0; a < 3; a++) cset(cdisp[a], c, -kvec[a] / kmag2 * im, kvec[a] / kmag2 * re);
        cset(cdelta, c, re, im);
      }
  free(rho);
  if (deltak_out) memcpy(deltak_out, cdelta, sizeof(double) * 2 * tot);
  free(cdelta);
  lpt_from_cdisp(ip, cdisp, D1, D2, source2k_out);
}
