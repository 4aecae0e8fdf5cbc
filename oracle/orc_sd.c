/*
 * Oracle scale-dependent displacement fields (test infrastructure only):
 * from_cdisp_store_to_ZA, src/2LPT.c:1539-1735, for a single task, in double
 * precision.
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846

static double kcomp(int i, int N, double box) {
  if (i < N / 2) return i * 2 * PI / box;
  return -(N - i) * 2 * PI / box;
}

void orc_sd_field(orc_cosmo *c, const double *stored, int N, int Ns, double box, double A, double AFF,
                  int fieldtype, int order, double *out) {
  const int NH = N / 2 + 1;
  const size_t tot = (size_t)N * N * NH, P = 2 * (size_t)NH;
  const double nmesh3 = (double)N * (double)N * (double)N;
  /* growth function of the order (2LPT.c:1547-1557) */
  int f0 = order == 1 ? 0 : 3;
  double normfactor = order == 1 ? 1.0 : -3.0 / 7.0 / nmesh3;
  double *disp[3];
  for (int a = 0; a < 3; a++) disp[a] = malloc(sizeof(double) * 2 * tot);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t cc = ((size_t)i * N + j) * NH + k;
        double kv[3] = {kcomp(i, N, box), kcomp(j, N, box), kcomp(k, N, box)};
        double kmag2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2], kmag = sqrt(kmag2);
        double g = 1.0;
        if (kmag2 > 0.0) {
          if (fieldtype == ORC_FIELD_D) g = normfactor * orc_growth_sd(c, f0, kmag, A);
          if (fieldtype == ORC_FIELD_dDdy) g = normfactor * orc_growth_sd(c, f0 + 1, kmag, A);
          if (fieldtype == ORC_FIELD_ddDddy) g = normfactor * orc_growth_sd(c, f0 + 2, kmag, A);
          if (fieldtype == ORC_FIELD_deltaD)
            g = normfactor * (orc_growth_sd(c, f0, kmag, AFF) - orc_growth_sd(c, f0, kmag, A));
        }
        for (int a = 0; a < 3; a++) {
          if (kmag2 > 0.0) {
            disp[a][2 * cc] = -stored[2 * cc + 1] * kv[a] / kmag2 * g;
            disp[a][2 * cc + 1] = stored[2 * cc] * kv[a] / kmag2 * g;
          } else {
            disp[a][2 * cc] = disp[a][2 * cc + 1] = 0.0;
          }
        }
      }
  for (int a = 0; a < 3; a++) orc_fft_c2r(N, disp[a]);
  /* read-out at the Lagrangian lattice (2LPT.c:1642-1704) and mean removal
   * (2LPT.c:1714-1728) */
  const long np = (long)Ns * Ns * Ns;
  double sum[3] = {0, 0, 0};
  for (int n = 0; n < Ns; n++)
    for (int m = 0; m < Ns; m++)
      for (int p = 0; p < Ns; p++) {
        long coord = ((long)n * Ns + m) * Ns + p;
        double u = (double)(n * N) / (double)Ns, v = (double)(m * N) / (double)Ns, w = (double)(p * N) / (double)Ns;
        int i = (int)u, j = (int)v, k = (int)w;
        if (i == N) i = N - 1;
        if (j == N) j = N - 1;
        if (k == N) k = N - 1;
        u -= i; v -= j; w -= k;
        int ii = i + 1, jj = j + 1, kk = k + 1;
        if (ii >= N) ii -= N; /* the ghost slice of one task is slice 0 */
        if (jj >= N) jj -= N;
        if (kk >= N) kk -= N;
        double f[8] = {(1 - u) * (1 - v) * (1 - w), (1 - u) * (1 - v) * (w), (1 - u) * (v) * (1 - w), (1 - u) * (v) * (w),
                       (u) * (1 - v) * (1 - w),     (u) * (1 - v) * (w),     (u) * (v) * (1 - w),     (u) * (v) * (w)};
        size_t id[8] = {((size_t)i * N + j) * P + k,  ((size_t)i * N + j) * P + kk,  ((size_t)i * N + jj) * P + k,
                        ((size_t)i * N + jj) * P + kk, ((size_t)ii * N + j) * P + k, ((size_t)ii * N + j) * P + kk,
                        ((size_t)ii * N + jj) * P + k, ((size_t)ii * N + jj) * P + kk};
        for (int a = 0; a < 3; a++) {
          double d = 0;
          for (int t = 0; t < 8; t++) d += disp[a][id[t]] * f[t];
          out[3 * coord + a] = d;
          sum[a] += d;
        }
      }
  for (int a = 0; a < 3; a++) sum[a] /= (double)np;
  for (long q = 0; q < np; q++)
    for (int a = 0; a < 3; a++) out[3 * q + a] -= sum[a];
  for (int a = 0; a < 3; a++) free(disp[a]);
}
