/*
 * Oracle modified-gravity fifth force (test infrastructure only):
 * ComputeFifthForce (src/user_defined_functions.h:687-719) and the screening
 * passes of src/mg.h, in double precision.
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define INVERSE_H0_MPCH 2997.92458
#define PI 3.14159265358979323846

static inline long rk_of(int N, int i, int j, int k) {
  long ii = i > N / 2 ? N - i : i;
  return (long)k * k + ii * ii + (long)j * j;
}

/* DivideByLaplacian, src/mg.h:21-64 */
static void divide_by_laplacian(const orc_mg *m, double a, int N, double box, const double *dk, double *out) {
  const int NH = N / 2 + 1;
  double normfactor = 1.0 / pow((double)N, 3);
  normfactor *= 1.5 * m->omega / a * pow(box / INVERSE_H0_MPCH / (2.0 * PI), 2);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t ind = ((size_t)i * N + j) * NH + k;
        int jj = j > N / 2 ? N - j : j;
        long RK = rk_of(N, i, jj, k);
        if (RK == 0) { out[2 * ind] = out[2 * ind + 1] = 0.0; continue; }
        double KK = -1.0 / (double)RK;
        out[2 * ind] = normfactor * dk[2 * ind] * KK;
        out[2 * ind + 1] = normfactor * dk[2 * ind + 1] * KK;
      }
}

/* EffDensitykToPhiofk, src/mg.h:74-116 */
static void eff_density_to_phik(const orc_mg *m, double a, int N, double box, double *c) {
  const int NH = N / 2 + 1;
  double normfactor = orc_coupling(m, a);
  double massterm2 = pow(a, 2) * orc_mass2_of_a(m, a) / pow((2.0 * PI) * INVERSE_H0_MPCH / box, 2);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t ind = ((size_t)i * N + j) * NH + k;
        int jj = j > N / 2 ? N - j : j;
        long RK = rk_of(N, i, jj, k);
        if (RK == 0) { c[2 * ind] = c[2 * ind + 1] = 0.0; continue; }
        double KK = (double)RK / ((double)RK + massterm2);
        c[2 * ind] = normfactor * c[2 * ind] * KK;
        c[2 * ind + 1] = normfactor * c[2 * ind + 1] * KK;
      }
}

/* smoothing_filter, src/mg.h:318-338 */
static double smoothing_filter(int type, double kR) {
  if (type == 1) return exp(-0.5 * kR * kR);
  if (type == 2) { if (kR < 1e-5) return 1.0; return 3.0 / (kR * kR * kR) * (sin(kR) - kR * cos(kR)); }
  if (type == 3) return kR < 1.0 ? 1.0 : 0.0;
  return 1.0;
}

/* SmoothDensityField, src/mg.h:268-309 */
static void smooth_density(const orc_mg *m, int N, double box, const double *dk, double *out) {
  const int NH = N / 2 + 1;
  double normfactor = 1.0 / pow((double)N, 3);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < NH; k++) {
        size_t ind = ((size_t)i * N + j) * NH + k;
        int jj = j > N / 2 ? N - j : j;
        long RK = rk_of(N, i, jj, k);
        double smooth = smoothing_filter(m->smoothing_filter, sqrt((double)RK) * 2.0 * PI / box * m->rsmooth) * normfactor;
        out[2 * ind] = dk[2 * ind] * smooth;
        out[2 * ind + 1] = dk[2 * ind + 1] * smooth;
      }
}

void orc_fifth_force(const orc_mg *m, double a, int N, double box, const double *density_x,
                     double *deltak, double *mgk) {
  const int NH = N / 2 + 1;
  const size_t total = (size_t)N * N * NH;
  if (!m->mg_active) return;
  if (m->model == ORC_FOFR || m->model == ORC_MBETA) {
    /* ComputeFifthForce_PotentialScreening, src/mg.h:147-189 */
    if (!m->include_screening) {
      memcpy(mgk, density_x, sizeof(double) * 2 * total);
      orc_fft_r2c(N, mgk);
      eff_density_to_phik(m, a, N, box, mgk);
      return;
    }
    double *phi = malloc(sizeof(double) * 2 * total);
    divide_by_laplacian(m, a, N, box, deltak, phi);
    orc_fft_c2r(N, phi);
    memcpy(mgk, density_x, sizeof(double) * 2 * total);
    #pragma omp parallel for schedule(static)
    for (size_t j = 0; j < 2 * total; j++) mgk[j] *= orc_screen_potential(m, a, phi[j]);
    free(phi);
    orc_fft_r2c(N, mgk);
    eff_density_to_phik(m, a, N, box, mgk);
  } else if (m->model == ORC_DGP) {
    /* ComputeFifthForce_DensityScreening, src/mg.h:197-260 */
    double coupling = orc_coupling(m, a);
    if (!m->include_screening) {
      #pragma omp parallel for schedule(static)
      for (size_t i = 0; i < 2 * total; i++) mgk[i] = deltak[i] * coupling;
      return;
    }
    double *sm = malloc(sizeof(double) * 2 * total);
    smooth_density(m, N, box, deltak, sm);
    orc_fft_c2r(N, sm);
    memcpy(mgk, density_x, sizeof(double) * 2 * total);
    #pragma omp parallel for schedule(static)
    for (size_t j = 0; j < 2 * total; j++) mgk[j] *= coupling * orc_screen_density(m, a, sm[j]);
    free(sm);
    orc_fft_r2c(N, mgk);
  } else if (m->model == ORC_JBD_GEFF) {
    /* ComputeFifthForce_TimeDepGeffModels, src/mg.h:127-137 */
    double g = orc_geff(m, a, 0.0);
    #pragma omp parallel for schedule(static)
    for (size_t j = 0; j < 2 * total; j++) deltak[j] *= g;
  }
}
