/*
 * Oracle (test infrastructure only): massive neutrinos as the reference's
 * MASSIVE_NEUTRINOS build runs them.
 *
 *  - CAMB transfer functions read from an info file and one file per
 *    redshift, kept as 2D bicubic tables over (ln k, z)
 *    (src/read_CAMB_data.h:41-170, 238-278);
 *  - OmegaNu / OmegaCDM (init_modified_version,
 *    src/user_defined_functions.h:50-75);
 *  - the factors mu_nu of the growth equations
 *    (GeffoverG_neutrino_1LPT/_2LPT, src/user_defined_functions.h:662-684);
 *  - the CDM+baryon power spectrum (src/read_CAMB_data.h:210-226,
 *    src/power.c:376-380);
 *  - the neutrino density added to delta(k) every step
 *    (src/auxPM.c:383-421).
 */
#include "orc.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { NU_T_NU = 0, NU_T_CDM = 1, NU_T_B = 2, NU_T_TOT = 3 };

struct orc_nu_s {
  orc_bicubic T[4];
  double omega, omega_b, omega_nu, omega_cdm, h, ns;
  int include;
};

/* one CAMB file: a header line, then rows of 13 numbers; k/h in column 0,
 * T_cdm 1, T_b 2, T_massive-nu 5, T_total 6 */
static int read_one(const char *path, double **cols, int *n) {
  FILE *fp = fopen(path, "r");
  if (!fp) return -1;
  int ch;
  while ((ch = fgetc(fp)) != EOF && ch != '\n') {
  }
  int cap = 256, rows = 0;
  for (int c = 0; c < 5; c++) cols[c] = malloc(sizeof(double) * cap);
  double v[13];
  for (;;) {
    int got = 0;
    while (got < 13 && fscanf(fp, "%lf", &v[got]) == 1) got++;
    if (got < 13) break;
    if (rows == cap) {
      cap *= 2;
      for (int c = 0; c < 5; c++) cols[c] = realloc(cols[c], sizeof(double) * cap);
    }
    cols[0][rows] = log(v[0]);
    cols[1][rows] = v[5];
    cols[2][rows] = v[1];
    cols[3][rows] = v[2];
    cols[4][rows] = v[6];
    rows++;
  }
  fclose(fp);
  *n = rows;
  return 0;
}

orc_nu *orc_nu_create(const char *infofile, double omega, double omega_b, double h, double ns, double sum_mnu_ev,
                      int include) {
  FILE *fp = fopen(infofile, "r");
  if (!fp) return NULL;
  char dir[512], name[512];
  int nz = 0;
  if (fscanf(fp, "%511s %d", dir, &nz) != 2 || nz < 2) {
    fclose(fp);
    return NULL;
  }
  double *z = malloc(sizeof(double) * nz), *logk = NULL;
  double *tab[4] = {NULL, NULL, NULL, NULL};
  int nk = 0, ok = 1;
  for (int iz = 0; iz < nz && ok; iz++) {
    if (fscanf(fp, "%511s %lf", name, &z[iz]) != 2) { ok = 0; break; }
    char path[1100];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    double *cols[5];
    int n = 0;
    if (read_one(path, cols, &n)) { ok = 0; break; }
    if (iz == 0) {
      nk = n;
      logk = malloc(sizeof(double) * nk);
      memcpy(logk, cols[0], sizeof(double) * nk);
      for (int t = 0; t < 4; t++) tab[t] = malloc(sizeof(double) * nk * nz);
    }
    if (n != nk) ok = 0;
    /* tables z[iz * nk + ik]: x = ln k, y = z */
    for (int t = 0; t < 4 && ok; t++) memcpy(tab[t] + (size_t)iz * nk, cols[t + 1], sizeof(double) * nk);
    for (int c = 0; c < 5; c++) free(cols[c]);
  }
  fclose(fp);
  orc_nu *nu = NULL;
  if (ok) {
    nu = calloc(1, sizeof(orc_nu));
    for (int t = 0; t < 4; t++) orc_bicubic_init(&nu->T[t], logk, z, tab[t], nk, nz);
    nu->omega = omega;
    nu->omega_b = omega_b;
    nu->h = h;
    nu->ns = ns;
    nu->omega_nu = sum_mnu_ev / (93.14 * h * h);
    nu->omega_cdm = omega - omega_b - nu->omega_nu;
    nu->include = include;
    if (nu->omega_nu < 1e-6) {
      nu->omega_nu = 0.0;
      nu->omega_cdm = omega - omega_b;
      nu->include = 0;
    }
  }
  for (int t = 0; t < 4; t++) free(tab[t]);
  free(logk);
  free(z);
  return nu;
}

void orc_nu_free(orc_nu *nu) {
  if (!nu) return;
  for (int t = 0; t < 4; t++) orc_bicubic_free(&nu->T[t]);
  free(nu);
}

double orc_nu_omega_nu(const orc_nu *nu) { return nu->omega_nu; }
double orc_nu_omega_cdm(const orc_nu *nu) { return nu->omega_cdm; }

/* Lookup_GSL_2D_Spline (src/wrappers.c:129-136) of a transfer table at
 * (ln k, z = 1/a - 1): clamp into the table, then evaluate */
double orc_nu_transfer(const orc_nu *nu, int which, double k, double a) {
  const orc_bicubic *b = &nu->T[which];
  double x = log(k), y = 1.0 / a - 1.0;
  if (x < b->x[0]) x = b->x[0];
  if (x > b->x[b->nx - 1]) x = b->x[b->nx - 1];
  if (y < b->y[0]) y = b->y[0];
  if (y > b->y[b->ny - 1]) y = b->y[b->ny - 1];
  return orc_bicubic_eval(b, x, y);
}

/* get_cdm_baryon_transfer_function with the OmegaCDM in force when it runs */
double orc_nu_Tcb(const orc_nu *nu, double k, double a, double omega_cdm) {
  return (nu->omega_b * orc_nu_transfer(nu, NU_T_B, k, a) + omega_cdm * orc_nu_transfer(nu, NU_T_CDM, k, a)) /
         (nu->omega_b + omega_cdm);
}

double orc_nu_mu1(const orc_nu *nu, double a, double k) {
  if (!nu || !(nu->omega_nu > 1e-6)) return 1.0;
  return (nu->omega - nu->omega_nu) / nu->omega +
         nu->omega_nu / nu->omega * orc_nu_transfer(nu, NU_T_NU, k, a) / orc_nu_Tcb(nu, k, a, nu->omega_cdm);
}

double orc_nu_mu2(const orc_nu *nu) {
  if (!nu || !(nu->omega_nu > 1e-6)) return 1.0;
  return (nu->omega - nu->omega_nu) / nu->omega;
}

/* get_cdm_baryon_power_spectrum: the total spectrum 2 pi^2 T_tot^2 (k h)
 * (k h / 0.05)^(ns - 1) h^3 at z = 0 times (T_cb / T_tot)^2 */
double orc_nu_pofk_cb(const orc_nu *nu, double k, double omega_cdm) {
  const double h = nu->h;
  const double Tt = orc_nu_transfer(nu, NU_T_TOT, k, 1.0), Tcb = orc_nu_Tcb(nu, k, 1.0, omega_cdm);
  const double ptot = 2.0 * M_PI * M_PI * Tt * Tt * (k * h) * pow(k * h / 0.05, nu->ns - 1.0) * h * h * h;
  return ptot * (Tcb / Tt) * (Tcb / Tt);
}

/* PtoMesh's neutrino block: every mode but k = 0 of the padded delta(k)
 * grid becomes cdmfac delta + nufac(k, a) delta_cdm(k), nufac =
 * OmegaNu / Omega N^3 T_nu(k, a) / T_cb(k, 1); delta_cdm is the stored IC
 * field (cdelta_cdm).  Nothing happens without nu_include_massive_neutrinos. */
void orc_nu_add_density(const orc_nu *nu, double a, int N, double box, double *grid, const double *cdelta) {
  if (!nu || !nu->include) return;
  const int NH = N / 2 + 1;
  const double cdmfac = (nu->omega - nu->omega_nu) / nu->omega;
  const double nf0 = nu->omega_nu / nu->omega * (double)N * N * N;
  for (int i = 0; i < N; i++) {
    const int di = i > N / 2 ? i - N : i;
    for (int j = 0; j < N; j++) {
      const int dj = j > N / 2 ? j - N : j;
      for (int k = 0; k < NH; k++) {
        if (i == 0 && j == 0 && k == 0) continue;
        const double kmag = 2.0 * M_PI / box * sqrt((double)di * di + (double)dj * dj + (double)k * k);
        const double nf = nf0 * orc_nu_transfer(nu, NU_T_NU, kmag, a) / orc_nu_Tcb(nu, kmag, 1.0, nu->omega_cdm);
        const size_t q = 2 * (((size_t)i * N + j) * NH + k);
        grid[q] = cdmfac * grid[q] + nf * cdelta[q];
        grid[q + 1] = cdmfac * grid[q + 1] + nf * cdelta[q + 1];
      }
    }
  }
}
