/*
 * Oracle end-to-end run (test infrastructure only): 2LPT IC + the KDK loop of
 * src/main.c:394-611 for one output redshift, scale-independent growth.
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* main.c:75-81, 400-455: COLA steps linearly in a with Sq/Sphi (StdDA 0);
 * the non-COLA run steps in ln a (stepDistr 1) with SqStd/SphiStd (StdDA 2) */
static double step_da(const orc_run_params *rp, double A, double ao, int n) {
  return rp->usecola ? (ao - A) / (double)n : (log(ao) - log(A)) / (double)n;
}
static double step_mid(const orc_run_params *rp, double A, double da) { return rp->usecola ? A + 0.5 * da : A * exp(0.5 * da); }
static double step_end(const orc_run_params *rp, double A, double da) { return rp->usecola ? A + da : A * exp(da); }
static double kick_dda(const orc_run_params *rp, orc_cosmo *c, double AI, double AF, double A) {
  return rp->usecola ? orc_Sphi(c, AI, AF, A) : orc_SphiStd(c, AI, AF);
}
static double drift_dyyy(const orc_run_params *rp, orc_cosmo *c, double A, double AFF, double AF) {
  return rp->usecola ? orc_Sq(c, A, AFF, AF) : orc_SqStd(c, A, AFF);
}

int orc_run(const orc_run_params *rp, double *pos_out, double *vel_out,
            double *kbin, double *pk, double *kmean, double *nmodes) {
  const int N = rp->ic.N, Ns = rp->ic.Ns, NH = N / 2 + 1;
  const double Box = rp->ic.box;
  const long np = (long)Ns * Ns * Ns;
  const size_t tot = (size_t)N * N * NH;
  const int sd = rp->mg.scaledependent;
  orc_cosmo *c = orc_cosmo_create_sd(&rp->mg, rp->init_redshift, Box, N);
  double *D1 = malloc(8 * 3 * np), *D2 = malloc(8 * 3 * np), *pos = malloc(8 * 3 * np), *vel = calloc(3 * np, 8);
  double *disp = malloc(8 * 3 * np);
  /* SCALEDEPENDENT: the stored delta(k) and -source(k) (2LPT.c:301-309,
   * 1336-1344) and the particle fields dDdy/dD2dy (vars.h:303-311); D1/D2
   * then play P.D/P.D2, which hold D at the IC and ddDddy in the loop */
  double *cdelta = NULL, *cdelta2 = NULL, *V1 = NULL, *V2 = NULL;
  if (sd) {
    cdelta = malloc(sizeof(double) * 2 * tot);
    cdelta2 = malloc(sizeof(double) * 2 * tot);
    V1 = malloc(8 * 3 * np);
    V2 = malloc(8 * 3 * np);
  }
  double A = 1.0 / (1.0 + rp->init_redshift);
  if (rp->ic_pos01) {
    /* ReadFilesMakeDisplacementField (src/readICfromfile.c:533-700):
     * delta(k) of the particles x D_LCDM(1)/D_LCDM(a_i)/N^3 */
    const double normfac = 1.0 / ((double)N * N * N) / orc_growth_DLCDM(c, A);
    orc_ic_2lpt_from_particles(&rp->ic, rp->ic_pos01, rp->ic_n, normfac, rp->ic_rescale_rk, D1, D2, cdelta, cdelta2);
  } else {
    orc_ic_2lpt(&rp->ic, &rp->pw, D1, D2, cdelta, cdelta2);
  }
  double Di = orc_growth_D(c, A), Di2 = orc_growth_D2(c, A);
  if (sd) {
    /* main.c:244-251 */
    orc_sd_field(c, cdelta, N, Ns, Box, A, A, ORC_FIELD_D, 1, D1);
    orc_sd_field(c, cdelta2, N, Ns, Box, A, A, ORC_FIELD_D, 2, D2);
    orc_sd_field(c, cdelta, N, Ns, Box, A, A, ORC_FIELD_dDdy, 1, V1);
    orc_sd_field(c, cdelta2, N, Ns, Box, A, A, ORC_FIELD_dDdy, 2, V2);
  }
  /* main.c:256-307: x = q + D Di + D2 Di2, or q + D + D2 when scale dependent;
   * v = 0 for COLA, else the 2LPT velocity */
  double fD = sd ? 1.0 : Di, fD2 = sd ? 1.0 : Di2;
  for (long p = 0; p < np; p++) {
    long i = p / ((long)Ns * Ns), j = (p / Ns) % Ns, k = p % Ns;
    long q[3] = {i, j, k};
    for (int a = 0; a < 3; a++) {
      pos[3 * p + a] = orc_periodic_wrap(q[a] * (Box / (double)Ns) + D1[3 * p + a] * fD + D2[3 * p + a] * fD2, Box);
      if (!rp->usecola)
        vel[3 * p + a] = sd ? V1[3 * p + a] + V2[3 * p + a]
                            : D1[3 * p + a] * orc_growth_dDdy(c, A) + D2[3 * p + a] * orc_growth_dD2dy(c, A);
    }
  }
  double AI = A, AF = A, AFF = A, da = 0;
  double *grid = malloc(sizeof(double) * 2 * tot), *dens_x = malloc(sizeof(double) * 2 * tot);
  double *mgk = malloc(sizeof(double) * 2 * tot);
  double *f[3];
  for (int a = 0; a < 3; a++) f[a] = malloc(sizeof(double) * 2 * tot);
  double sumv[3] = {0, 0, 0};
  int nb = rp->pofk_nbins;
  int uses_mgk = rp->mg.mg_active && (rp->mg.model == ORC_FOFR || rp->mg.model == ORC_MBETA || rp->mg.model == ORC_DGP);
  const int Noutputs = 1;
  for (int io = 0; io <= Noutputs; io++) {
    int nsteps;
    if (io == Noutputs) nsteps = 1;
    else {
      nsteps = rp->nsteps;
      double ao = 1.0 / (1.0 + rp->final_redshift);
      da = step_da(rp, A, ao, nsteps);
    }
    for (int ts = 0; ts < nsteps; ts++) {
      if (ts == 0 && io != 0) AF = A;
      else AF = step_mid(rp, A, da);
      AFF = step_end(rp, A, da);
      /* GetDisplacements (auxPM.c:37-103) */
      orc_cic(pos, np, N, Ns, Box, grid);
      memcpy(dens_x, grid, sizeof(double) * 2 * tot);
      orc_fft_r2c(N, grid);
      nb = rp->pofk_nbins;
      orc_pofk(grid, N, Ns, Box, &nb, rp->pofk_bintype, rp->pofk_subtract_shotnoise, rp->pofk_kmin,
               rp->pofk_kmax, kbin, pk, kmean, nmodes);
      if (sd && rp->mg.nu) {
        /* massive neutrinos (auxPM.c:383-426): the outputs then hold the
         * total matter P(k) */
        orc_nu_add_density(rp->mg.nu, A, N, Box, grid, cdelta);
        nb = rp->pofk_nbins;
        orc_pofk(grid, N, Ns, Box, &nb, rp->pofk_bintype, rp->pofk_subtract_shotnoise, rp->pofk_kmin,
                 rp->pofk_kmax, kbin, pk, kmean, nmodes);
      }
      if (rp->stop_step > 0 && io == 0 && ts == rp->stop_step) {
        for (long p = 0; p < np; p++)
          for (int a = 0; a < 3; a++) {
            pos_out[3 * p + a] = pos[3 * p + a];
            vel_out[3 * p + a] = vel[3 * p + a] - sumv[a];
          }
        goto done;
      }
      if (rp->mg.mg_active) orc_fifth_force(&rp->mg, A, N, Box, dens_x, grid, mgk);
      orc_forces_kspace(grid, uses_mgk ? mgk : NULL, N, Box, f[0], f[1], f[2]);
      for (int a = 0; a < 3; a++) orc_fft_c2r(N, f[a]);
      double sumD[3];
      orc_interp(f[0], f[1], f[2], N, Box, pos, np, disp, sumD);
      if (sd) {
        /* main.c:487-503: [deltaD] into dDdy/dD2dy, [ddDddy] into D/D2 */
        orc_sd_field(c, cdelta, N, Ns, Box, A, AFF, ORC_FIELD_deltaD, 1, V1);
        orc_sd_field(c, cdelta2, N, Ns, Box, A, AFF, ORC_FIELD_deltaD, 2, V2);
        orc_sd_field(c, cdelta, N, Ns, Box, A, AFF, ORC_FIELD_ddDddy, 1, D1);
        orc_sd_field(c, cdelta2, N, Ns, Box, A, AFF, ORC_FIELD_ddDddy, 2, D2);
      }
      /* Kick (main.c:688-742); the scale-dependent Kick uses D + D2 */
      double dda = kick_dda(rp, c, AI, AF, A);
      orc_kick(np, vel, disp, D1, D2, sumD, rp->mg.omega, dda, sd ? 1.0 : orc_growth_ddDddy(c, A),
               sd ? 1.0 : orc_growth_ddD2ddy(c, A), A, rp->usecola, sumv);
      if (ts == 0 && io != 0) {
        /* output step (main.c:516-549): the last output ends the run; the
         * scale-dependent Output first puts [dDdy] into dDdy/dD2dy
         * (main.c:807-823) */
        if (sd) {
          orc_sd_field(c, cdelta, N, Ns, Box, A, AFF, ORC_FIELD_dDdy, 1, V1);
          orc_sd_field(c, cdelta2, N, Ns, Box, A, AFF, ORC_FIELD_dDdy, 2, V2);
        }
        double dDdy = orc_growth_dDdy(c, A), dD2dy = orc_growth_dD2dy(c, A);
        for (long p = 0; p < np; p++)
          for (int a = 0; a < 3; a++) {
            pos_out[3 * p + a] = pos[3 * p + a];
            double lpt = sd ? V1[3 * p + a] + V2[3 * p + a] : D1[3 * p + a] * dDdy + D2[3 * p + a] * dD2dy;
            vel_out[3 * p + a] = vel[3 * p + a] - sumv[a] + lpt * rp->usecola;
          }
        goto done;
      }
      /* Drift (main.c:747-787); the scale-dependent Drift adds dDdy + dD2dy,
       * which hold [deltaD] here */
      double dyyy = drift_dyyy(rp, c, A, AFF, AF);
      if (sd) {
        orc_drift(np, pos, vel, V1, V2, sumv, dyyy, 1.0, 1.0, rp->usecola, Box);
      } else {
        double dD = orc_growth_D(c, AFF) - Di, dD2 = orc_growth_D2(c, AFF) - Di2;
        orc_drift(np, pos, vel, D1, D2, sumv, dyyy, dD, dD2, rp->usecola, Box);
      }
      A = AFF;
      AI = AF;
      Di = orc_growth_D(c, A);
      Di2 = orc_growth_D2(c, A);
    }
  }
done:
  for (int a = 0; a < 3; a++) free(f[a]);
  free(grid); free(dens_x); free(mgk); free(D1); free(D2); free(pos); free(vel); free(disp);
  free(cdelta); free(cdelta2); free(V1); free(V2);
  orc_cosmo_free(c);
  return nb;
}

/* CPU baseline: IC (untimed) then `nsteps` KDK steps of the same loop body,
 * timed with the wall clock.  Returns seconds per step, or -1. */
#include <sys/time.h>
static double now_s(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

double orc_time_steps(const orc_run_params *rp, int nsteps) {
  const int N = rp->ic.N, Ns = rp->ic.Ns, NH = N / 2 + 1;
  const double Box = rp->ic.box;
  const long np = (long)Ns * Ns * Ns;
  const size_t tot = (size_t)N * N * NH;
  const int sd = rp->mg.scaledependent;
  orc_cosmo *c = orc_cosmo_create_sd(&rp->mg, rp->init_redshift, Box, N);
  double *D1 = malloc(8 * 3 * np), *D2 = malloc(8 * 3 * np), *pos = malloc(8 * 3 * np), *vel = calloc(3 * np, 8);
  double *disp = malloc(8 * 3 * np);
  /* scale-dependent build: stored delta(k), -source(k) and the per-step
   * fields, as orc_run */
  double *cdelta = NULL, *cdelta2 = NULL, *V1 = NULL, *V2 = NULL;
  if (sd) {
    cdelta = malloc(sizeof(double) * 2 * tot);
    cdelta2 = malloc(sizeof(double) * 2 * tot);
    V1 = malloc(8 * 3 * np);
    V2 = malloc(8 * 3 * np);
  }
  orc_ic_2lpt(&rp->ic, &rp->pw, D1, D2, cdelta, cdelta2);
  double A = 1.0 / (1.0 + rp->init_redshift);
  double Di = orc_growth_D(c, A), Di2 = orc_growth_D2(c, A);
  if (sd) {
    orc_sd_field(c, cdelta, N, Ns, Box, A, A, ORC_FIELD_D, 1, D1);
    orc_sd_field(c, cdelta2, N, Ns, Box, A, A, ORC_FIELD_D, 2, D2);
  }
  const double fD = sd ? 1.0 : Di, fD2 = sd ? 1.0 : Di2;
  for (long p = 0; p < np; p++) {
    long q[3] = {p / ((long)Ns * Ns), (p / Ns) % Ns, p % Ns};
    for (int a = 0; a < 3; a++)
      pos[3 * p + a] = orc_periodic_wrap(q[a] * (Box / (double)Ns) + D1[3 * p + a] * fD + D2[3 * p + a] * fD2, Box);
  }
  double *grid = malloc(sizeof(double) * 2 * tot), *dens_x = malloc(sizeof(double) * 2 * tot);
  double *mgk = malloc(sizeof(double) * 2 * tot), *f[3];
  for (int a = 0; a < 3; a++) f[a] = malloc(sizeof(double) * 2 * tot);
  int cap = rp->pofk_nbins > N ? rp->pofk_nbins : N;
  double *kb = malloc(8 * cap), *pk = malloc(8 * cap), *km = malloc(8 * cap), *nm = malloc(8 * cap);
  int uses_mgk = rp->mg.mg_active && (rp->mg.model == ORC_FOFR || rp->mg.model == ORC_MBETA || rp->mg.model == ORC_DGP);
  double da = step_da(rp, A, 1.0 / (1.0 + rp->final_redshift), rp->nsteps), AI = A, sumv[3];
  double t0 = now_s();
  for (int ts = 0; ts < nsteps; ts++) {
    double AF = step_mid(rp, A, da), AFF = step_end(rp, A, da);
    orc_cic(pos, np, N, Ns, Box, grid);
    memcpy(dens_x, grid, sizeof(double) * 2 * tot);
    orc_fft_r2c(N, grid);
    int nb = rp->pofk_nbins;
    orc_pofk(grid, N, Ns, Box, &nb, rp->pofk_bintype, rp->pofk_subtract_shotnoise, rp->pofk_kmin, rp->pofk_kmax, kb, pk,
             km, nm);
    if (sd && rp->mg.nu) {
      orc_nu_add_density(rp->mg.nu, A, N, Box, grid, cdelta);
      nb = rp->pofk_nbins;
      orc_pofk(grid, N, Ns, Box, &nb, rp->pofk_bintype, rp->pofk_subtract_shotnoise, rp->pofk_kmin, rp->pofk_kmax, kb,
               pk, km, nm);
    }
    if (rp->mg.mg_active) orc_fifth_force(&rp->mg, A, N, Box, dens_x, grid, mgk);
    orc_forces_kspace(grid, uses_mgk ? mgk : NULL, N, Box, f[0], f[1], f[2]);
    for (int a = 0; a < 3; a++) orc_fft_c2r(N, f[a]);
    double sumD[3];
    orc_interp(f[0], f[1], f[2], N, Box, pos, np, disp, sumD);
    if (sd) {
      orc_sd_field(c, cdelta, N, Ns, Box, A, AFF, ORC_FIELD_deltaD, 1, V1);
      orc_sd_field(c, cdelta2, N, Ns, Box, A, AFF, ORC_FIELD_deltaD, 2, V2);
      orc_sd_field(c, cdelta, N, Ns, Box, A, AFF, ORC_FIELD_ddDddy, 1, D1);
      orc_sd_field(c, cdelta2, N, Ns, Box, A, AFF, ORC_FIELD_ddDddy, 2, D2);
    }
    orc_kick(np, vel, disp, D1, D2, sumD, rp->mg.omega, kick_dda(rp, c, AI, AF, A), sd ? 1.0 : orc_growth_ddDddy(c, A),
             sd ? 1.0 : orc_growth_ddD2ddy(c, A), A, rp->usecola, sumv);
    if (sd)
      orc_drift(np, pos, vel, V1, V2, sumv, drift_dyyy(rp, c, A, AFF, AF), 1.0, 1.0, rp->usecola, Box);
    else
      orc_drift(np, pos, vel, D1, D2, sumv, drift_dyyy(rp, c, A, AFF, AF), orc_growth_D(c, AFF) - Di,
                orc_growth_D2(c, AFF) - Di2, rp->usecola, Box);
    A = AFF;
    AI = AF;
    Di = orc_growth_D(c, A);
    Di2 = orc_growth_D2(c, A);
  }
  double dt = (now_s() - t0) / (nsteps > 0 ? nsteps : 1);
  for (int a = 0; a < 3; a++) free(f[a]);
  free(grid); free(dens_x); free(mgk); free(D1); free(D2); free(pos); free(vel); free(disp);
  free(kb); free(pk); free(km); free(nm);
  free(cdelta); free(cdelta2); free(V1); free(V2);
  orc_cosmo_free(c);
  return dt;
}
