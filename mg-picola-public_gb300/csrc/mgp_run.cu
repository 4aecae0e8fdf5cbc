// The COLA time loop of main (src/main.c:394-611) with snapshot and P(k)
// output, on top of the step entry points of mgp_api.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <vector>

#include "mgp_internal.h"
#include "mgp_io.h"

#define RET_IF(x)                  \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != MGP_OK) return rc_; \
  } while (0)

// Output (src/main.c:792-1061) at scale factor A for output redshift z.
static int write_rsd_now(mgp_ctx *c, double A);

static int output(mgp_ctx *c, double A, double z, int gadget) {
  // RSD multipoles at output (src/main.c:875-880), not for the IC output
  int first_step = fabs(c->p.Init_Redshift - z) / c->p.Init_Redshift <= 1.0E-6;
  if (c->p.pofk_compute_rsd_pofk >= 1 && !first_step) RET_IF(write_rsd_now(c, A));
  mgp_units u;
  mgp_units_init(&c->p, &u);
  const size_t np = (size_t)c->np, bytes = sizeof(float) * 3 * np;
  double fac = u.Hubble / pow(A, 1.5);
  double dDdy = mgp_cosmo_growth(&c->cosmo, 1, A), dD2dy = mgp_cosmo_growth(&c->cosmo, 4, A);
  const float *L1 = c->D1, *L2 = c->D2;
  long long lstride = c->np;
  int lpitch = c->Ns;
  if (c->sd) {
    // the scale-dependent Output first assigns [dDdy] (main.c:807-823)
    if (c->sd_kind[2] != MGP_FIELD_dDdy || c->sd_a[2] != A) {
      const int t = MGP_FIELD_dDdy;
      RET_IF(mgp_sd_fields(c, A, A, 1, &t));
    }
    L1 = L2 = c->sd_slot[2];
    dDdy = 1.0;
    dD2dy = 0.0;
    lstride = c->sd_grid;
    lpitch = c->sd_pitch;
  }
  float *d = NULL;
  MGP_CUDA(cudaMalloc(&d, 2 * bytes));
  std::vector<float> pos(3 * np), vel(3 * np);
  int rc = mgp_launch_output(c->s, c->v, L1, L2, lstride, lpitch, c->dstate, c->np, c->Ns, c->p.Box, u.lengthfac,
                             u.velfac * fac, dDdy, dD2dy, c->p.UseCOLA ? 1.0 : 0.0, d, d + 3 * np, c->stream);
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(pos.data(), d, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vel.data(), d + 3 * np, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = mgp_set_error(MGP_ECUDA, "output download: %s", cudaGetErrorString(e));
  }
  cudaFree(d);
  if (rc) return rc;
  char fn[1200];
  mgp_snapshot_name(&c->p, z, fn, sizeof(fn));
  RET_IF(gadget ? mgp_write_gadget(fn, &c->p, A, pos.data(), vel.data(), np)
                : mgp_write_ascii(fn, pos.data(), vel.data(), np));
  return mgp_write_info(&c->p, A, np);
}

static int write_rsd_now(mgp_ctx *c, double A) {
  int nb = c->pk_nbins;
  std::vector<double> k(nb), P0(nb), P2(nb), P4(nb), s0(nb), s2(nb), s4(nb), n(nb);
  RET_IF(mgp_pofk_rsd(c, A, nb, &nb, k.data(), P0.data(), P2.data(), P4.data(), s0.data(), s2.data(), s4.data(),
                      n.data()));
  return mgp_write_pofk_rsd(&c->p, A, nb, k.data(), P0.data(), P2.data(), P4.data(), s0.data(), s2.data(), s4.data(),
                            n.data());
}

static int write_pofk_now(mgp_ctx *c, double A, const char *label) {
  int nb = c->pk_nbins;
  std::vector<double> k(nb), pk(nb), km(nb), n(nb);
  RET_IF(mgp_pofk(c, nb, &nb, k.data(), pk.data(), km.data(), n.data()));
  return mgp_write_pofk(&c->p, A, label, nb, k.data(), pk.data(), km.data(), n.data());
}

extern "C" int mgp_run(mgp_ctx *c, int gadget) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  const mgp_params *p = &c->p;
  mkdir(p->OutputDir, 0755);
  RET_IF(mgp_displacement_fields(c));
  double A = 1.0 / (1.0 + p->Init_Redshift), AI = A, AF = A, AFF = A, da = 0.0;
  int NoutputStart = 0;
  const int Noutputs = p->Noutputs;
  if (((p->Init_Redshift - p->output_redshift[0]) / p->Init_Redshift <= 1.0E-6) || (p->Init_Redshift <= 1.0e-6)) {
    // output the initial conditions (main.c:327-351): v = 0, mean 0
    RET_IF(output(c, A, p->output_redshift[0], gadget));
    if (Noutputs == 1) return MGP_OK;
    NoutputStart++;
  }
  for (int i = NoutputStart; i <= Noutputs; i++) {
    int nsteps = 1;
    if (i != Noutputs) {
      nsteps = p->output_nsteps[i];
      double ao = 1.0 / (1.0 + p->output_redshift[i]);
      da = (ao - A) / (double)nsteps;  // stepDistr = 0 for COLA (main.c:75-81)
    }
    for (int ts = 0; ts < nsteps; ts++) {
      int output_step = (ts == 0) && (i != NoutputStart);
      AF = output_step ? A : A + da * 0.5;
      AFF = A + da;
      // RSD every step except at outputs (src/compute_pofk.c call in auxPM.c:376-381)
      if (c->p.pofk_compute_rsd_pofk == 1 && !output_step) RET_IF(write_rsd_now(c, A));
      RET_IF(mgp_get_displacements(c, A));
      if (p->pofk_compute_every_step) RET_IF(write_pofk_now(c, A, "CDM"));
      if (c->sd) {
        // scale-dependent fields of this step (main.c:487-503)
        const int types[2] = {MGP_FIELD_ddDddy, MGP_FIELD_deltaD};
        RET_IF(mgp_sd_fields(c, A, AFF, 2, types));
      }
      if (output_step) {
        RET_IF(mgp_kick_drift(c, AI, AF, A, AFF, 0));
        RET_IF(output(c, A, p->output_redshift[i - 1], gadget));
        if (i == Noutputs) return MGP_OK;
        // the RSD deposits used the force grids as scratch: rebuild them at A
        if (!c->have_forces) RET_IF(mgp_get_displacements(c, A));
        AI = A;
        AF = A + da * 0.5;
        RET_IF(mgp_kick_drift(c, AI, AF, A, AFF, 1));
      } else {
        RET_IF(mgp_kick_drift(c, AI, AF, A, AFF, 1));
      }
      A = AFF;
      AI = AF;
    }
  }
  return MGP_OK;
}
