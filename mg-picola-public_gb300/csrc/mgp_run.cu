// The COLA time loop of main (src/main.c:394-611) with snapshot and P(k)
// output, on top of the step entry points of mgp_api.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <chrono>
#include <string>
#include <thread>
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

// The snapshot writers: snapshot k is written from pinned host slot k % 2 by
// a host thread while the GPU runs the next steps, so an output waits only
// for the writer of two snapshots before (whose slot it reuses).
struct out_slot {
  std::thread th;
  bool active = false;
  int rc = MGP_OK;
  std::string msg;
  double wait_ms = 0.0, file_ms = 0.0;  // this slot's last snapshot
};
struct out_writer {
  out_slot slot[2];
  int next = 0;             // slot of the next snapshot
  int count = 0;
  double wait_ms = 0.0;     // writers: waiting for the GPU to reach the snapshot and its download
  double file_ms = 0.0;     // writers: file writes
  double blocked_ms = 0.0;  // context's thread: output launches and waits for a writer
};

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int join_slot(out_writer *w, int k) {
  out_slot &o = w->slot[k];
  if (!o.active) return MGP_OK;
  const double t0 = now_ms();
  o.th.join();
  w->blocked_ms += now_ms() - t0;
  o.active = false;
  w->wait_ms += o.wait_ms;
  w->file_ms += o.file_ms;
  if (o.rc != MGP_OK) return mgp_set_error(o.rc, "%s", o.msg.c_str());
  return MGP_OK;
}

// Wait for every pending snapshot write; returns the first failure.
static int out_join(mgp_ctx *c) {
  out_writer *w = (out_writer *)c->out_writer;
  if (!w) return MGP_OK;
  const int r0 = join_slot(w, w->next), r1 = join_slot(w, w->next ^ 1);
  return r0 != MGP_OK ? r0 : r1;
}

// Snapshot statistics since the context was created (host milliseconds).
extern "C" int mgp_output_stats(mgp_ctx *c, int *count, double *wait_ms, double *file_ms, double *blocked_ms) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  const out_writer *w = (const out_writer *)c->out_writer;
  if (count) *count = w ? w->count : 0;
  if (wait_ms) *wait_ms = w ? w->wait_ms : 0.0;
  if (file_ms) *file_ms = w ? w->file_ms : 0.0;
  if (blocked_ms) *blocked_ms = w ? w->blocked_ms : 0.0;
  return MGP_OK;
}

int mgp_run_release(mgp_ctx *c) {
  int rc = out_join(c);
  delete (out_writer *)c->out_writer;
  c->out_writer = NULL;
  if (c->out_dev) cudaFree(c->out_dev);
  if (c->out_host) cudaFreeHost(c->out_host);
  for (int k = 0; k < 2; k++)
    if (c->out_ev[k]) cudaEventDestroy(c->out_ev[k]);
  if (c->out_stream) cudaStreamDestroy(c->out_stream);
  c->out_dev = c->out_host = NULL;
  c->out_ev[0] = c->out_ev[1] = NULL;
  c->out_stream = NULL;
  return rc;
}

static int out_buffers(mgp_ctx *c) {
  const size_t floats = 2 * 6 * (size_t)c->np;  // two slots of positions + velocities
  if (!c->out_writer) c->out_writer = new out_writer();
  if (!c->out_dev) MGP_CUDA(cudaMalloc(&c->out_dev, sizeof(float) * floats));
  if (!c->out_host) MGP_CUDA(cudaMallocHost(&c->out_host, sizeof(float) * floats));
  if (!c->out_stream) MGP_CUDA(cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking));
  for (int k = 0; k < 2; k++)
    if (!c->out_ev[k]) MGP_CUDA(cudaEventCreateWithFlags(&c->out_ev[k], cudaEventDisableTiming));
  return MGP_OK;
}

static int output(mgp_ctx *c, double A, double z, int gadget) {
  RET_IF(mgp_particles_canonical(c));  // snapshots list the particles in lattice order
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
  RET_IF(out_buffers(c));
  out_writer *w = (out_writer *)c->out_writer;
  const int k = w->next;
  RET_IF(join_slot(w, k));  // the writer of two snapshots before frees slot k
  const double t_enter = now_ms();
  float *d = c->out_dev + (size_t)k * 6 * np;
  float *h = c->out_host + (size_t)k * 6 * np;
  RET_IF(mgp_launch_output(c->s, c->v, L1, L2, lstride, lpitch, c->dstate, c->np, c->Ns, c->p.Box, u.lengthfac,
                           u.velfac * fac, dDdy, dD2dy, c->p.UseCOLA ? 1.0 : 0.0, d, d + 3 * np, c->stream));
  // download on the copy stream once the output kernel is done; the next
  // steps on the context's stream do not touch the staging slot
  cudaEvent_t ev = c->out_ev[k];
  MGP_CUDA(cudaEventRecord(ev, c->stream));
  MGP_CUDA(cudaStreamWaitEvent(c->out_stream, ev, 0));
  MGP_CUDA(cudaMemcpyAsync(h, d, 2 * bytes, cudaMemcpyDeviceToHost, c->out_stream));
  MGP_CUDA(cudaEventRecord(ev, c->out_stream));
  char fn[1200];
  mgp_snapshot_name(&c->p, z, fn, sizeof(fn));
  out_slot *o = &w->slot[k];
  o->rc = MGP_OK;
  o->msg.clear();
  const std::string path(fn);
  const float *pos = h, *vel = h + 3 * np;
  const mgp_params *p = &c->p;
  o->th = std::thread([o, path, ev, pos, vel, np, p, A, gadget]() {
    const double t0 = now_ms();
    cudaError_t e = cudaEventSynchronize(ev);
    const double t1 = now_ms();
    int rc = e == cudaSuccess ? MGP_OK : mgp_set_error(MGP_ECUDA, "output download: %s", cudaGetErrorString(e));
    if (rc == MGP_OK)
      rc = gadget ? mgp_write_gadget(path.c_str(), p, A, pos, vel, np) : mgp_write_ascii(path.c_str(), pos, vel, np);
    if (rc == MGP_OK) rc = mgp_write_info(p, A, np);
    if (rc != MGP_OK) o->msg = mgp_last_error();  // this thread's error string
    o->rc = rc;
    o->wait_ms = t1 - t0;
    o->file_ms = now_ms() - t1;
  });
  o->active = true;
  w->next = k ^ 1;
  w->count++;
  w->blocked_ms += now_ms() - t_enter;
  return MGP_OK;
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
  RET_IF((strcmp(label, "total") ? mgp_pofk : mgp_pofk_total)(c, nb, &nb, k.data(), pk.data(), km.data(), n.data()));
  return mgp_write_pofk(&c->p, A, label, nb, k.data(), pk.data(), km.data(), n.data());
}

static int run_loop(mgp_ctx *c, int gadget);

// The time loop; snapshot files are complete when it returns.
extern "C" int mgp_run(mgp_ctx *c, int gadget) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  const int rc = run_loop(c, gadget);
  const int wrc = out_join(c);
  return rc != MGP_OK ? rc : wrc;
}

static int run_loop(mgp_ctx *c, int gadget) {
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
      // steps in a for COLA, in ln a otherwise (stepDistr, main.c:75-81, 400-404)
      da = mgp_cosmo_step_da(p, A, ao, nsteps);
    }
    for (int ts = 0; ts < nsteps; ts++) {
      int output_step = (ts == 0) && (i != NoutputStart);
      AF = output_step ? A : mgp_cosmo_step_mid(p, A, da);
      AFF = mgp_cosmo_step_end(p, A, da);
      // RSD every step except at outputs (src/compute_pofk.c call in auxPM.c:376-381)
      if (c->p.pofk_compute_rsd_pofk == 1 && !output_step) RET_IF(write_rsd_now(c, A));
      RET_IF(mgp_get_displacements(c, A));
      if (p->pofk_compute_every_step) {
        RET_IF(write_pofk_now(c, A, "CDM"));
        if (c->cosmo.nu) RET_IF(write_pofk_now(c, A, "total"));  // src/auxPM.c:423-426
      }
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
        AF = mgp_cosmo_step_mid(p, A, da);
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
