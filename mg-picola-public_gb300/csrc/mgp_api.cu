// C ABI of the GB300 COLA library: context set-up, the PM step, the 2LPT IC
// and particle I/O.  See include/mgpicola.h for the reference interface each
// entry point replaces.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <cstddef>
#include <vector>

#include "mgp_internal.h"
#include "mgp_io.h"
#include "mgp_rng.h"

static thread_local char g_err[1024] = "";

extern "C" int mgp_set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char *mgp_last_error(void) { return g_err; }

#define RET_IF(x)          \
  do {                     \
    int rc_ = (x);         \
    if (rc_ != MGP_OK) return rc_; \
  } while (0)

// ----------------------------------------------------------------- timing
static const char *k_timer_names[MGP_NTIMERS] = {"cic",    "r2c",  "pofk",          "mg",         "forces",
                                                   "c2r",    "interp_kick_drift", "step", "lpt_fields", "closure",
                                                   "closure_conv", "fill", "sort"};

void mgp_tstart(mgp_ctx *c, int t) {
  if (c->timing) {
    cudaEventRecord(c->ev[t][0], c->stream);
    if (c->hev) {
      const int slot = c->hstep % c->hcap;
      cudaEventRecord(c->hev[((size_t)slot * MGP_NTIMERS + t) * 2], c->stream);
    }
  }
}
void mgp_tstop(mgp_ctx *c, int t);
static void tstart(mgp_ctx *c, int t) { mgp_tstart(c, t); }
static void tstop(mgp_ctx *c, int t) { mgp_tstop(c, t); }
void mgp_tstop(mgp_ctx *c, int t) {
  if (c->timing) {
    cudaEventRecord(c->ev[t][1], c->stream);
    c->timed[t] = 1;
    if (c->hev) {
      const int slot = c->hstep % c->hcap;
      cudaEventRecord(c->hev[((size_t)slot * MGP_NTIMERS + t) * 2 + 1], c->stream);
      c->htimed[(size_t)slot * MGP_NTIMERS + t] = 1;
    }
  }
}

static void free_history(mgp_ctx *c) {
  if (c->hev)
    for (int i = 0; i < c->hcap * MGP_NTIMERS * 2; i++)
      if (c->hev[i]) cudaEventDestroy(c->hev[i]);
  free(c->hev);
  free(c->htimed);
  c->hev = NULL;
  c->htimed = NULL;
  c->hcap = c->hstep = 0;
}

extern "C" int mgp_set_timing(mgp_ctx *c, int enable) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  c->timing = enable ? 1 : 0;
  for (int t = 0; t < MGP_NTIMERS; t++) c->timed[t] = 0;
  if (enable > 1) {
    // keep the stage events of the last `enable` steps
    if (c->hcap != enable) {
      MGP_CUDA(cudaStreamSynchronize(c->stream));
      free_history(c);
      const size_t ne = (size_t)enable * MGP_NTIMERS * 2;
      c->hev = (cudaEvent_t *)calloc(ne, sizeof(cudaEvent_t));
      c->htimed = (unsigned char *)calloc((size_t)enable * MGP_NTIMERS, 1);
      if (!c->hev || !c->htimed) {
        free_history(c);
        return mgp_set_error(MGP_ENOMEM, "timing history of %d steps", enable);
      }
      c->hcap = enable;
      for (size_t i = 0; i < ne; i++) MGP_CUDA(cudaEventCreate(&c->hev[i]));
    }
    memset(c->htimed, 0, (size_t)c->hcap * MGP_NTIMERS);
    c->hstep = 0;
  } else if (c->hev) {
    MGP_CUDA(cudaStreamSynchronize(c->stream));
    free_history(c);
  }
  return MGP_OK;
}

extern "C" double mgp_kernel_ms_step(mgp_ctx *c, const char *name, int step) {
  if (!c || !name || !c->hev || step < 0 || step >= c->hstep || step < c->hstep - c->hcap) return -1.0;
  const int slot = step % c->hcap;
  for (int t = 0; t < MGP_NTIMERS; t++) {
    if (strcmp(name, k_timer_names[t]) == 0) {
      if (!c->htimed[(size_t)slot * MGP_NTIMERS + t]) return -1.0;
      cudaEvent_t *e = c->hev + ((size_t)slot * MGP_NTIMERS + t) * 2;
      float ms = 0.f;
      if (cudaEventSynchronize(e[1]) != cudaSuccess) return -1.0;
      if (cudaEventElapsedTime(&ms, e[0], e[1]) != cudaSuccess) return -1.0;
      return ms;
    }
  }
  return -1.0;
}

extern "C" double mgp_kernel_ms(mgp_ctx *c, const char *name) {
  if (!c || !name) return -1.0;
  for (int t = 0; t < MGP_NTIMERS; t++) {
    if (strcmp(name, k_timer_names[t]) == 0) {
      if (!c->timed[t]) return -1.0;
      float ms = 0.f;
      cudaEventSynchronize(c->ev[t][1]);
      if (cudaEventElapsedTime(&ms, c->ev[t][0], c->ev[t][1]) != cudaSuccess) return -1.0;
      return ms;
    }
  }
  return -1.0;
}

extern "C" int mgp_set_particle_order(mgp_ctx *c, int tiles) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (c->nbox != 1 && tiles) return mgp_set_error(MGP_EINVAL, "a batch keeps the lattice order");
  MGP_CUDA(cudaSetDevice(c->device));
  if (tiles < 0 || tiles > 2) return mgp_set_error(MGP_EINVAL, "particle order %d (0, 1 or 2)", tiles);
  RET_IF(mgp_particles_canonical(c));
  c->tile_mode = tiles != 0;
  c->tile_kick = tiles == 2;
  return MGP_OK;
}

extern "C" int mgp_set_fft_mode(mgp_ctx *c, int mode) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (mode < 0 || mode > 1) return mgp_set_error(MGP_EINVAL, "FFT mode %d (0 or 1)", mode);
  c->fft_mode = mode;
  return MGP_OK;
}

// Whether this context's transforms take the strided passes of mgp_fft.cu.
static bool own_fft(const mgp_ctx *c) { return c->fft_mode && mgp_fft_supported(c); }

extern "C" int mgp_mark(mgp_ctx *c, int slot) {
  if (!c || slot < 0 || slot > 3) return mgp_set_error(MGP_EINVAL, "mark slot %d out of range", slot);
  MGP_CUDA(cudaEventRecord(c->ev_mark[slot], c->stream));
  return MGP_OK;
}

extern "C" double mgp_mark_ms(mgp_ctx *c, int from, int to) {
  if (!c || from < 0 || from > 3 || to < 0 || to > 3) return -1.0;
  float ms = 0.f;
  if (cudaEventSynchronize(c->ev_mark[to]) != cudaSuccess) return -1.0;
  if (cudaEventElapsedTime(&ms, c->ev_mark[from], c->ev_mark[to]) != cudaSuccess) return -1.0;
  return ms;
}

extern "C" long long mgp_launch_count(mgp_ctx *c) { return c ? mgp_kernel_launches() : -1; }


// P(k) binning blocks per box for a budget of per_sm blocks per SM.
static int pk_blocks_for(const mgp_ctx *c, int per_sm) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  long long nb = ((long long)sms * per_sm + c->nbox - 1) / c->nbox;
  const long long rows_blocks = ((long long)c->g.N * c->g.N + 7) / 8;
  if (nb > rows_blocks) nb = rows_blocks;
  if (nb < 1) nb = 1;
  return (int)nb;
}

// ----------------------------------------------------------- P(k) tables
// adjust_pofk_parameters (src/compute_pofk.c:758-805) in integer k units.
static void adjust_pofk(int N, int *nbins, int *bintype, int *sub, double *kmin, double *kmax) {
  if (!(*bintype == 0 || *bintype == 1)) *bintype = 0;
  if (!(*sub == 0 || *sub == 1)) *sub = 1;
  if (*nbins <= 0) *nbins = N;
  if (*kmax <= *kmin) {
    if (*bintype == 0) *kmin = 0.0;
    if (*bintype == 1) *kmin = 1.0;
    *kmax = (double)N;
  }
  if (*kmin < 0.0) {
    if (*bintype == 0) *kmin = 0.0;
    if (*bintype == 1) *kmin = 1.0;
  }
  if (*bintype == 1 && *kmin == 0.0) *kmin = 1.0;
  if (*kmax > sqrt(3.0) * (double)N) *kmax = (double)N;
}

// pofk_bin_index (src/compute_pofk.c:30-46)
static int pofk_bin_index(double kmag, double kmin, double kmax, int nbins, int bintype) {
  if (bintype == 0) return (int)((kmag - kmin) / (kmax - kmin) * nbins + 0.5);
  if (bintype == 1) {
    if (kmag <= 0.0) return -1;
    return (int)(log(kmag / kmin) / log(kmax / kmin) * nbins + 0.5);
  }
  return 0;
}

// k_from_index (src/compute_pofk.c:51-64)
static double k_from_index(int index, double kmin, double kmax, int nbins, int bintype, double box) {
  if (bintype == 0) return (kmin + (kmax - kmin) / (double)nbins * index) * 2.0 * M_PI / box;
  return exp(log(kmin) + log(kmax / kmin) / (double)nbins * index) * 2.0 * M_PI / box;
}

static int setup_pofk(mgp_ctx *c) {
  const int N = c->g.N;
  int nbins = c->p.pofk_nbins, bt = c->p.pofk_bintype, sub = c->p.pofk_subtract_shotnoise;
  double kmin = c->p.pofk_kmin * c->p.Box / (2.0 * M_PI), kmax = c->p.pofk_kmax * c->p.Box / (2.0 * M_PI);
  adjust_pofk(N, &nbins, &bt, &sub, &kmin, &kmax);
  if (nbins > 24576) return mgp_set_error(MGP_EINVAL, "pofk_nbins = %d exceeds 24576", nbins);
  c->pk_nbins = nbins;
  c->pk_bintype = bt;
  c->pk_sub = sub;
  c->pk_kmin = kmin;
  c->pk_kmax = kmax;
  const int h = N / 2;
  const int rkmax = 3 * h * h;
  std::vector<int> rkb(rkmax + 1);
  for (int rk = 0; rk <= rkmax; rk++) {
    int nk = pofk_bin_index(sqrt((double)rk), kmin, kmax, nbins, bt);
    rkb[rk] = (nk >= 0 && nk < nbins) ? nk : -1;
  }
  std::vector<float> win(h + 1);
  for (int d = 0; d <= h; d++) {
    double g = d == 0 ? 1.0 : sin((M_PI * d) / (double)N) / ((M_PI * d) / (double)N);
    win[d] = (float)(1.0 / pow(g, 4.0));
  }
  c->pk_n = (double *)calloc(nbins, sizeof(double));
  c->pk_k = (double *)calloc(nbins, sizeof(double));
  c->pk_host = (double *)calloc(nbins, sizeof(double));
  // geometric mode counts and |k| sums with the reference's weights
  for (int d0 = 0; d0 <= h; d0++) {
    double m0 = (d0 == 0 || d0 == h) ? 1.0 : 2.0;
    for (int d1 = 0; d1 <= h; d1++) {
      double m1 = (d1 == 0 || d1 == h) ? 1.0 : 2.0;
      for (int d2 = 0; d2 <= h; d2++) {
        int rk = d0 * d0 + d1 * d1 + d2 * d2;
        int b = rkb[rk];
        if (b < 0) continue;
        double w = m0 * m1 * ((d2 == 0 || d2 == h) ? 1.0 : 2.0);
        c->pk_n[b] += w;
        c->pk_k[b] += w * sqrt((double)rk);
      }
    }
  }
  MGP_CUDA(cudaMalloc(&c->rk_bin, sizeof(int) * (rkmax + 1)));
  MGP_CUDA(cudaMemcpy(c->rk_bin, rkb.data(), sizeof(int) * (rkmax + 1), cudaMemcpyHostToDevice));
  // first |k|^2 of each bin: the bin index is monotone in |k|^2 over one
  // contiguous range [rlo, rhi) and -1 outside it
  {
    int rlo = -1, rhi = 0;
    for (int rk = 0; rk <= rkmax; rk++)
      if (rkb[rk] >= 0) {
        if (rlo < 0) rlo = rk;
        rhi = rk + 1;
      }
    if (rlo < 0) rlo = rhi = 0;
    std::vector<int> thr(nbins + 1);
    int rk = rlo;
    for (int b = 0; b < nbins; b++) {
      while (rk < rhi && rkb[rk] < b) rk++;
      thr[b] = rk;
    }
    thr[nbins] = rhi;
    for (int q = rlo; q < rhi; q++)
      if (rkb[q] < 0) return mgp_set_error(MGP_EINVAL, "P(k) binning is not monotone in |k|");
    MGP_CUDA(cudaMalloc(&c->pk_thr, sizeof(int) * (nbins + 1)));
    MGP_CUDA(cudaMemcpy(c->pk_thr, thr.data(), sizeof(int) * (nbins + 1), cudaMemcpyHostToDevice));
  }
  MGP_CUDA(cudaMalloc(&c->win1d, sizeof(float) * (h + 1)));
  MGP_CUDA(cudaMemcpy(c->win1d, win.data(), sizeof(float) * (h + 1), cudaMemcpyHostToDevice));
  // enough warps to cover the SMs (4 blocks per SM; a batch shares that
  // budget among its boxes); each warp owns whole (i, j) rows.  The partial
  // buffer holds up to 16 blocks per SM for the batch autotuner.
  c->pk_blocks = pk_blocks_for(c, 4);
  c->pk_blocks_cap = pk_blocks_for(c, 16);
  MGP_CUDA(cudaMalloc(&c->pk_block, sizeof(double) * (size_t)c->pk_blocks_cap * nbins * c->nbox));
  MGP_CUDA(cudaMalloc(&c->pk_sum, sizeof(double) * nbins * c->nbox));
  return MGP_OK;
}

// ------------------------------------------------------------- lifecycle
static int make_plans(mgp_ctx *c) {
  const int N = c->g.N;
  long long n[3] = {N, N, N};
  long long rembed[3] = {N, N, c->g.P};
  long long cembed[3] = {N, N, c->g.NH};
  long long rdist = c->g.nreal, cdist = c->g.ncomplex;
  size_t ws[3] = {0, 0, 0};
  // single-grid plans only: a batch of three in-place C2R runs markedly
  // slower per grid (and needs a 3-grid work area) than three single calls
  cufftHandle *plans[3] = {&c->plan_r2c_oop, &c->plan_r2c_ip, &c->plan_c2r_1};
  for (int i = 0; i < 3; i++) {
    MGP_CUFFT(cufftCreate(plans[i]));
    MGP_CUFFT(cufftSetAutoAllocation(*plans[i], 0));
  }
  MGP_CUFFT(cufftMakePlanMany64(c->plan_r2c_oop, 3, n, rembed, 1, rdist, cembed, 1, cdist, CUFFT_R2C, 1, &ws[0]));
  MGP_CUFFT(cufftMakePlanMany64(c->plan_r2c_ip, 3, n, rembed, 1, rdist, cembed, 1, cdist, CUFFT_R2C, 1, &ws[1]));
  MGP_CUFFT(cufftMakePlanMany64(c->plan_c2r_1, 3, n, cembed, 1, cdist, rembed, 1, rdist, CUFFT_C2R, 1, &ws[2]));
  size_t w = 0;
  for (int i = 0; i < 3; i++) w = ws[i] > w ? ws[i] : w;
  // a batch also transforms all boxes per call (the force grids of one box
  // are three consecutive grids, so their batch stride is 3 grids)
  cufftHandle *bplans[4] = {&c->plan_r2c_oop_b, &c->plan_r2c_ip_b, &c->plan_c2r_b, &c->plan_c2r_frc_b};
  const int nbp = c->nbox > 1 ? 4 : 0;
  for (int i = 0; i < nbp; i++) {
    size_t wb = 0;
    MGP_CUFFT(cufftCreate(bplans[i]));
    MGP_CUFFT(cufftSetAutoAllocation(*bplans[i], 0));
    if (i < 2)
      MGP_CUFFT(cufftMakePlanMany64(*bplans[i], 3, n, rembed, 1, rdist, cembed, 1, cdist, CUFFT_R2C, c->nbox, &wb));
    else if (i == 2)
      MGP_CUFFT(cufftMakePlanMany64(*bplans[i], 3, n, cembed, 1, cdist, rembed, 1, rdist, CUFFT_C2R, c->nbox, &wb));
    else
      MGP_CUFFT(cufftMakePlanMany64(*bplans[i], 3, n, cembed, 1, 3 * cdist, rembed, 1, 3 * rdist, CUFFT_C2R, c->nbox,
                                    &wb));
    w = wb > w ? wb : w;
  }
  c->fft_work_bytes = w;
  if (w) MGP_CUDA(cudaMalloc(&c->fft_work, w));
  for (int i = 0; i < 3; i++) {
    MGP_CUFFT(cufftSetWorkArea(*plans[i], c->fft_work));
    MGP_CUFFT(cufftSetStream(*plans[i], c->stream));
  }
  for (int i = 0; i < nbp; i++) {
    MGP_CUFFT(cufftSetWorkArea(*bplans[i], c->fft_work));
    MGP_CUFFT(cufftSetStream(*bplans[i], c->stream));
  }
  return MGP_OK;
}

static int needs_mg1(const mgp_params *p) {
  if (!p->modified_gravity_active) return 0;
  if ((p->model == MGP_MODEL_FOFR || p->model == MGP_MODEL_MBETA)) return 1;
  if (p->model == MGP_MODEL_DGP && p->include_screening) return 1;
  return 0;
}

static int validate(const mgp_params *p) {
  if (p->Nmesh < 4 || p->Nmesh % 2) return mgp_set_error(MGP_EINVAL, "Nmesh = %d must be even and >= 4", p->Nmesh);
  if (p->Nmesh > 4096) return mgp_set_error(MGP_EINVAL, "Nmesh = %d exceeds 4096", p->Nmesh);
  if (p->Nsample < 1 || p->Nsample > 2048) return mgp_set_error(MGP_EINVAL, "Nsample = %d out of range", p->Nsample);
  if (!(p->Box > 0)) return mgp_set_error(MGP_EINVAL, "Box must be positive");
  if (p->model < 0 || p->model > 4) return mgp_set_error(MGP_EINVAL, "unknown model %d", p->model);
  if (p->scaledependent && p->Nsample % 2)
    return mgp_set_error(MGP_EINVAL, "scale-dependent growth needs an even Nsample (Nsample = %d)", p->Nsample);
  if ((p->WhichSpectrum != 0) && (p->WhichTransfer != 0))
    return mgp_set_error(MGP_EINVAL, "can't run with both power spectrum and transfer function");
  if ((p->WhichSpectrum == 0) && (p->WhichTransfer == 0))
    return mgp_set_error(MGP_EINVAL, "can't run with neither power spectrum nor transfer function");
  return MGP_OK;
}

extern "C" int mgp_destroy(mgp_ctx *c) {
  if (!c) return MGP_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  mgp_run_release(c);  // a snapshot write still in flight
  cufftHandle plans[7] = {c->plan_r2c_oop, c->plan_r2c_ip, c->plan_c2r_1, c->plan_r2c_oop_b, c->plan_r2c_ip_b,
                          c->plan_c2r_b, c->plan_c2r_frc_b};
  for (int i = 0; i < 7; i++)
    if (plans[i]) cufftDestroy(plans[i]);
  mgp_fft_free(c);
  mgp_sd_free(c);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  for (int q = 0; q < 2; q++)
    if (c->bev[q]) cudaEventDestroy(c->bev[q]);
  if (c->box_bs) cudaFree(c->box_bs);
  if (c->pk_hist) cudaFree(c->pk_hist);
  if (c->box_cosmo) {
    for (int b = 1; b < c->nbox; b++) mgp_cosmo_free(&c->box_cosmo[b]);
    free(c->box_cosmo);
  }
  free(c->box_p);
  void *bufs[] = {c->ic_scratch, c->s, c->v, c->D1, c->D2, c->dstate, c->partials, c->stage, c->rho, c->dk, c->frc, c->mg1,
                  c->fft_work, c->rk_bin, c->pk_thr, c->win1d, c->pk_block, c->pk_sum, c->rsd_block, c->rsd_sum,
                  c->pk_sum_tot, c->nu_tab_d, c->nu_row_d, c->nu_x_d, c->nu_den_d, c->scr_tab};
  for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++)
    if (bufs[i]) cudaFree(bufs[i]);
  if (c->nu_row_h) cudaFreeHost(c->nu_row_h);
  for (int q = 0; q < 2; q++)
    if (c->nu_ev[q]) cudaEventDestroy(c->nu_ev[q]);
  for (int k = 0; k < MGP_POS_CHUNKS; k++)
    if (c->ev_chunk[k]) cudaEventDestroy(c->ev_chunk[k]);
  free_history(c);
  mgp_tiles_free(c);
  for (int t = 0; t < MGP_NTIMERS; t++) {
    if (t < 4 && c->ev_mark[t]) cudaEventDestroy(c->ev_mark[t]);
    if (c->ev[t][0]) cudaEventDestroy(c->ev[t][0]);
    if (c->ev[t][1]) cudaEventDestroy(c->ev[t][1]);
  }
  if (c->side) cudaStreamDestroy(c->side);
  for (int q = 0; q < 2; q++)
    if (c->ev_side[q]) cudaEventDestroy(c->ev_side[q]);
  if (c->stream) cudaStreamDestroy(c->stream);
  free(c->pk_n);
  free(c->pk_k);
  free(c->pk_host);
  mgp_cosmo_free(&c->cosmo);
  free(c);
  return MGP_OK;
}

// Parameters of box b of a batch: the common set with the box's overrides.
static mgp_params box_params(const mgp_params *p, const mgp_box_params *bp) {
  mgp_params q = *p;
  q.Seed = bp->Seed;
  q.inverted_initial_condition = bp->inverted_initial_condition;
  q.amplitude_fixed_initial_condition = bp->amplitude_fixed_initial_condition;
  if (bp->fofr0 > 0) q.fofr0 = bp->fofr0;
  if (bp->rcH0_DGP > 0) q.rcH0_DGP = bp->rcH0_DGP;
  return q;
}

static const mgp_cosmo *cosmo_of(const mgp_ctx *c, int b) { return b == 0 ? &c->cosmo : &c->box_cosmo[b]; }

static int create_impl(const mgp_params *p, int nbox, const mgp_box_params *boxes, int device, mgp_ctx **out,
                       const mgp_model_hooks *hooks = NULL) {
  if (!p || !out) return mgp_set_error(MGP_EINVAL, "null argument");
  *out = NULL;
  RET_IF(validate(p));
  if (nbox < 1 || nbox > 65535) return mgp_set_error(MGP_EINVAL, "nbox = %d out of range", nbox);
  if (nbox > 1 && p->scaledependent)
    return mgp_set_error(MGP_EINVAL, "a batch of boxes runs scale-independent growth only");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return mgp_set_error(MGP_ECUDA, "no CUDA device available: the library has no CPU path");
  if (device < 0 || device >= ndev) return mgp_set_error(MGP_EINVAL, "device %d out of range", device);
  mgp_ctx *c = (mgp_ctx *)calloc(1, sizeof(mgp_ctx));
  c->nbox = nbox;
  c->box_p = (mgp_params *)calloc(nbox, sizeof(mgp_params));
  for (int b = 0; b < nbox; b++) c->box_p[b] = boxes ? box_params(p, &boxes[b]) : *p;
  c->p = c->box_p[0];
  c->device = device;
  c->tile_mode = nbox == 1;
  c->tile_kick = nbox == 1;
  c->fft_mode = 1;
  char err[512] = "";
  int rc = mgp_cosmo_init_hooks(&c->cosmo, &c->box_p[0], hooks, err, sizeof(err));
  if (rc) {
    free(c->box_p);
    free(c);
    return mgp_set_error(rc, "%s", err);
  }
  if (nbox > 1) {
    c->box_cosmo = (mgp_cosmo *)calloc(nbox, sizeof(mgp_cosmo));
    for (int b = 1; b < nbox && rc == MGP_OK; b++) {
      rc = mgp_cosmo_init(&c->box_cosmo[b], &c->box_p[b], err, sizeof(err));
      if (rc == MGP_OK && c->box_cosmo[b].p.Omega != c->cosmo.p.Omega) {
        snprintf(err, sizeof(err), "the boxes of a batch must share the background (box %d)", b);
        rc = MGP_EINVAL;
      }
    }
    if (rc) {
      std::string e = err;
      mgp_destroy(c);
      return mgp_set_error(rc, "%s", e.c_str());
    }
  }
  // the Brans-Dicke background solve replaces Omega and h (init_modified_version,
  // src/user_defined_functions.h:135-143); the time step uses the new values
  c->p.Omega = c->cosmo.p.Omega;
  c->p.HubbleParam = c->cosmo.p.HubbleParam;
#define TRY(x)            \
  do {                    \
    int r_ = (x);         \
    if (r_ != MGP_OK) {   \
      std::string e_ = g_err; \
      mgp_destroy(c);     \
      mgp_set_error(r_, "%s", e_.c_str()); \
      return r_;          \
    }                     \
  } while (0)
#define TRYCUDA(x) TRY([&]() -> int { MGP_CUDA(x); return MGP_OK; }())
  TRYCUDA(cudaSetDevice(device));
  TRYCUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (int t = 0; t < MGP_NTIMERS; t++) {
    if (t < 4) TRYCUDA(cudaEventCreate(&c->ev_mark[t]));
    TRYCUDA(cudaEventCreate(&c->ev[t][0]));
    TRYCUDA(cudaEventCreate(&c->ev[t][1]));
  }
  const int N = p->Nmesh;
  c->g.N = N;
  c->g.NH = N / 2 + 1;
  c->g.P = 2LL * (N / 2 + 1);
  c->g.nreal = (long long)N * N * c->g.P;
  c->g.ncomplex = (long long)N * N * c->g.NH;
  c->Ns = p->Nsample;
  c->np = (long long)p->Nsample * p->Nsample * p->Nsample;
  const size_t pbytes = sizeof(float) * 3 * (size_t)c->np * nbox;
  TRYCUDA(cudaMalloc(&c->s, pbytes));
  TRYCUDA(cudaMalloc(&c->v, pbytes));
  TRYCUDA(cudaMemset(c->s, 0, pbytes));
  TRYCUDA(cudaMemset(c->v, 0, pbytes));
  if (!p->scaledependent) {
    // scale-dependent runs keep their LPT fields in the lattice slots instead
    TRYCUDA(cudaMalloc(&c->D1, pbytes));
    TRYCUDA(cudaMalloc(&c->D2, pbytes));
    TRYCUDA(cudaMemset(c->D1, 0, pbytes));
    TRYCUDA(cudaMemset(c->D2, 0, pbytes));
  }
  TRYCUDA(cudaMalloc(&c->dstate, sizeof(mgp_dstate) * nbox));
  TRYCUDA(cudaMemset(c->dstate, 0, sizeof(mgp_dstate) * nbox));
  c->max_blocks = mgp_ikd_blocks(c->np) > 4096 ? mgp_ikd_blocks(c->np) : 4096;
  TRYCUDA(cudaMalloc(&c->partials, sizeof(double) * 6 * (size_t)c->max_blocks * nbox));
  const size_t gbytes = sizeof(float) * (size_t)c->g.nreal * nbox;
  TRYCUDA(cudaMalloc(&c->rho, gbytes));
  TRYCUDA(cudaMalloc(&c->dk, gbytes));
  TRYCUDA(cudaMalloc(&c->frc, 3 * gbytes));
  if (needs_mg1(p)) TRYCUDA(cudaMalloc(&c->mg1, gbytes));
  TRY(make_plans(c));
  TRY(setup_pofk(c));
  c->tune[0] = c->tune[1] = c->tune[2] = MGP_BUDGET_DEFAULT;  // deposit, grid passes, kick
  c->tune[3] = 4;                                             // P(k) binning
  if (p->scaledependent) TRY(mgp_sd_alloc(c));
  if (nbox > 1) {
    TRYCUDA(cudaEventCreate(&c->bev[0]));
    TRYCUDA(cudaEventCreate(&c->bev[1]));
  }
#undef TRYCUDA
#undef TRY
  *out = c;
  return MGP_OK;
}

extern "C" int mgp_create(const mgp_params *p, int device, mgp_ctx **out) {
  return create_impl(p, 1, NULL, device, out);
}

extern "C" int mgp_create_with_hooks(const mgp_params *p, const mgp_model_hooks *hooks, int device, mgp_ctx **out) {
  return create_impl(p, 1, NULL, device, out, hooks);
}

extern "C" int mgp_batch_create(const mgp_params *p, int nbox, const mgp_box_params *boxes, int device,
                                mgp_ctx **out) {
  if (!boxes) return mgp_set_error(MGP_EINVAL, "null box list");
  return create_impl(p, nbox, boxes, device, out);
}

// ---------------------------------------------------------------- IC
// displacement_fields + the particle assignment of main.c:231-309 for box b
// (single-grid transforms; box b's particle arrays and state).
// 2LPT initial conditions of box bx (displacement_fields, src/2LPT.c:185-495,
// 1209-1519): delta(k) from the Gaussian draw, or, given pos01 (particles in
// [0,1) of the box, the ReadParticlesFromFile path of
// src/readICfromfile.c:533-777), from the particles' density; then the 2LPT
// fields, the lattice read-out and the particle state.
static int ic_box(mgp_ctx *c, int bx, const double *pos01 = NULL, size_t npos = 0) {
  const mgp_params *pb = &c->box_p[bx];
  const mgp_cosmo *cb = cosmo_of(c, bx);
  float *dkb = c->dk + (size_t)bx * c->g.nreal;
  const size_t po = (size_t)bx * 3 * c->np;
  const int N = c->g.N, Ns = c->Ns, h = N / 2;
  const double box = pb->Box;
  // seed table, src/2LPT.c:262-271
  std::vector<uint32_t> seeds((size_t)N * N);
  {
    uint64_t n = 0;
    uint32_t sd = (uint32_t)pb->Seed;
    auto draw = [&]() { return (uint32_t)(0x7fffffff * mgp_uniform(sd, n++)); };
    for (int i = 0; i < N / 2; i++) {
      for (int j = 0; j < i; j++) seeds[(size_t)i * N + j] = draw();
      for (int j = 0; j < i + 1; j++) seeds[(size_t)j * N + i] = draw();
      for (int j = 0; j < i; j++) seeds[(size_t)(N - 1 - i) * N + j] = draw();
      for (int j = 0; j < i + 1; j++) seeds[(size_t)(N - 1 - j) * N + i] = draw();
      for (int j = 0; j < i; j++) seeds[(size_t)i * N + (N - 1 - j)] = draw();
      for (int j = 0; j < i + 1; j++) seeds[(size_t)j * N + (N - 1 - i)] = draw();
      for (int j = 0; j < i; j++) seeds[(size_t)(N - 1 - i) * N + (N - 1 - j)] = draw();
      for (int j = 0; j < i + 1; j++) seeds[(size_t)(N - 1 - j) * N + (N - 1 - i)] = draw();
    }
  }
  // amplitude per integer |k|^2 (k in h/Mpc = 2 pi/Box sqrt(RK)), with the
  // P(k) rescaling for MG runs whose input spectrum is LCDM (2LPT.c:323-327,
  // 395-407): mg_pofk_ratio(k, 1), per k when the growth is scale dependent
  const int rkmax = 3 * h * h;
  std::vector<double> amp(rkmax + 1), kk(rkmax + 1), ratio(rkmax + 1, 1.0);
  for (int rk = 0; rk <= rkmax; rk++) kk[rk] = 2.0 * M_PI / box * sqrt((double)rk);
  double s8fac = 1.0;
  if (pb->modified_gravity_active && pb->input_pofk_is_for_lcdm) {
    mgp_cosmo_pofk_ratio_many(cb, 1.0, rkmax, kk.data() + 1, ratio.data() + 1);
    if (!pb->input_sigma8_is_for_lcdm) {
      double e = mgp_cosmo_sigma8_enh(cb, 1.0);
      s8fac = 1.0 / (e * e);
    }
  }
  for (int rk = 0; rk <= rkmax; rk++) {
    double pk = rk == 0 ? 0.0 : mgp_cosmo_power(cb, kk[rk]) * ratio[rk] * s8fac;
    amp[rk] = pow(box, -1.5) * sqrt(pk);
  }
  // cube cut of 2LPT.c:383-386 with the reference's double expression
  std::vector<unsigned char> cut(h + 1);
  for (int d = 0; d <= h; d++) {
    double kv = d * 2 * 3.14159265358979323846 / box;
    cut[d] = (fabs(kv) * box / (2 * 3.14159265358979323846) > Ns / 2) ? 1 : 0;
  }
  uint32_t *d_seeds = NULL;
  double *d_amp = NULL;
  unsigned char *d_cut = NULL;
  float *g6 = NULL;
  int rc = MGP_OK;
  const long long gf = c->g.nreal;
  const double Di = mgp_cosmo_growth(cb, 0, 1.0 / (1.0 + pb->Init_Redshift));
  const double Di2 = mgp_cosmo_growth(cb, 3, 1.0 / (1.0 + pb->Init_Redshift));
  // without COLA the particles start with the 2LPT velocity (main.c:276-283)
  const double vD = pb->UseCOLA ? 0.0 : mgp_cosmo_growth(cb, 1, 1.0 / (1.0 + pb->Init_Redshift));
  const double vD2 = pb->UseCOLA ? 0.0 : mgp_cosmo_growth(cb, 4, 1.0 / (1.0 + pb->Init_Redshift));
  const int nblk = mgp_ikd_blocks(c->np);
#define CK(x)                      \
  do {                             \
    rc = (x);                      \
    if (rc != MGP_OK) goto cleanup; \
  } while (0)
#define CKC(x)                                                                                           \
  do {                                                                                                   \
    cudaError_t e_ = (x);                                                                                \
    if (e_ != cudaSuccess) {                                                                             \
      rc = mgp_set_error(MGP_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));   \
      goto cleanup;                                                                                      \
    }                                                                                                    \
  } while (0)
#define CKF(x)                                                                                         \
  do {                                                                                                 \
    cufftResult r_ = (x);                                                                              \
    if (r_ != CUFFT_SUCCESS) {                                                                         \
      rc = mgp_set_error(MGP_ECUFFT, "%s:%d %s: cufft error %d", __FILE__, __LINE__, #x, (int)r_);   \
      goto cleanup;                                                                                    \
    }                                                                                                  \
  } while (0)
  CKC(cudaMalloc(&d_seeds, sizeof(uint32_t) * seeds.size()));
  CKC(cudaMalloc(&d_amp, sizeof(double) * amp.size()));
  CKC(cudaMalloc(&d_cut, cut.size()));
  // six scratch grids for the displacement gradients and the six
  // displacement fields (2LPT.c:1214-1219, 1300-1306), kept by the context
  // for its next IC (runs of many ICs -- the boxes of a batch, repeated
  // runs -- allocate them once)
  if (!c->ic_scratch) CKC(cudaMalloc(&c->ic_scratch, sizeof(float) * 6 * (size_t)gf));
  g6 = c->ic_scratch;
  CKC(cudaMemcpyAsync(d_seeds, seeds.data(), sizeof(uint32_t) * seeds.size(), cudaMemcpyHostToDevice, c->stream));
  CKC(cudaMemcpyAsync(d_amp, amp.data(), sizeof(double) * amp.size(), cudaMemcpyHostToDevice, c->stream));
  CKC(cudaMemcpyAsync(d_cut, cut.data(), cut.size(), cudaMemcpyHostToDevice, c->stream));
  if (pos01) {
    // the particles' CIC density at a_i as the LCDM linear field, brought to
    // a = 1 (readICfromfile.c:640-676), deconvolved and rescaled (701-777)
    std::vector<double> gcw(h + 1), resc(rkmax + 1);
    for (int d = 0; d <= h; d++) {
      const double x = M_PI * d / (double)N, sc = d == 0 ? 1.0 : sin(x) / x;
      gcw[d] = 1.0 / (sc * sc);
    }
    {
      std::vector<double> r2(rkmax + 1, 1.0);
      mgp_cosmo_pofk_ratio_many(cb, 1.0, rkmax, kk.data() + 1, r2.data() + 1);
      const double s8 = pb->input_sigma8_is_for_lcdm ? 1.0 : mgp_cosmo_sigma8_enh(cb, 1.0);
      for (int rk = 0; rk <= rkmax; rk++) resc[rk] = sqrt(r2[rk]) / s8;
    }
    const double normfac = 1.0 / ((double)N * N * N) / mgp_cosmo_growth(cb, 6, 1.0 / (1.0 + pb->Init_Redshift));
    struct dbuf {  // freed on every exit from this block
      double *p = NULL;
      ~dbuf() {
        if (p) cudaFree(p);
      }
    } b_pos, b_gc, b_resc;
    CKC(cudaMalloc(&b_pos.p, sizeof(double) * 3 * npos));
    CKC(cudaMalloc(&b_gc.p, sizeof(double) * gcw.size()));
    CKC(cudaMalloc(&b_resc.p, sizeof(double) * resc.size()));
    double *d_pos = b_pos.p, *d_gc = b_gc.p, *d_resc = b_resc.p;
    CKC(cudaMemcpyAsync(d_pos, pos01, sizeof(double) * 3 * npos, cudaMemcpyHostToDevice, c->stream));
    CKC(cudaMemcpyAsync(d_gc, gcw.data(), sizeof(double) * gcw.size(), cudaMemcpyHostToDevice, c->stream));
    CKC(cudaMemcpyAsync(d_resc, resc.data(), sizeof(double) * resc.size(), cudaMemcpyHostToDevice, c->stream));
    rc = mgp_launch_fill(c->rho, gf, -1.0f, c->stream);
    if (rc == MGP_OK)
      rc = mgp_launch_cic_unit(d_pos, (long long)npos, N, c->g.P, (float)pow((double)N / Ns, 3), c->rho, c->stream);
    if (rc == MGP_OK && cufftExecR2C(c->plan_r2c_oop, (cufftReal *)c->rho, (cufftComplex *)dkb) != CUFFT_SUCCESS)
      rc = mgp_set_error(MGP_ECUFFT, "IC density transform");
    if (rc == MGP_OK) rc = mgp_launch_ic_from_density(dkb, N, Ns, normfac, d_gc, d_resc, c->stream);
    cudaStreamSynchronize(c->stream);
    if (rc != MGP_OK) goto cleanup;
  } else {
    CKC(cudaMemsetAsync(dkb, 0, sizeof(float) * (size_t)gf, c->stream));
    CK(mgp_launch_ic_delta(d_seeds, d_amp, d_cut, N, Ns, box, pb->amplitude_fixed_initial_condition,
                           pb->inverted_initial_condition, pb->SphereMode == 1, dkb, c->stream));
  }
  CK(mgp_launch_ic_grad6(dkb, g6, gf, N, c->stream));
  for (int g = 0; g < 3; g++) CKF(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)(g6 + g * gf), (cufftReal *)(g6 + g * gf)));
  for (int g = 3; g < 6; g++) CKF(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)(g6 + g * gf), (cufftReal *)(g6 + g * gf)));
  CK(mgp_launch_ic_source(g6, gf, N, c->g.P, c->stream));
  CKF(cufftExecR2C(c->plan_r2c_ip, (cufftReal *)(g6 + 3 * gf), (cufftComplex *)(g6 + 3 * gf)));
  if (c->sd) {
    // SCALEDEPENDENT: keep delta(k) and the source (2LPT.c:1336-1344), then
    // x = q + D + D2 and v = dDdy + dD2dy (or 0) at a_i (main.c:244-307)
    const double Ai = 1.0 / (1.0 + c->p.Init_Redshift);
    const int types[2] = {MGP_FIELD_D, MGP_FIELD_dDdy};
    CK(mgp_sd_store(c, c->dk, g6 + 3 * gf));
    CK(mgp_sd_fields(c, Ai, Ai, 2, types));
    CK(mgp_sd_init_particles(c));
    CKC(cudaMemsetAsync(c->dstate, 0, sizeof(mgp_dstate), c->stream));
    CKC(cudaStreamSynchronize(c->stream));
    c->have_density = c->have_forces = 0;
    goto cleanup;
  }
  CK(mgp_launch_ic_disp(dkb, g6 + 3 * gf, g6, gf, N, box, c->stream));
  for (int g = 0; g < 3; g++) CKF(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)(g6 + g * gf), (cufftReal *)(g6 + g * gf)));
  for (int g = 3; g < 6; g++) CKF(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)(g6 + g * gf), (cufftReal *)(g6 + g * gf)));
  CK(mgp_launch_ic_readout(g6, gf, N, c->g.P, Ns, c->D1 + po, c->D2 + po, c->partials, nblk, c->stream));
  CK(mgp_launch_ic_finish(c->D1 + po, c->D2 + po, c->s + po, c->v + po, c->np, c->partials, nblk, (float)Di,
                          (float)Di2, (float)vD, (float)vD2, c->stream));
  c->lpt_ver++;  // new D1/D2
  CKC(cudaMemsetAsync(c->dstate + bx, 0, sizeof(mgp_dstate), c->stream));
  CKC(cudaStreamSynchronize(c->stream));
  c->have_density = c->have_forces = 0;
cleanup:
  if (d_seeds) cudaFree(d_seeds);
  if (d_amp) cudaFree(d_amp);
  if (d_cut) cudaFree(d_cut);
  (void)g6;  // the context's IC scratch, freed by mgp_destroy
#undef CK
#undef CKC
#undef CKF
  return rc;
}

extern "C" int mgp_displacement_fields(mgp_ctx *c) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (c->nbox != 1) return mgp_set_error(MGP_ESTATE, "single-box call on a batch of %d boxes", c->nbox);
  MGP_CUDA(cudaSetDevice(c->device));
  // the IC writes every particle array in lattice order
  c->permuted = 0;
  c->tile_ready = 0;
  if (c->p.ReadParticlesFromFile) {
    // ReadFilesMakeDisplacementField (src/readICfromfile.c:533-699)
    double *pos = NULL;
    size_t n = 0;
    RET_IF(mgp_read_particle_files(&c->p, &pos, &n));
    const int rc = ic_box(c, 0, pos, n);
    free(pos);
    return rc;
  }
  return ic_box(c, 0);
}

// The same from particles held by the caller: positions in Mpc/h, [n][3],
// wrapped into [0, Box).
extern "C" int mgp_displacement_fields_from_positions(mgp_ctx *c, const double *pos, size_t n) {
  if (!c || (!pos && n)) return mgp_set_error(MGP_EINVAL, "null argument");
  if (c->nbox != 1) return mgp_set_error(MGP_ESTATE, "single-box call on a batch of %d boxes", c->nbox);
  MGP_CUDA(cudaSetDevice(c->device));
  // the IC writes every particle array in lattice order
  c->permuted = 0;
  c->tile_ready = 0;
  std::vector<double> u(3 * n);
  const double inv = 1.0 / c->p.Box;
  for (size_t q = 0; q < 3 * n; q++) {
    double x = pos[q] * inv;
    x -= floor(x);
    if (x >= 1.0) x = 0.0;
    u[q] = x;
  }
  return ic_box(c, 0, u.data(), n);
}

// ------------------------------------------------------------ PM step
static int require_particles(mgp_ctx *c) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (c->nbox != 1) return mgp_set_error(MGP_ESTATE, "single-box call on a batch of %d boxes", c->nbox);
  MGP_CUDA(cudaSetDevice(c->device));
  return MGP_OK;
}

// A user's screening_factor_potential (density = 0, argument the Newtonian
// potential of mg1) or screening_factor_density (density = 1, argument the
// smoothed density of mg1) applied to rho through a table of the function at
// this a: MGP_SCREEN_TABLE values at t = asinh(u/u_s) uniform in [t0, t1],
// copied from pageable memory (the copy has been staged when it returns).
static int user_screening(mgp_ctx *c, double A, int density, double mult, long long nr) {
  const mgp_model_hooks *h = &c->cosmo.hooks;
  const int nt = MGP_SCREEN_TABLE;
  const double us = density ? 1.0 : 1e-8, t0 = density ? -1.5 : -25.0, t1 = density ? 20.0 : 25.0;
  const double dt = (t1 - t0) / (nt - 1);
  if (!c->scr_tab) MGP_CUDA(cudaMalloc(&c->scr_tab, sizeof(float) * nt));
  std::vector<float> tab(nt);
  for (int j = 0; j < nt; j++) {
    const double u = us * sinh(t0 + dt * j);
    tab[j] = (float)(density ? h->screening_factor_density(A, u, h->user) : h->screening_factor_potential(A, u, h->user));
  }
  MGP_CUDA(cudaMemcpyAsync(c->scr_tab, tab.data(), sizeof(float) * nt, cudaMemcpyHostToDevice, c->stream));
  return mgp_launch_screen_table(c->rho, c->mg1, nr, (float)mult, c->scr_tab, nt, us, t0, dt, c->stream);
}

// MG fifth force (ComputeFifthForce, src/user_defined_functions.h:687-719 and
// src/mg.h) given delta(x) in rho and delta(k) in dk.  Leaves the MG source
// for the force pass in rho (as complex) and returns the fused k-space mode.
static int fifth_force(mgp_ctx *c, double A, int filtered, int *mg_kind, float *coupling, float *mass2) {
  const mgp_params *p = &c->p;
  const int N = c->g.N;
  *mg_kind = 0;
  *coupling = 0.f;
  *mass2 = 0.f;
  if (!p->modified_gravity_active) return MGP_OK;
  const long long nr = c->g.nreal;
  if (p->model == MGP_MODEL_FOFR || p->model == MGP_MODEL_MBETA) {
    // ComputeFifthForce_PotentialScreening, src/mg.h:147-189
    if (p->include_screening) {
      double norm = 1.0 / pow((double)N, 3) * 1.5 * p->Omega / A * pow(p->Box / 2997.92458 / (2.0 * M_PI), 2);
      if (own_fft(c) && !filtered) {
        // the inverse Laplacian applied in the first inverse pass (mgp_fft.cu)
        RET_IF(mgp_fft_c2r_filtered(c, c->dk, c->mg1, 2, 0, 0.f, (float)norm));
      } else {
        if (!filtered) RET_IF(mgp_launch_div_laplacian(c->dk, c->mg1, N, (float)norm, c->stream));
        if (own_fft(c))
          RET_IF(mgp_fft_c2r(c, c->mg1));
        else
          MGP_CUFFT(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)c->mg1, (cufftReal *)c->mg1));
      }
      if (mgp_cosmo_user_screening(&c->cosmo, 0))
        RET_IF(user_screening(c, A, 0, 1.0, nr));
      else
        RET_IF(mgp_launch_screen_potential(c->rho, c->mg1, nr, (float)mgp_phicrit(&c->cosmo, A), c->stream));
    }
    if (own_fft(c))
      RET_IF(mgp_fft_r2c(c, c->rho, c->rho));
    else
      MGP_CUFFT(cufftExecR2C(c->plan_r2c_ip, (cufftReal *)c->rho, (cufftComplex *)c->rho));
    *mg_kind = 1;
    *coupling = (float)mgp_coupling(&c->cosmo, A);
    *mass2 = (float)(A * A * mgp_mass2_of_a(&c->cosmo, A) / pow(2.0 * M_PI * 2997.92458 / p->Box, 2));
  } else if (p->model == MGP_MODEL_DGP) {
    // ComputeFifthForce_DensityScreening, src/mg.h:197-260
    double coupling_d = mgp_coupling(&c->cosmo, A);
    if (!p->include_screening) {
      *mg_kind = 3;
      *coupling = (float)coupling_d;
      return MGP_OK;
    }
    double kR1 = 2.0 * M_PI / p->Box * p->Rsmooth;
    if (own_fft(c) && !filtered) {
      // the smoothing filter applied in the first inverse pass (mgp_fft.cu)
      RET_IF(mgp_fft_c2r_filtered(c, c->dk, c->mg1, 1, p->smoothing_filter, (float)kR1,
                                  (float)(1.0 / pow((double)N, 3))));
    } else {
      if (!filtered)
        RET_IF(mgp_launch_smooth(c->dk, c->mg1, N, p->smoothing_filter, (float)kR1,
                                 (float)(1.0 / pow((double)N, 3)), c->stream));
      if (own_fft(c))
        RET_IF(mgp_fft_c2r(c, c->mg1));
      else
        MGP_CUFFT(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)c->mg1, (cufftReal *)c->mg1));
    }
    // Without massive neutrinos delta(k) is the transform of rho itself, so
    // the screening pass writes delta + source, rho (1 + coupling S), and the
    // force pass reads that one spectrum (mg_kind 4) instead of delta(k) and
    // the source (the sum P3D + P3D_mg of auxPM.c:450-455, formed in real
    // space; the transform is linear)
    const int fold = !c->cosmo.nu && !mgp_cosmo_user_screening(&c->cosmo, 1);
    if (mgp_cosmo_user_screening(&c->cosmo, 1))
      RET_IF(user_screening(c, A, 1, coupling_d, nr));
    else
      RET_IF(mgp_launch_screen_density(c->rho, c->mg1, nr, (float)coupling_d,
                                       (float)mgp_dgp_screen_prefactor(&c->cosmo, A), c->stream, 1, NULL,
                                       fold ? 1.0f : 0.0f));
    if (own_fft(c))
      RET_IF(mgp_fft_r2c(c, c->rho, c->rho));
    else
      MGP_CUFFT(cufftExecR2C(c->plan_r2c_ip, (cufftReal *)c->rho, (cufftComplex *)c->rho));
    *mg_kind = fold ? 4 : 2;
  } else if (p->model == MGP_MODEL_BRANSDICKE) {
    // ComputeFifthForce_TimeDepGeffModels (src/mg.h:127-137): the source
    // is delta(k) Geff/G(a), applied inside the force pass
    *mg_kind = 3;
    *coupling = (float)(mgp_geff(&c->cosmo, A, 0.0) - 1.0);
  }
  return MGP_OK;
}

// k-space filter of the fifth force that can ride on the P(k) pass
// (both read delta(k) once): 1 smoothing for density screening, 2 inverse
// Laplacian for potential screening; 0 none.
static int mg_filter_kind(const mgp_params *p) {
  if (!p->modified_gravity_active || !p->include_screening) return 0;
  if (p->model == MGP_MODEL_DGP) return 1;
  if (p->model == MGP_MODEL_FOFR || p->model == MGP_MODEL_MBETA) return 2;
  return 0;
}

// P(k) sums of the current delta(k) into `sums` (c->pk_sum by default).
static int pofk_now(mgp_ctx *c, int fuse_kind, double A, double *sums = NULL) {
  const mgp_params *p = &c->p;
  const int N = c->g.N;
  float fa = 0.f, fb = 0.f;
  if (fuse_kind == 1) {
    fa = (float)(2.0 * M_PI / p->Box * p->Rsmooth);
    fb = (float)(1.0 / pow((double)N, 3));
  } else if (fuse_kind == 2) {
    fb = (float)(1.0 / pow((double)N, 3) * 1.5 * p->Omega / A * pow(p->Box / 2997.92458 / (2.0 * M_PI), 2));
  }
  RET_IF(mgp_launch_pofk_thr(c->dk, N, c->pk_thr, c->win1d, c->pk_nbins, c->pk_bintype, c->pk_kmin, c->pk_kmax,
                             c->pk_block, c->pk_blocks, sums ? sums : c->pk_sum, fuse_kind, p->smoothing_filter,
                             fuse_kind ? c->mg1 : NULL, fa, fb, c->stream));
  return MGP_OK;
}

// Massive neutrinos (src/auxPM.c:383-428).  The factor depends on |k|^2
// only: the host restricts the transfer table to this step's redshift (one
// row over the ln k nodes), uploads it before the step's first launch, and
// k_nu_table evaluates the factor for every integer |k|^2 on the device.
static int nu_prepare(mgp_ctx *c, double A) {
  const int N = c->g.N, h = N / 2;
  const int nrk = 3 * h * h + 1;
  if (!c->nu_row_h) {
    int nx = 0;
    const double *lnk = mgp_cosmo_nu_lnk(&c->cosmo, &nx);
    c->nu_nx = nx;
    MGP_CUDA(cudaMallocHost(&c->nu_row_h, sizeof(double) * 4 * nx));
    MGP_CUDA(cudaMalloc(&c->nu_row_d, sizeof(double) * 2 * nx));
    MGP_CUDA(cudaMalloc(&c->nu_x_d, sizeof(double) * nx));
    MGP_CUDA(cudaMalloc(&c->nu_den_d, sizeof(double) * nrk));
    MGP_CUDA(cudaMalloc(&c->nu_tab_d, sizeof(float) * nrk));
    for (int q = 0; q < 2; q++) MGP_CUDA(cudaEventCreateWithFlags(&c->nu_ev[q], cudaEventDisableTiming));
    std::vector<double> den(nrk);
    mgp_cosmo_nu_den(&c->cosmo, N, nrk, den.data());
    MGP_CUDA(cudaMemcpy(c->nu_den_d, den.data(), sizeof(double) * nrk, cudaMemcpyHostToDevice));
    MGP_CUDA(cudaMemcpy(c->nu_x_d, lnk, sizeof(double) * nx, cudaMemcpyHostToDevice));
  }
  const int nx = c->nu_nx;
  c->nu_slot ^= 1;
  double *row = c->nu_row_h + (size_t)c->nu_slot * 2 * nx;
  MGP_CUDA(cudaEventSynchronize(c->nu_ev[c->nu_slot]));  // its upload two steps ago is done
  mgp_cosmo_nu_row(&c->cosmo, A, row, row + nx);
  MGP_CUDA(cudaMemcpyAsync(c->nu_row_d, row, sizeof(double) * 2 * nx, cudaMemcpyHostToDevice, c->stream));
  MGP_CUDA(cudaEventRecord(c->nu_ev[c->nu_slot], c->stream));
  const mgp_cosmo *cs = &c->cosmo;
  const double fac = cs->OmegaNu / cs->p.Omega * (double)N * (double)N * (double)N;
  c->nu_cdmfac = (cs->p.Omega - cs->OmegaNu) / cs->p.Omega;
  return mgp_launch_nu_table(c->nu_tab_d, nrk, 2.0 * M_PI / cs->p.Box, fac, c->nu_x_d, c->nu_row_d, c->nu_row_d + nx, nx,
                             c->nu_den_d, c->stream);
}

// delta(k) becomes the total matter density, cdmfac delta_cdm(k) + the
// neutrino term grown from the stored IC field, and its P(k) ("total") is
// binned; that pass also writes the fifth-force filter output (fuse_kind),
// which the MG solver reads from the total field.
static int add_neutrinos(mgp_ctx *c, double A, int fuse_kind) {
  if (!c->sd_dk[0]) return mgp_set_error(MGP_ESTATE, "massive neutrinos need the scale-dependent IC field");
  RET_IF(mgp_launch_nu_add(c->dk, c->sd_dk[0], c->g.N, c->nu_cdmfac, c->nu_tab_d, c->stream));
  if (c->p.pofk_compute_every_step) {
    if (!c->pk_sum_tot) MGP_CUDA(cudaMalloc(&c->pk_sum_tot, sizeof(double) * c->pk_nbins));
    RET_IF(pofk_now(c, fuse_kind, A, c->pk_sum_tot));
  }
  return MGP_OK;
}

static int fields_from_density(mgp_ctx *c, double A);

extern "C" int mgp_get_displacements(mgp_ctx *c, double A) {
  RET_IF(require_particles(c));
  const int N = c->g.N;
  if (c->cosmo.nu) RET_IF(nu_prepare(c, A));
  // PtoMesh, src/auxPM.c:280-432
  const bool tiles = c->tile_mode && mgp_tile_side(N, c->np) > 0;
  if (tiles) {
    // bucket the particles by cell tile (mgp_tiles.cu) for the deposit and
    // the kick of this step
    tstart(c, T_SORT);
    RET_IF(mgp_tiles_sort(c, mgp_tile_side(N, c->np)));
    tstop(c, T_SORT);
  }
  // the tile deposit stores every cell of the mesh itself (owner writes),
  // the particle-order deposit adds to a mesh pre-set to -1
  tstart(c, T_FILL);
  if (!tiles) RET_IF(mgp_launch_fill(c->rho, c->g.nreal, -1.0f, c->stream));
  tstop(c, T_FILL);
  tstart(c, T_CIC);
  double wpar = pow((double)N / (double)c->Ns, 3);
  if (tiles)
    RET_IF(mgp_cic_tiles_own(c, (float)wpar));
  else
    RET_IF(mgp_launch_cic(c->s, c->dstate, c->np, c->Ns, N, c->p.Box, (float)wpar, c->rho, c->g.P, c->stream));
  tstop(c, T_CIC);
  return fields_from_density(c, A);
}

// The rest of GetDisplacements once the density is on the mesh: R2C, P(k),
// neutrinos, fifth force, forces and the three C2R.
static int fields_from_density(mgp_ctx *c, double A) {
  const int N = c->g.N;
  tstart(c, T_R2C);
  if (own_fft(c))
    RET_IF(mgp_fft_r2c(c, c->rho, c->dk));
  else
    MGP_CUFFT(cufftExecR2C(c->plan_r2c_oop, (cufftReal *)c->rho, (cufftComplex *)c->dk));
  tstop(c, T_R2C);
  c->have_density = 1;
  c->last_density_a = A;
  int fused = 0;
  if (c->p.pofk_compute_every_step) {
    // with massive neutrinos the fifth-force filter reads the total field:
    // it is fused into the total P(k) pass instead of the CDM one.  With the
    // y pass of mgp_fft.cu the filter rides on the first inverse pass of
    // the solver's transform instead (P(k) then only reads delta(k)).
    fused = own_fft(c) ? 0 : mg_filter_kind(&c->p);
    tstart(c, T_POFK);
    RET_IF(pofk_now(c, c->cosmo.nu ? 0 : fused, A));
    tstop(c, T_POFK);
  }
  if (c->cosmo.nu) RET_IF(add_neutrinos(c, A, fused));
  int mg_kind = 0;
  float coupling = 0.f, mass2 = 0.f;
  tstart(c, T_MG);
  RET_IF(fifth_force(c, A, fused, &mg_kind, &coupling, &mass2));
  tstop(c, T_MG);
  // Forces, src/auxPM.c:437-555
  if (own_fft(c) && !c->closure && (mg_kind == 0 || mg_kind == 3 || mg_kind == 4)) {
    // one spectrum: the force pass fused into the inverse x and y passes
    // (mgp_fft.cu); nDGP without screening scales delta by 1 + coupling
    const float *spec = mg_kind == 4 ? c->rho : c->dk;
    RET_IF(mgp_fft_forces(c, spec, mg_kind == 3 ? 1.0f + coupling : 1.0f, T_FORCES, T_C2R));
    c->have_forces = 1;
    return MGP_OK;
  }
  tstart(c, T_FORCES);
  if (mg_kind == 4)  // rho holds delta + the fifth-force source
    RET_IF(mgp_launch_forces(c->rho, NULL, 0.f, 0.f, 0, N, c->p.Box, c->frc, c->g.nreal, c->stream));
  else
    RET_IF(mgp_launch_forces(c->dk, c->rho, coupling, mass2, mg_kind, N, c->p.Box, c->frc, c->g.nreal, c->stream));
  tstop(c, T_FORCES);
  if (c->closure) {  // learned residual force, added to the force transforms
    tstart(c, T_NN);
    RET_IF(mgp_closure_apply(c->closure, c, A));
    tstop(c, T_NN);
  }
  tstart(c, T_C2R);
  for (int g = 0; g < 3; g++) {
    if (own_fft(c))
      RET_IF(mgp_fft_c2r(c, c->frc + g * c->g.nreal));
    else
      MGP_CUFFT(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)(c->frc + g * c->g.nreal),
                             (cufftReal *)(c->frc + g * c->g.nreal)));
  }
  tstop(c, T_C2R);
  c->have_forces = 1;
  return MGP_OK;
}

static void kd_args(mgp_ctx *c, double AI, double AF, double A, double AFF, int do_drift, mgp_kd_args *a) {
  const mgp_cosmo *cs = &c->cosmo;
  const double om = c->p.Omega, cola = c->p.UseCOLA ? 1.0 : 0.0;
  double dda = mgp_cosmo_kick_dda(cs, AI, AF, A);  // StdDA 0 (COLA) or 2 (main.c:696-701)
  memset(a, 0, sizeof(*a));
  a->scale = (float)(c->g.N / c->p.Box);
  a->inv_scale = (float)(c->p.Box / c->g.N);
  a->kick_disp = (float)(-1.5 * om * dda);
  a->dda_omega = 1.5 * om * dda;
  a->do_drift = do_drift;
  if (c->sd) {
    // scale-dependent Kick/Drift (main.c:703-719, 758-770): D1 is the slot of
    // P.D + P.D2 (= the ddDddy fields), D2 the slot of P.dDdy + P.dD2dy
    // (= the deltaD fields), both already multiplied by their growth factors
    a->kick_d1 = (float)(-cola / A * dda);
    a->kick_d2 = 0.0f;
    a->lpt_stride = c->sd_grid;
    a->lpt_pitch = c->sd_pitch;
  } else {
    a->kick_d1 = (float)(-cola * mgp_cosmo_growth(cs, 2, A) / A * dda);
    a->kick_d2 = (float)(-cola * mgp_cosmo_growth(cs, 5, A) / A * dda);
    a->lpt_stride = c->np;
    a->lpt_pitch = c->Ns;
  }
  if (do_drift) {
    double dyyy = mgp_cosmo_drift_dyyy(cs, A, AFF, AF);
    a->dyyy = (float)dyyy;
    a->dyyy_d = dyyy;
    if (c->sd) {
      a->dD1 = 0.0f;
      a->dD2 = (float)cola;
    } else {
      a->dD1 = (float)(cola * (mgp_cosmo_growth(cs, 0, AFF) - mgp_cosmo_growth(cs, 0, A)));
      a->dD2 = (float)(cola * (mgp_cosmo_growth(cs, 3, AFF) - mgp_cosmo_growth(cs, 3, A)));
    }
  }
}

extern "C" int mgp_kick_drift(mgp_ctx *c, double AI, double AF, double A, double AFF, int do_drift) {
  RET_IF(require_particles(c));
  if (!c->have_forces) return mgp_set_error(MGP_ESTATE, "mgp_kick_drift before mgp_get_displacements");
  if (c->side_pending) {
    // velocities / LPT displacements still arriving on the side stream
    MGP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_side[1], 0));
    c->side_pending = 0;
  }
  if (c->sd) {
    if (c->sd_kind[0] != MGP_FIELD_ddDddy || c->sd_a[0] != A)
      return mgp_set_error(MGP_ESTATE, "scale-dependent kick at a = %g needs the ddDddy fields at that a "
                                       "(mgp_assign_displacement_fields)", A);
    if (do_drift && (c->sd_kind[1] != MGP_FIELD_deltaD || c->sd_a[1] != A || c->sd_aff[1] != AFF))
      return mgp_set_error(MGP_ESTATE, "scale-dependent drift %g -> %g needs the deltaD fields of that step", A, AFF);
  }
  mgp_kd_args a;
  kd_args(c, AI, AF, A, AFF, do_drift, &a);
  int nblk = mgp_ikd_blocks(c->np);
  const float *D1 = c->sd ? c->sd_slot[0] : c->D1, *D2 = c->sd ? c->sd_slot[1] : c->D2;
  tstart(c, T_IKD);
  if (c->tile_kick && c->tile_ready && !c->sd) {
    // per cell tile of this step's deposit sort, forces staged in shared
    // memory; the particle arrays are rewritten in the tile order
    RET_IF(mgp_ikd_tiles(c, &a, &nblk));
    RET_IF(mgp_launch_finalize_kd(c->dstate, c->partials, nblk, c->np, a.dda_omega, a.dyyy_d, a.do_drift,
                                  c->stream));
  } else {
    // particles in array order; with the arrays in tile order, q gives the
    // lattice points
    RET_IF(mgp_launch_ikd(c->frc, c->g.nreal, c->g.N, c->g.P, c->Ns, c->np, c->s, c->v, D1, D2, c->dstate,
                          c->partials, nblk, &a, c->stream, 1, NULL, c->permuted ? c->q : NULL));
  }
  tstop(c, T_IKD);
  if (do_drift) c->have_density = 0;
  return MGP_OK;
}

extern "C" int mgp_step(mgp_ctx *c, double A, double AI, double AF, double AFF) {
  RET_IF(require_particles(c));
  tstart(c, T_MISC);
  RET_IF(mgp_get_displacements(c, A));
  if (c->sd) {
    // main.c:487-503: [deltaD] and [ddDddy] for this step
    const int types[2] = {MGP_FIELD_ddDddy, MGP_FIELD_deltaD};
    tstart(c, T_SD);
    RET_IF(mgp_sd_fields(c, A, AFF, 2, types));
    tstop(c, T_SD);
  }
  RET_IF(mgp_kick_drift(c, AI, AF, A, AFF, 1));
  tstop(c, T_MISC);
  if (c->timing && c->hev) {
    c->hstep++;
    memset(c->htimed + (size_t)(c->hstep % c->hcap) * MGP_NTIMERS, 0, MGP_NTIMERS);
  }
  return MGP_OK;
}

static int pofk_out(mgp_ctx *c, int total, int cap, int *nbins, double *k, double *pk, double *kmean, double *n) {
  RET_IF(require_particles(c));
  if (!c->have_density) return mgp_set_error(MGP_ESTATE, "no density: call mgp_get_displacements first");
  // without P(k) every step the sums are taken now from delta(k), which is
  // the total matter field once massive neutrinos were added
  if (!c->p.pofk_compute_every_step) RET_IF(pofk_now(c, 0, c->last_density_a));
  const double *sums = total && c->cosmo.nu && c->p.pofk_compute_every_step ? c->pk_sum_tot : c->pk_sum;
  const int nb = c->pk_nbins;
  if (nbins) *nbins = nb;
  if (cap < nb) return mgp_set_error(MGP_EINVAL, "P(k) capacity %d < %d bins", cap, nb);
  MGP_CUDA(cudaMemcpyAsync(c->pk_host, sums, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  const double N = c->g.N, box = c->p.Box;
  const double norm = pow(box, 3) / pow(N, 6), shot = pow(box / (double)c->Ns, 3);
  for (int b = 0; b < nb; b++) {
    double P = 0.0, K = 0.0;
    if (c->pk_n[b] > 0) {
      P = c->pk_host[b] / c->pk_n[b] * norm;
      if (c->pk_sub) P -= shot;
      K = c->pk_k[b] / c->pk_n[b] * 2.0 * M_PI / box;
    }
    if (k) k[b] = k_from_index(b, c->pk_kmin, c->pk_kmax, nb, c->pk_bintype, box);
    if (pk) pk[b] = P;
    if (kmean) kmean[b] = K;
    if (n) n[b] = c->pk_n[b];
  }
  return MGP_OK;
}

// P(k) of the last density (compute_power_spectrum "CDM"), and the total
// matter P(k) of a run with massive neutrinos ("total"; the CDM one without)
extern "C" int mgp_pofk(mgp_ctx *c, int cap, int *nbins, double *k, double *pk, double *kmean, double *n) {
  return pofk_out(c, 0, cap, nbins, k, pk, kmean, n);
}
extern "C" int mgp_pofk_total(mgp_ctx *c, int cap, int *nbins, double *k, double *pk, double *kmean, double *n) {
  return pofk_out(c, 1, cap, nbins, k, pk, kmean, n);
}

// compute_RSD_powerspectrum (src/compute_pofk.c:403-512): redshift-space
// deposits with the y and z axes as line of sight, P0/P2/P4 per axis, their
// mean and |difference|/sqrt(2).  Uses the force grids as scratch.
extern "C" int mgp_pofk_rsd(mgp_ctx *c, double A, int cap, int *nbins, double *k, double *P0, double *P2, double *P4,
                            double *s0, double *s2, double *s4, double *n) {
  RET_IF(require_particles(c));
  RET_IF(mgp_particles_canonical(c));  // lattice order for the caller's arrays
  const int nb = c->pk_nbins, N = c->g.N;
  if (nbins) *nbins = nb;
  if (cap < nb) return mgp_set_error(MGP_EINVAL, "RSD capacity %d < %d bins", cap, nb);
  if (!c->rsd_block) {
    MGP_CUDA(cudaMalloc(&c->rsd_block, sizeof(double) * 3 * (size_t)nb * c->pk_blocks));
    MGP_CUDA(cudaMalloc(&c->rsd_sum, sizeof(double) * 3 * (size_t)nb));
  }
  const mgp_params *p = &c->p;
  // velfac = Hubble/A with Hubble = HUBBLE * UnitTime (src/2LPT.c:35-42)
  const double hub = 3.2407789e-18 * (p->UnitLength_in_cm / p->UnitVelocity_in_cm_per_s);
  const double vnorm = (hub / A) / (100.0 * A * mgp_hubble(&c->cosmo, A)) * (double)N / p->Box;
  const double cola = p->UseCOLA ? 1.0 : 0.0;
  float g1 = (float)(cola * mgp_cosmo_growth(&c->cosmo, 1, A)), g2 = (float)(cola * mgp_cosmo_growth(&c->cosmo, 4, A));
  const float *L1 = c->D1, *L2 = c->D2;
  long long lstride = c->np;
  int lpitch = c->Ns;
  if (c->sd) {
    // V = Vel + dDdy + dD2dy with the scale-dependent fields at A
    // (compute_pofk.c:323-325, 409-429)
    if (c->sd_kind[2] != MGP_FIELD_dDdy || c->sd_a[2] != A) {
      const int t = MGP_FIELD_dDdy;
      RET_IF(mgp_sd_fields(c, A, A, 1, &t));
    }
    L1 = L2 = c->sd_slot[2];
    g1 = (float)cola;
    g2 = 0.0f;
    lstride = c->sd_grid;
    lpitch = c->sd_pitch;
  }
  const double wpar = pow((double)N / (double)c->Ns, 3);
  float *dens = c->frc, *dkr = c->frc + c->g.nreal;
  std::vector<double> sums(3 * (size_t)nb), res[2][3];
  const double norm = pow(p->Box, 3) / pow((double)N, 6), shot = c->pk_sub ? pow(p->Box / (double)c->Ns, 3) : 0.0;
  for (int ax = 0; ax < 2; ax++) {
    RET_IF(mgp_launch_fill(dens, c->g.nreal, -1.0f, c->stream));
    RET_IF(mgp_launch_cic_rsd(c->s, c->v, L1, L2, lstride, lpitch, c->dstate, c->np, c->Ns, N, p->Box, (float)wpar,
                              ax + 1, (float)vnorm, g1, g2, dens, c->g.P, c->stream));
    MGP_CUFFT(cufftExecR2C(c->plan_r2c_oop, (cufftReal *)dens, (cufftComplex *)dkr));
    RET_IF(mgp_launch_pofk_mu(dkr, N, c->rk_bin, c->win1d, nb, c->rsd_block, c->pk_blocks, c->rsd_sum, c->stream));
    MGP_CUDA(cudaMemcpyAsync(sums.data(), c->rsd_sum, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, c->stream));
    MGP_CUDA(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 3; q++) res[ax][q].assign(nb, 0.0);
    for (int b = 0; b < nb; b++) {
      double nn = c->pk_n[b];
      if (!(nn > 0)) continue;
      double p0 = sums[b] / nn * norm, p2 = sums[nb + b] / nn * norm, p4 = sums[2 * nb + b] / nn * norm;
      p4 = 9.0 * (35.0 * p4 - 30.0 * p2 + 3.0 * p0) / 8.0;  // order as compute_pofk.c:704-706
      p2 = 5.0 * (3.0 * p2 - 1.0 * p0) / 2.0;
      res[ax][0][b] = p0 - shot;
      res[ax][1][b] = p2 - shot;
      res[ax][2][b] = p4 - shot;
    }
  }
  c->have_forces = 0;
  for (int b = 0; b < nb; b++) {
    double nn = c->pk_n[b];
    if (k) k[b] = nn > 0 ? k_from_index(b, c->pk_kmin, c->pk_kmax, nb, c->pk_bintype, p->Box) : 0.0;
    if (P0) P0[b] = (res[0][0][b] + res[1][0][b]) / 2.0;
    if (P2) P2[b] = (res[0][1][b] + res[1][1][b]) / 2.0;
    if (P4) P4[b] = (res[0][2][b] + res[1][2][b]) / 2.0;
    if (s0) s0[b] = fabs(res[0][0][b] - res[1][0][b]) / sqrt(2.0);
    if (s2) s2[b] = fabs(res[0][1][b] - res[1][1][b]) / sqrt(2.0);
    if (s4) s4[b] = fabs(res[0][2][b] - res[1][2][b]) / sqrt(2.0);
    if (n) n[b] = nn;
  }
  return MGP_OK;
}

// ---------------------------------------------------------- particles
static int ensure_stage(mgp_ctx *c, int arrays = 2) {
  // `arrays` [np][3] float staging arrays
  if (c->stage_arrays < arrays) {
    if (c->stage) {
      MGP_CUDA(cudaStreamSynchronize(c->stream));
      cudaFree(c->stage);
      c->stage = NULL;
      c->stage_arrays = 0;
    }
    MGP_CUDA(cudaMalloc(&c->stage, sizeof(float) * 3 * arrays * (size_t)c->np));
    c->stage_arrays = arrays;
  }
  return MGP_OK;
}

extern "C" int mgp_get_particles(mgp_ctx *c, float *pos, float *vel, float *D1, float *D2, size_t np) {
  RET_IF(require_particles(c));
  RET_IF(mgp_particles_canonical(c));  // lattice order for the caller's arrays
  if ((long long)np != c->np) return mgp_set_error(MGP_EINVAL, "np = %zu, context holds %lld", np, c->np);
  RET_IF(ensure_stage(c));
  const size_t bytes = sizeof(float) * 3 * np;
  float *dpos = c->stage, *dvel = c->stage + 3 * np;
  if (pos || vel) {
    RET_IF(mgp_launch_positions(c->s, c->dstate, c->np, c->Ns, c->p.Box, pos ? dpos : NULL, vel ? dvel : NULL, c->v,
                                c->stream));
    if (pos) MGP_CUDA(cudaMemcpyAsync(pos, dpos, bytes, cudaMemcpyDeviceToHost, c->stream));
    if (vel) MGP_CUDA(cudaMemcpyAsync(vel, dvel, bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  // D1/D2 SoA -> AoS on the host; with scale-dependent growth the two slots
  // the kick and the drift read (lattice rows of pitch Ps)
  const float *srcs[2] = {c->sd ? c->sd_slot[0] : c->D1, c->sd ? c->sd_slot[1] : c->D2};
  float *dsts[2] = {D1, D2};
  std::vector<float> h;
  for (int q = 0; q < 2; q++) {
    if (!dsts[q]) continue;
    h.resize(3 * np);
    if (c->sd) {
      for (int a = 0; a < 3; a++)
        MGP_CUDA(cudaMemcpy2D(h.data() + a * np, sizeof(float) * c->Ns, srcs[q] + a * c->sd_grid,
                              sizeof(float) * c->sd_pitch, sizeof(float) * c->Ns, (size_t)c->Ns * c->Ns,
                              cudaMemcpyDeviceToHost));
    } else {
      MGP_CUDA(cudaMemcpy(h.data(), srcs[q], bytes, cudaMemcpyDeviceToHost));
    }
    for (size_t i = 0; i < np; i++)
      for (int a = 0; a < 3; a++) dsts[q][3 * i + a] = h[a * np + i];
  }
  return MGP_OK;
}

// New absolute positions (velocities) restart the position (velocity) offset
// from zero; the other offset stays, or the particles would move.
static int reset_offsets(mgp_ctx *c, int pos_set, int vel_set, cudaStream_t st) {
  if (pos_set) MGP_CUDA(cudaMemsetAsync((char *)c->dstate + offsetof(mgp_dstate, cx), 0, sizeof(double) * 3, st));
  if (vel_set) MGP_CUDA(cudaMemsetAsync((char *)c->dstate + offsetof(mgp_dstate, cv), 0, sizeof(double) * 3, st));
  return MGP_OK;
}

extern "C" int mgp_set_particles(mgp_ctx *c, const float *pos, const float *vel, const float *D1, const float *D2,
                                 size_t np) {
  RET_IF(require_particles(c));
  RET_IF(mgp_particles_canonical(c));  // lattice order for the caller's arrays
  if ((long long)np != c->np) return mgp_set_error(MGP_EINVAL, "np = %zu, context holds %lld", np, c->np);
  RET_IF(ensure_stage(c));
  const size_t bytes = sizeof(float) * 3 * np;
  float *a = c->stage, *b = c->stage + 3 * np;
  if (pos) MGP_CUDA(cudaMemcpyAsync(a, pos, bytes, cudaMemcpyHostToDevice, c->stream));
  if (vel) MGP_CUDA(cudaMemcpyAsync(b, vel, bytes, cudaMemcpyHostToDevice, c->stream));
  if (pos || vel) {
    RET_IF(mgp_launch_set_state(c->s, c->v, pos ? a : NULL, vel ? b : NULL, c->np, c->Ns, c->p.Box, c->stream));
    RET_IF(reset_offsets(c, pos != NULL, vel != NULL, c->stream));
  }
  // with scale-dependent growth the LPT fields are recomputed from the stored
  // delta(k) before every use, so D1/D2 are not read
  const float *srcs[2] = {c->sd ? NULL : D1, c->sd ? NULL : D2};
  float *dsts[2] = {c->D1, c->D2};
  for (int q = 0; q < 2; q++) {
    if (!srcs[q]) continue;
    float *st = q == 0 ? a : b;
    MGP_CUDA(cudaMemcpyAsync(st, srcs[q], bytes, cudaMemcpyHostToDevice, c->stream));
    RET_IF(mgp_launch_aos_to_soa(st, dsts[q], c->np, c->stream));
    c->lpt_ver++;  // new D1/D2
  }
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  c->have_density = c->have_forces = 0;
  return MGP_OK;
}

extern "C" int mgp_host_register(void *ptr, size_t bytes) {
  MGP_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return MGP_OK;
}

extern "C" int mgp_host_alloc(void **ptr, size_t bytes) {
  if (!ptr) return mgp_set_error(MGP_EINVAL, "null argument");
  *ptr = NULL;
  MGP_CUDA(cudaMallocHost(ptr, bytes));
  return MGP_OK;
}

extern "C" int mgp_host_free(void *ptr) {
  if (ptr) MGP_CUDA(cudaFreeHost(ptr));
  return MGP_OK;
}

extern "C" int mgp_host_unregister(void *ptr) {
  MGP_CUDA(cudaHostUnregister(ptr));
  return MGP_OK;
}

// The positions go first, in chunks that are deposited as they arrive; the
// velocities and the LPT displacements, which only the kick reads, are
// copied and converted on a second stream while the deposit, the FFTs and
// the force pass run, and the kick waits for them.  With scale-dependent
// growth the step assigns its own LPT fields and D1/D2 are not read.
extern "C" int mgp_step_host(mgp_ctx *c, double A, double AI, double AF, double AFF, float *pos, float *vel,
                             const float *D1, const float *D2, size_t np) {
  RET_IF(require_particles(c));
  RET_IF(mgp_particles_canonical(c));  // lattice order for the caller's arrays
  if ((long long)np != c->np) return mgp_set_error(MGP_EINVAL, "np = %zu, context holds %lld", np, c->np);
  {
    if (!c->side) {
      MGP_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
      MGP_CUDA(cudaEventCreateWithFlags(&c->ev_side[0], cudaEventDisableTiming));
      MGP_CUDA(cudaEventCreateWithFlags(&c->ev_side[1], cudaEventDisableTiming));
    }
    RET_IF(ensure_stage(c, 4));
    const size_t bytes = sizeof(float) * 3 * np;
    float *st[4] = {c->stage, c->stage + 3 * np, c->stage + 6 * np, c->stage + 9 * np};
    RET_IF(reset_offsets(c, pos != NULL, vel != NULL, c->stream));
    // the side stream starts after everything queued so far (earlier readers
    // of the staging slots, s, v, D1 and D2 included)
    MGP_CUDA(cudaEventRecord(c->ev_side[0], c->stream));
    MGP_CUDA(cudaStreamWaitEvent(c->side, c->ev_side[0], 0));
    if (pos) {
      // positions first, in chunks: each is converted and deposited while
      // the next one is still on the link (PtoMesh, src/auxPM.c:280-343)
      if (!c->ev_chunk[0])
        for (int k = 0; k < MGP_POS_CHUNKS; k++) MGP_CUDA(cudaEventCreateWithFlags(&c->ev_chunk[k], cudaEventDisableTiming));
      const int N = c->g.N;
      const double wpar = pow((double)N / (double)c->Ns, 3);
      tstart(c, T_FILL);
      RET_IF(mgp_launch_fill(c->rho, c->g.nreal, -1.0f, c->stream));
      tstop(c, T_FILL);
      tstart(c, T_CIC);
      for (int k = 0; k < MGP_POS_CHUNKS; k++) {
        const long long p0 = c->np * k / MGP_POS_CHUNKS, p1 = c->np * (k + 1) / MGP_POS_CHUNKS;
        if (p1 <= p0) continue;
        MGP_CUDA(cudaMemcpyAsync(st[0] + 3 * p0, pos + 3 * p0, sizeof(float) * 3 * (p1 - p0), cudaMemcpyHostToDevice,
                                 c->side));
        MGP_CUDA(cudaEventRecord(c->ev_chunk[k], c->side));
        MGP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_chunk[k], 0));
        RET_IF(mgp_launch_set_state_range(c->s, c->v, st[0], NULL, c->np, c->Ns, c->p.Box, p0, p1, c->stream));
        RET_IF(mgp_launch_cic_range(c->s, c->dstate, c->np, p0, p1, c->Ns, N, c->p.Box, (float)wpar, c->rho, c->g.P,
                                    c->stream));
      }
      tstop(c, T_CIC);
    }
    // with scale-dependent growth the step assigns the LPT fields itself
    const float *src[3] = {vel, c->sd ? NULL : D1, c->sd ? NULL : D2};
    float *dst[3] = {c->v, c->D1, c->D2};
    for (int q = 0; q < 3; q++) {
      if (!src[q]) continue;
      MGP_CUDA(cudaMemcpyAsync(st[1 + q], src[q], bytes, cudaMemcpyHostToDevice, c->side));
      RET_IF(mgp_launch_aos_to_soa(st[1 + q], dst[q], c->np, c->side));
      if (q > 0) c->lpt_ver++;  // new D1/D2
    }
    MGP_CUDA(cudaEventRecord(c->ev_side[1], c->side));
    c->side_pending = 1;
    c->have_density = c->have_forces = 0;
    if (pos) {
      // the density is on the mesh: the rest of the step as mgp_step
      tstart(c, T_MISC);
      RET_IF(fields_from_density(c, A));
      if (c->sd) {
        const int types[2] = {MGP_FIELD_ddDddy, MGP_FIELD_deltaD};
        tstart(c, T_SD);
        RET_IF(mgp_sd_fields(c, A, AFF, 2, types));
        tstop(c, T_SD);
      }
      RET_IF(mgp_kick_drift(c, AI, AF, A, AFF, 1));
      tstop(c, T_MISC);
      RET_IF(mgp_get_particles(c, pos, vel, NULL, NULL, np));
      return MGP_OK;
    }
  }
  RET_IF(mgp_step(c, A, AI, AF, AFF));
  RET_IF(mgp_get_particles(c, pos, vel, NULL, NULL, np));
  return MGP_OK;
}

extern "C" int mgp_copy_grid(mgp_ctx *c, int which, float *host, size_t count) {
  RET_IF(require_particles(c));
  const float *src = NULL;
  switch (which) {
    case 0: src = c->rho; break;
    case 1: src = c->dk; break;
    case 2: case 3: case 4: src = c->frc + (which - 2) * c->g.nreal; break;
    case 5: src = c->rho; break;
    case 6: src = c->mg1; break;
    case 7: src = c->sd_dk[0]; break;
    default: return mgp_set_error(MGP_EINVAL, "unknown grid %d", which);
  }
  if (!src) return mgp_set_error(MGP_ESTATE, "grid %d is not allocated", which);
  if ((long long)count > c->g.nreal) return mgp_set_error(MGP_EINVAL, "count %zu exceeds grid size", count);
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  MGP_CUDA(cudaMemcpy(host, src, sizeof(float) * count, cudaMemcpyDeviceToHost));
  return MGP_OK;
}

extern "C" double mgp_growth(mgp_ctx *c, int which, double a) { return c ? mgp_cosmo_growth(&c->cosmo, which, a) : NAN; }
extern "C" double mgp_Sq(mgp_ctx *c, double ai, double af, double aref) { return c ? mgp_cosmo_Sq(&c->cosmo, ai, af, aref) : NAN; }
extern "C" double mgp_Sphi(mgp_ctx *c, double ai, double af, double aref) { return c ? mgp_cosmo_Sphi(&c->cosmo, ai, af, aref) : NAN; }
extern "C" double mgp_power_spectrum(mgp_ctx *c, double k) { return c ? mgp_cosmo_power(&c->cosmo, k) : NAN; }

// ----------------------------------------------------------------- batches
// A batch runs nbox independent boxes in lock step: every kernel of the PM
// step covers all boxes (the box is blockIdx.y), every FFT is one batched
// cuFFT call, and the whole KDK loop (src/main.c:394-611 for one output) is
// captured once into a CUDA graph and replayed with one launch.  The
// reference runs one box per MPI job; a sweep is many jobs.

struct batch_step {
  double A, AI, AF, AFF;
  int drift;
  mgp_kd_args kd;
};

// Time steps of main.c:394-611 for one output at z_final (stepDistr = 0):
// nsteps kick+drift steps, then the output step's kick (AF = A, no drift).
static void batch_schedule(const mgp_ctx *c, int nsteps, double zf, std::vector<batch_step> &st,
                           std::vector<mgp_box_scalars> &bs) {
  const mgp_params *p = &c->p;
  const double A0 = 1.0 / (1.0 + p->Init_Redshift), ao = 1.0 / (1.0 + zf);
  const double da = mgp_cosmo_step_da(p, A0, ao, nsteps), cola = p->UseCOLA ? 1.0 : 0.0, om = p->Omega;
  st.assign(nsteps + 1, batch_step());
  bs.assign((size_t)(nsteps + 1) * c->nbox, mgp_box_scalars());
  double A = A0, AI = A0;
  for (int t = 0; t <= nsteps; t++) {
    batch_step &q = st[t];
    q.drift = t < nsteps;
    q.A = A;
    q.AI = AI;
    q.AF = q.drift ? mgp_cosmo_step_mid(p, A, da) : A;
    q.AFF = mgp_cosmo_step_end(p, A, da);
    const mgp_cosmo *c0 = &c->cosmo;
    double dda = mgp_cosmo_kick_dda(c0, q.AI, q.AF, A);
    memset(&q.kd, 0, sizeof(q.kd));
    q.kd.scale = (float)(c->g.N / p->Box);
    q.kd.inv_scale = (float)(p->Box / c->g.N);
    q.kd.kick_disp = (float)(-1.5 * om * dda);
    q.kd.dda_omega = 1.5 * om * dda;
    q.kd.do_drift = q.drift;
    q.kd.lpt_stride = c->np;
    q.kd.lpt_pitch = c->Ns;
    if (q.drift) {
      double dyyy = mgp_cosmo_drift_dyyy(c0, A, q.AFF, q.AF);
      q.kd.dyyy = (float)dyyy;
      q.kd.dyyy_d = dyyy;
    }
    for (int b = 0; b < c->nbox; b++) {
      const mgp_cosmo *cb = cosmo_of(c, b);
      const mgp_params *pb = &c->box_p[b];
      mgp_box_scalars &o = bs[(size_t)t * c->nbox + b];
      o.kick_d1 = (float)(-cola * mgp_cosmo_growth(cb, 2, A) / A * dda);
      o.kick_d2 = (float)(-cola * mgp_cosmo_growth(cb, 5, A) / A * dda);
      if (q.drift) {
        o.dD1 = (float)(cola * (mgp_cosmo_growth(cb, 0, q.AFF) - mgp_cosmo_growth(cb, 0, A)));
        o.dD2 = (float)(cola * (mgp_cosmo_growth(cb, 3, q.AFF) - mgp_cosmo_growth(cb, 3, A)));
      }
      if (!pb->modified_gravity_active) continue;
      if (pb->model == MGP_MODEL_FOFR || pb->model == MGP_MODEL_MBETA) {
        o.phicrit = (float)mgp_phicrit(cb, A);
        o.coupling = (float)mgp_coupling(cb, A);
        o.mass2 = (float)(A * A * mgp_mass2_of_a(cb, A) / pow(2.0 * M_PI * 2997.92458 / pb->Box, 2));
      } else if (pb->model == MGP_MODEL_DGP) {
        o.coupling = (float)mgp_coupling(cb, A);
        o.pref = (float)mgp_dgp_screen_prefactor(cb, A);
      } else if (pb->model == MGP_MODEL_BRANSDICKE) {
        o.coupling = (float)(mgp_geff(cb, A, 0.0) - 1.0);
      }
    }
    A = q.AFF;
    AI = q.AF;
  }
}

// One batched PM step (GetDisplacements + P(k) + Kick/Drift) for all boxes,
// stream-ordered and free of host synchronisation (it is graph-captured).
static int batch_step_launch(mgp_ctx *c, const batch_step &q, const mgp_box_scalars *bs, double *pk_sums) {
  const mgp_params *p = &c->p;
  const int N = c->g.N, B = c->nbox;
  const long long gf = c->g.nreal;
  // batched plans when there are several boxes (a single box uses its own)
  const cufftHandle r2c_oop = B > 1 ? c->plan_r2c_oop_b : c->plan_r2c_oop;
  const cufftHandle r2c_ip = B > 1 ? c->plan_r2c_ip_b : c->plan_r2c_ip;
  const cufftHandle c2r = B > 1 ? c->plan_c2r_b : c->plan_c2r_1;
  const cufftHandle c2r_frc = B > 1 ? c->plan_c2r_frc_b : c->plan_c2r_1;
  const double wpar = pow((double)N / (double)c->Ns, 3);
  if (c->batch_tile) RET_IF(mgp_tiles_sort(c, c->batch_tile));  // all boxes' particles by tile
  RET_IF(mgp_launch_fill(c->rho, gf * B, -1.0f, c->stream));
  if (c->batch_tile)
    RET_IF(mgp_cic_tiles(c, (float)wpar, c->tune[0]));
  else
    RET_IF(mgp_launch_cic(c->s, c->dstate, c->np, c->Ns, N, p->Box, (float)wpar, c->rho, c->g.P, c->stream, B, gf));
  MGP_CUFFT(cufftExecR2C(r2c_oop, (cufftReal *)c->rho, (cufftComplex *)c->dk));
  const int fused = p->pofk_compute_every_step ? mg_filter_kind(p) : 0;
  const double n3 = pow((double)N, 3);
  if (p->pofk_compute_every_step) {
    float fa = 0.f, fb = 0.f;
    if (fused == 1) {
      fa = (float)(2.0 * M_PI / p->Box * p->Rsmooth);
      fb = (float)(1.0 / n3);
    } else if (fused == 2) {
      fb = (float)(1.0 / n3 * 1.5 * p->Omega / q.A * pow(p->Box / 2997.92458 / (2.0 * M_PI), 2));
    }
    RET_IF(mgp_launch_pofk_thr(c->dk, N, c->pk_thr, c->win1d, c->pk_nbins, c->pk_bintype, c->pk_kmin, c->pk_kmax,
                               c->pk_block, c->pk_blocks, pk_sums, fused, p->smoothing_filter, fused ? c->mg1 : NULL,
                               fa, fb, c->stream, B, gf, c->pk_nbins));
  }
  int mg_kind = 0;
  if (p->modified_gravity_active) {
    if (p->model == MGP_MODEL_FOFR || p->model == MGP_MODEL_MBETA) {
      if (p->include_screening) {
        double norm = 1.0 / n3 * 1.5 * p->Omega / q.A * pow(p->Box / 2997.92458 / (2.0 * M_PI), 2);
        if (!fused) RET_IF(mgp_launch_div_laplacian(c->dk, c->mg1, N, (float)norm, c->stream, B, gf));
        MGP_CUFFT(cufftExecC2R(c2r, (cufftComplex *)c->mg1, (cufftReal *)c->mg1));
        RET_IF(mgp_launch_screen_potential(c->rho, c->mg1, gf, 0.f, c->stream, B, bs));
      }
      MGP_CUFFT(cufftExecR2C(r2c_ip, (cufftReal *)c->rho, (cufftComplex *)c->rho));
      mg_kind = 1;
    } else if (p->model == MGP_MODEL_DGP) {
      if (p->include_screening) {
        if (!fused)
          RET_IF(mgp_launch_smooth(c->dk, c->mg1, N, p->smoothing_filter, (float)(2.0 * M_PI / p->Box * p->Rsmooth),
                                   (float)(1.0 / n3), c->stream, B, gf));
        MGP_CUFFT(cufftExecC2R(c2r, (cufftComplex *)c->mg1, (cufftReal *)c->mg1));
        RET_IF(mgp_launch_screen_density(c->rho, c->mg1, gf, 0.f, 0.f, c->stream, B, bs));
        MGP_CUFFT(cufftExecR2C(r2c_ip, (cufftReal *)c->rho, (cufftComplex *)c->rho));
        mg_kind = 2;
      } else {
        mg_kind = 3;
      }
    } else if (p->model == MGP_MODEL_BRANSDICKE) {
      mg_kind = 3;
    }
  }
  RET_IF(mgp_launch_forces(c->dk, c->rho, 0.f, 0.f, mg_kind, N, p->Box, c->frc, gf, c->stream, B, bs));
  for (int g = 0; g < 3; g++)
    MGP_CUFFT(cufftExecC2R(c2r_frc, (cufftComplex *)(c->frc + g * gf), (cufftReal *)(c->frc + g * gf)));
  int nblk = mgp_blocks_per_box(c->np, c->tune[2], B);
  if (nblk > c->max_blocks) nblk = c->max_blocks;  // the per-block partials buffer
  RET_IF(mgp_launch_ikd(c->frc, gf, N, c->g.P, c->Ns, c->np, c->s, c->v, c->D1, c->D2, c->dstate, c->partials, nblk,
                        &q.kd, c->stream, B, bs));
  return MGP_OK;
}

static int batch_build_graph(mgp_ctx *c, int nsteps, double zf) {
  std::vector<batch_step> st;
  std::vector<mgp_box_scalars> bs;
  batch_schedule(c, nsteps, zf, st, bs);
  if (nsteps + 1 > c->hist_steps) {
    if (c->box_bs) cudaFree(c->box_bs);
    if (c->pk_hist) cudaFree(c->pk_hist);
    c->box_bs = NULL;
    c->pk_hist = NULL;
    c->hist_steps = 0;
    MGP_CUDA(cudaMalloc(&c->box_bs, sizeof(mgp_box_scalars) * bs.size()));
    MGP_CUDA(cudaMalloc(&c->pk_hist, sizeof(double) * (size_t)(nsteps + 1) * c->nbox * c->pk_nbins));
    c->hist_steps = nsteps + 1;
  }
  MGP_CUDA(cudaMemcpy(c->box_bs, bs.data(), sizeof(mgp_box_scalars) * bs.size(), cudaMemcpyHostToDevice));
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = NULL;
  c->graph = NULL;
  // the batch's launch budgets hold for the captured launches only
  const int pk_keep = c->pk_blocks;
  c->pk_blocks = pk_blocks_for(c, c->tune[3]);
  if (c->pk_blocks > c->pk_blocks_cap) c->pk_blocks = c->pk_blocks_cap;
  mgp_set_launch_budget(c->tune[0], c->tune[1]);
  if (c->batch_tile) RET_IF(mgp_tiles_alloc(c, c->batch_tile));  // no allocation inside the capture
  MGP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const long long k0 = g_kernel_launches;
  int rc = MGP_OK;
  for (int t = 0; t <= nsteps && rc == MGP_OK; t++)
    rc = batch_step_launch(c, st[t], c->box_bs + (size_t)t * c->nbox,
                           c->pk_hist + (size_t)t * c->nbox * c->pk_nbins);
  cudaGraph_t g = NULL;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  mgp_set_launch_budget(MGP_BUDGET_DEFAULT, MGP_BUDGET_DEFAULT);
  c->pk_blocks = pk_keep;
  if (rc != MGP_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return mgp_set_error(MGP_ECUDA, "graph capture: %s", cudaGetErrorString(e));
  c->graph = g;
  c->graph_kernels = (int)(g_kernel_launches - k0);
  MGP_CUDA(cudaGraphInstantiate(&c->graph_exec, g, 0));
  c->graph_nsteps = nsteps;
  c->graph_zf = zf;
  return MGP_OK;
}

extern "C" int mgp_batch_run(mgp_ctx *c, int nsteps, double z_final) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (nsteps < 1) return mgp_set_error(MGP_EINVAL, "nsteps = %d", nsteps);
  MGP_CUDA(cudaSetDevice(c->device));
  if (c->nbox == 1 && !c->bev[0]) {
    MGP_CUDA(cudaEventCreate(&c->bev[0]));
    MGP_CUDA(cudaEventCreate(&c->bev[1]));
  }
  if (c->sd) return mgp_set_error(MGP_EINVAL, "batch runs use scale-independent growth");
  // 2LPT ICs of every box (not captured: host-side seed tables), written
  // in lattice order
  c->permuted = 0;
  c->tile_ready = 0;
  MGP_CUDA(cudaEventRecord(c->bev[0], c->stream));
  for (int b = 0; b < c->nbox; b++) RET_IF(ic_box(c, b));
  MGP_CUDA(cudaEventRecord(c->bev[1], c->stream));
  MGP_CUDA(cudaEventSynchronize(c->bev[1]));
  MGP_CUDA(cudaEventElapsedTime(&c->batch_ic_ms, c->bev[0], c->bev[1]));
  if (!c->graph_exec || c->graph_nsteps != nsteps || c->graph_zf != z_final) RET_IF(batch_build_graph(c, nsteps, z_final));
  MGP_CUDA(cudaEventRecord(c->bev[0], c->stream));
  MGP_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
  MGP_CUDA(cudaEventRecord(c->bev[1], c->stream));
  MGP_CUDA(cudaEventSynchronize(c->bev[1]));
  MGP_CUDA(cudaEventElapsedTime(&c->batch_ms, c->bev[0], c->bev[1]));
  c->have_density = c->have_forces = 0;
  return MGP_OK;
}

// Launch budgets of a batch (resident blocks per SM): [0] deposit, [1] grid
// passes (fill, forces, MG passes), [2] interp+kick+drift, [3] P(k) binning.
// They change launch shapes only (sums may differ in rounding); the next
// mgp_batch_run captures a new graph with them.
extern "C" int mgp_batch_set_tuning(mgp_ctx *c, const int *tune) {
  if (!c || !tune) return mgp_set_error(MGP_EINVAL, "null argument");
  for (int q = 0; q < 4; q++)
    if (tune[q] < 1 || tune[q] > 64) return mgp_set_error(MGP_EINVAL, "launch budget %d out of [1, 64]", tune[q]);
  for (int q = 0; q < 4; q++) c->tune[q] = tune[q];
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = NULL;
  c->graph = NULL;
  return MGP_OK;
}

extern "C" int mgp_batch_get_tuning(mgp_ctx *c, int *tune) {
  if (!c || !tune) return mgp_set_error(MGP_EINVAL, "null argument");
  for (int q = 0; q < 4; q++) tune[q] = c->tune[q];
  return MGP_OK;
}

// Deposit form of a batch: 0 (default) one thread per particle in lattice
// order, eight global float reductions each; 8 or 16: every step all boxes'
// particles are bucketed by the side^3-cell tile of their CIC base cell and
// each tile is summed in shared memory, then added to the mesh with one
// float2 reduction per pair of cells.  The density is the same up to the
// order of float sums; the next mgp_batch_run captures a new graph.
extern "C" int mgp_batch_set_deposit_tiles(mgp_ctx *c, int side) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (side) RET_IF(mgp_tiles_check(c, side));
  c->batch_tile = side;
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = NULL;
  c->graph = NULL;
  return MGP_OK;
}

extern "C" int mgp_batch_get_deposit_tiles(mgp_ctx *c) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  return c->batch_tile;
}

// Autotuner: coordinate descent over the deposit form and the four budgets
// (grid passes first, then the deposit form {lattice order, 8^3 tiles, 16^3
// tiles}, the deposit budget, kick and P(k)), each budget over {1, 2, 4, 8,
// 16, 32} blocks per SM (P(k): {1, 2, 4, 8, 16}); every candidate is timed by
// one mgp_batch_run of nsteps (fresh ICs, a newly captured graph, the graph
// timed with CUDA events) and the fastest is kept.  *best_ms receives the
// graph time of the result.
extern "C" int mgp_batch_autotune(mgp_ctx *c, int nsteps, double z_final, double *best_ms) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  static const int cand[6] = {1, 2, 4, 8, 16, 32};
  static const int order[5] = {1, -1, 0, 2, 3};  // -1: the deposit form
  static const int sides[3] = {0, 8, 16};
  int best[4];
  for (int q = 0; q < 4; q++) best[q] = c->tune[q];
  RET_IF(mgp_batch_set_tuning(c, best));
  RET_IF(mgp_batch_run(c, nsteps, z_final));
  double best_t = c->batch_ms;
  for (int oi = 0; oi < 5; oi++) {
    const int q = order[oi];
    if (q < 0) {
      int best_side = c->batch_tile;
      for (int side : sides) {
        if (side == best_side || (side && mgp_tiles_check(c, side) != MGP_OK)) continue;
        RET_IF(mgp_batch_set_deposit_tiles(c, side));
        RET_IF(mgp_batch_run(c, nsteps, z_final));
        if (c->batch_ms < best_t) {
          best_t = c->batch_ms;
          best_side = side;
        }
      }
      RET_IF(mgp_batch_set_deposit_tiles(c, best_side));
      continue;
    }
    for (int ci = 0; ci < (q == 3 ? 5 : 6); ci++) {
      if (cand[ci] == best[q]) continue;
      int trial[4] = {best[0], best[1], best[2], best[3]};
      trial[q] = cand[ci];
      RET_IF(mgp_batch_set_tuning(c, trial));
      RET_IF(mgp_batch_run(c, nsteps, z_final));
      if (c->batch_ms < best_t) {
        best_t = c->batch_ms;
        best[q] = cand[ci];
      }
    }
  }
  RET_IF(mgp_batch_set_tuning(c, best));
  if (best_ms) *best_ms = best_t;
  return MGP_OK;
}

extern "C" double mgp_batch_ms(mgp_ctx *c, int what) {
  if (!c) return -1.0;
  return what == 0 ? c->batch_ms : c->batch_ic_ms;
}

extern "C" int mgp_batch_graph_kernels(mgp_ctx *c) { return c && c->graph ? c->graph_kernels : -1; }

extern "C" int mgp_batch_graph_nodes(mgp_ctx *c) {
  if (!c || !c->graph) return -1;
  size_t n = 0;
  if (cudaGraphGetNodes(c->graph, NULL, &n) != cudaSuccess) return -1;
  return (int)n;
}

extern "C" int mgp_batch_pofk(mgp_ctx *c, int box, int step, int cap, int *nbins, double *k, double *pk,
                              double *kmean, double *n) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (!c->pk_hist || !c->p.pofk_compute_every_step) return mgp_set_error(MGP_ESTATE, "no batch P(k) recorded");
  if (box < 0 || box >= c->nbox || step < 0 || step > c->graph_nsteps)
    return mgp_set_error(MGP_EINVAL, "box %d / step %d out of range", box, step);
  const int nb = c->pk_nbins;
  if (nbins) *nbins = nb;
  if (cap < nb) return mgp_set_error(MGP_EINVAL, "P(k) capacity %d < %d bins", cap, nb);
  MGP_CUDA(cudaSetDevice(c->device));
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  MGP_CUDA(cudaMemcpy(c->pk_host, c->pk_hist + ((size_t)step * c->nbox + box) * nb, sizeof(double) * nb,
                      cudaMemcpyDeviceToHost));
  const double N = c->g.N, bx = c->p.Box;
  const double norm = pow(bx, 3) / pow(N, 6), shot = pow(bx / (double)c->Ns, 3);
  for (int b = 0; b < nb; b++) {
    double P = 0.0, K = 0.0;
    if (c->pk_n[b] > 0) {
      P = c->pk_host[b] / c->pk_n[b] * norm;
      if (c->pk_sub) P -= shot;
      K = c->pk_k[b] / c->pk_n[b] * 2.0 * M_PI / bx;
    }
    if (k) k[b] = k_from_index(b, c->pk_kmin, c->pk_kmax, nb, c->pk_bintype, bx);
    if (pk) pk[b] = P;
    if (kmean) kmean[b] = K;
    if (n) n[b] = c->pk_n[b];
  }
  return MGP_OK;
}

extern "C" int mgp_batch_get_particles(mgp_ctx *c, int box, float *pos, float *vel, size_t np) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (box < 0 || box >= c->nbox) return mgp_set_error(MGP_EINVAL, "box %d out of range", box);
  if ((long long)np != c->np) return mgp_set_error(MGP_EINVAL, "np = %zu, a box holds %lld", np, c->np);
  MGP_CUDA(cudaSetDevice(c->device));
  RET_IF(ensure_stage(c));
  const size_t bytes = sizeof(float) * 3 * np, po = (size_t)box * 3 * np;
  float *dpos = c->stage, *dvel = c->stage + 3 * np;
  RET_IF(mgp_launch_positions(c->s + po, c->dstate + box, c->np, c->Ns, c->p.Box, pos ? dpos : NULL,
                              vel ? dvel : NULL, c->v + po, c->stream));
  if (pos) MGP_CUDA(cudaMemcpyAsync(pos, dpos, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (vel) MGP_CUDA(cudaMemcpyAsync(vel, dvel, bytes, cudaMemcpyDeviceToHost, c->stream));
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  return MGP_OK;
}
