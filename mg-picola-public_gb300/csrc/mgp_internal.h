/*
 * Internal state of an mgp_ctx and the kernel launchers of the GB300 COLA
 * library.  Not part of the public ABI.
 *
 * HBM layout (N = Nmesh, Ns = Nsample, P = 2(N/2+1), NH = N/2+1):
 *   particles, SoA float, lattice order p = (i*Ns + j)*Ns + k:
 *     s[3][Np]   displacement from the Lagrangian point q = (i,j,k) Box/Ns
 *     v[3][Np]   COLA velocity minus the running offset `cv`
 *     D1[3][Np]  ZA displacement, D2[3][Np] 2LPT displacement (times -3/7)
 *   true position x = wrap(q + s + cx), true velocity = v + cv, where cx, cv
 *   are FP64 3-vectors in `dstate` updated on the device after every kick.
 *   grids, FP32 (FFTW/cuFFT padded layout):
 *     rho  [N][N][P]      density (real) / MG effective density (in place)
 *     dk   [N][N][NH]c    delta(k)
 *     frc  3 x [N][N][P]  force grids (complex in, real out, batched C2R)
 *     mg1  [N][N][P]      MG scratch: Phi_N(k)->Phi_N(x) or smoothed delta
 */
#ifndef MGP_INTERNAL_H
#define MGP_INTERNAL_H

#include <cuda_runtime.h>
#include <cufft.h>
#include <stddef.h>
#include <stdint.h>

#include "mgp_cosmo.h"
#include "mgpicola.h"

/* FP64 device-side running state (one per context). */
typedef struct {
  double cx[3];        /* position offset (Mpc/h) */
  double cv[3];        /* velocity offset */
  double mean_disp[3]; /* sumDxyz of the last MtoParticles */
  double mean_v[3];    /* mean of the stored v after the last kick */
} mgp_dstate;

#define MGP_NTIMERS 13

typedef struct mgp_grid_geom {
  int N, NH;
  long long P;          /* padded row length in floats */
  long long nreal;      /* N*N*P floats */
  long long ncomplex;   /* N*N*NH complex values */
} mgp_grid_geom;

/* Per-box scalars of a batch of independent boxes (mgp_batch): one entry per
 * box, read by the batched kernels in place of their by-value scalars. */
typedef struct {
  float kick_d1, kick_d2, dD1, dD2; /* growth-dependent Kick/Drift factors (mgp_kd_args) */
  float phicrit;                    /* potential screening phi_crit(a) */
  float mass2;                      /* a^2 m^2(a) in RK units (force pass, mg_kind 1) */
  float coupling;                   /* force-pass or density-screening coupling */
  float pref;                       /* density-screening prefactor */
} mgp_box_scalars;

struct mgp_ctx {
  mgp_params p;
  mgp_cosmo cosmo;
  int device;
  cudaStream_t stream;
  mgp_grid_geom g;
  long long np;
  int Ns;

  /* particles */
  float *s, *v, *D1, *D2;  /* each 3*np */
  mgp_dstate *dstate;      /* device */
  double *partials;        /* per-block reduction scratch (double) */
  float *stage;            /* host-interface staging, stage_arrays x 3 np floats (lazy) */
  int stage_arrays;
  cudaStream_t side;       /* host-buffer step: copies that only the kick waits for */
  cudaEvent_t ev_side[2];
  /* host-buffer step: the position upload in MGP_POS_CHUNKS pieces, each
   * converted and deposited as soon as it has arrived */
  cudaEvent_t ev_chunk[8];
  int side_pending;
  int max_blocks;

  /* grids */
  float *rho, *dk, *frc, *mg1;
  float *ic_scratch;        /* six grids for the 2LPT IC (lazy, kept for the next IC) */
  void *fft_work;
  size_t fft_work_bytes;
  cufftHandle plan_r2c_oop, plan_r2c_ip, plan_c2r_1;
  /* 1024^3 grids (mgp_fft.cu): the y pass by this library's kernel (the
   * force pass fused into the inverse one), z rows and x lines by cuFFT's
   * 1D plans.  fft_mode 1 (default where supported) uses them, 0 the 3D
   * cuFFT plans. */
  int fft_mode, fft_ready;
  cufftHandle zplan_r2c_oop, zplan_r2c_ip, zplan_c2r, xplan;
  float *fft_tw;            /* device: W_1024^m, m = 0..1023 (float2) */
  float *fft_gauss;         /* device: Gaussian smoothing factor per stored index (lazy) */
  float fft_gauss_kR1;      /* the kR1 it was made for */

  /* P(k) */
  int pk_nbins, pk_bintype, pk_sub;
  double pk_kmin, pk_kmax;  /* integer-k units, adjusted */
  int *rk_bin;              /* device: bin index per integer |k|^2 (or -1) */
  int *pk_thr;              /* device: first |k|^2 of each bin, [nbins] = end */
  float *win1d;             /* device: 1/sinc^4 per |d| in [0, N/2] */
  double *pk_block;         /* device: per-block FP64 bin partials */
  double *pk_sum;           /* device: FP64 bin sums */
  double *rsd_block, *rsd_sum; /* device: RSD moment partials and sums (lazy) */
  double *pk_n, *pk_k;      /* host: mode counts and k sums per bin */
  double *pk_host;          /* host: last P(k) sums */
  double *pk_sum_tot;       /* device: total-matter P(k) sums with massive neutrinos (lazy) */
  /* massive neutrinos: the transfer row of the step (two pinned host slots
   * of value + d/d ln k, alternating per step, each reusable once its upload
   * event has passed), its device copy and ln k nodes, the T_cb(k, 1)
   * denominators and the factor table per integer |k|^2 on the device */
  double *nu_row_h, *nu_row_d, *nu_x_d, *nu_den_d;
  float *nu_tab_d;
  int nu_nx;
  cudaEvent_t nu_ev[2];
  int nu_slot;
  double nu_cdmfac;
  int pk_blocks;
  int pk_blocks_cap;        /* blocks the P(k) partial buffer holds (per box) */
  int tune[4];              /* batch launch budgets, blocks per SM: deposit, grid passes, kick, P(k) */
  int have_density, have_forces;
  double last_density_a;

  /* scale-dependent growth (SCALEDEPENDENT build).  The particles carry no
   * D1/D2 arrays; the LPT fields live on the Lagrangian lattice as three
   * padded real [Ns][Ns][Ps] grids per slot (Ps = 2(Ns/2+1)), which is the
   * particle order with a row pitch of Ps:
   *   slot 0 "D"     FIELD_D at the IC, FIELD_ddDddy in the loop (P.D + P.D2)
   *   slot 1 "dDdy"  FIELD_deltaD (P.dDdy + P.dD2dy as Drift reads them)
   *   slot 2 "vel"   FIELD_dDdy for outputs, RSD and the non-COLA IC velocity
   * each the sum of the 1LPT and 2LPT fields (every reader adds them). */
  int sd;
  int sd_fold;              /* Nmesh / Nsample (alias count per axis); 0 when Nmesh is
                               not a multiple of Nsample (full-mesh path) */
  float *sd_full;           /* full-mesh path: one padded real N^3 grid */
  double *sd_part;          /* full-mesh path: read-out partial sums */
  float *sd_dk[2];          /* delta(k), -source(k): complex [N][N][NH] */
  float *sd_slot[3];        /* 3 components x sd_grid floats each */
  long long sd_grid;        /* Ns*Ns*Ps floats */
  int sd_pitch;             /* Ps */
  int sd_kind[3];           /* field type held by each slot, -1 none */
  double sd_a[3], sd_aff[3];
  cufftHandle plan_c2r_s;   /* Ns^3 in-place C2R */
  double *sd_cols;          /* device: growth-table columns for the current call */
  float *sd_tab;            /* device: float4 per integer |k|^2 */
  long long sd_nmax;        /* largest integer |k|^2 = 3 (N/2)^2 */

  /* batch of independent boxes (mgp_batch_create; nbox = 1 otherwise).
   * Every particle array and grid holds nbox boxes back to back; box b has
   * its own parameters (seed, IC flags, f(R) fR0 or nDGP rcH0) and growth
   * tables, all boxes share Nmesh, Nsample, Box and the background H(a). */
  int nbox;
  mgp_params *box_p;        /* host: per-box parameters (nbox) */
  mgp_cosmo *box_cosmo;     /* host: per-box cosmologies for boxes 1..nbox-1 */
  cufftHandle plan_r2c_oop_b, plan_r2c_ip_b, plan_c2r_b, plan_c2r_frc_b; /* batched over boxes */
  mgp_box_scalars *box_bs;  /* device: [nsteps+1][nbox] per-step scalars */
  double *pk_hist;          /* device: [nsteps+1][nbox][nbins] P(k) bin sums */
  int hist_steps;           /* capacity of box_bs / pk_hist in steps */
  cudaGraph_t graph;
  cudaGraphExec_t graph_exec;
  int graph_nsteps;
  int graph_kernels;        /* this library's kernels per graph launch */
  double graph_zf;
  cudaEvent_t bev[2];
  float batch_ms, batch_ic_ms;

  /* snapshot output overlapped with the following steps (mgp_run): the
   * output kernel writes a device staging buffer, a copy stream downloads it
   * into pinned host memory and a host thread writes the files */
  float *out_dev, *out_host;   /* two slots of 2 x 3 np floats each (lazy) */
  cudaStream_t out_stream;
  cudaEvent_t out_ev[2];
  void *out_writer;            /* host writer thread state (mgp_run.cu) */

  /* cell-tile order of the particles (mgp_tiles.cu): tile of every
   * particle, particle indices bucketed by tile, tile counts / offsets /
   * scatter cursors, scan block totals */
  unsigned *tile_of, *tile_order, *tile_count, *tile_off, *tile_cursor, *tile_bsum;
  int tile_side, tile_n1, tile_nz, tile_ready;  /* shape code, tiles along x and y, along z */
  long long tile_cap;       /* tiles the count/offset arrays hold */
  /* owner-writes deposit of a single box: halo pairs of every tile, and the
   * slots of particles deposited after the interiors (np entries + count) */
  void *tile_halo;
  size_t tile_halo_bytes;
  unsigned *tile_spill;
  int batch_tile;           /* batch deposit: tile side (8, 16) or 0 for the lattice-order deposit */
  int tile_mode;            /* 1 (default): tile deposit where it applies; 0: particle order */
  /* particle arrays held in cell-tile order (single box, scale-independent
   * growth): with tile_kick the kick of every step reads the particles in
   * the deposit's tile order and writes s, v in that order (into the *_alt
   * buffers, then swapped); q[p] is then the lattice point of
   * slot p.  Entry points that read or write particles in lattice order
   * first restore it (mgp_particles_canonical). */
  unsigned *q, *q_alt;
  float *s_alt, *v_alt;
  /* D1/D2 stay in lattice order; the tile kick reads them packed, 32 bytes
   * per particle in lattice order (lpt), repacked when lpt_ver (bumped by
   * every writer of D1/D2) differs from the version packed */
  float *lpt;
  long long lpt_ver, lpt_built;
  int permuted, tile_kick;

  /* user screening functions: the device copy of the step's table */
  float *scr_tab;

  /* learned force closure added to the force grids (mgp_set_closure) */
  struct mgp_closure *closure;

  /* timing: per-stage events of the last call, and caller marks on the
   * context stream (mgp_mark) that bracket whole runs */
  cudaEvent_t ev_mark[4];
  int timing;
  cudaEvent_t ev[MGP_NTIMERS][2];
  float ms[MGP_NTIMERS];
  int timed[MGP_NTIMERS];
  /* timing history (mgp_set_timing with n > 1): the stage events of the
   * last n mgp_step calls, [slot][timer][start/stop], slot = step % n */
  cudaEvent_t *hev;
  unsigned char *htimed;  /* [slot][timer] */
  int hcap, hstep;
  long long launches;
};

enum { T_CIC = 0, T_R2C, T_POFK, T_MG, T_FORCES, T_C2R, T_IKD, T_MISC, T_SD, T_NN, T_NNCONV, T_FILL, T_SORT };
/* stage timer events of a context (current step and, when kept, its history) */
void mgp_tstart(mgp_ctx *c, int t);
void mgp_tstop(mgp_ctx *c, int t);

/* error plumbing (C linkage: also called from the C sources) */
#ifdef __cplusplus
extern "C" {
#endif
int mgp_set_error(int code, const char *fmt, ...);
#ifdef __cplusplus
}
#endif

#define MGP_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return mgp_set_error(MGP_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
                           cudaGetErrorString(e_));                                         \
  } while (0)
#define MGP_CUFFT(call)                                                                     \
  do {                                                                                      \
    cufftResult r_ = (call);                                                                \
    if (r_ != CUFFT_SUCCESS)                                                                \
      return mgp_set_error(MGP_ECUFFT, "%s:%d %s: cufft error %d", __FILE__, __LINE__, #call, \
                           (int)r_);                                                        \
  } while (0)
#define MGP_CHECK_LAUNCH()                                                                  \
  do {                                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                    \
    if (e_ != cudaSuccess)                                                                  \
      return mgp_set_error(MGP_ECUDA, "%s:%d kernel launch: %s", __FILE__, __LINE__,        \
                           cudaGetErrorString(e_));                                         \
  } while (0)

/* ------------------------------------------------------------ launchers */
/* Launchers that take `nbox` run the same kernel over nbox boxes laid out
 * back to back (grids g_bs floats apart, particles 3 Np floats apart), the box
 * being blockIdx.y; `bs` (device, nbox entries) replaces the by-value
 * scalars when non-NULL. */
int mgp_blocks_per_box(long long n_per_box, int per_sm, int nbox);
#define MGP_POS_CHUNKS 8  /* pieces of the position upload of mgp_step_host */
#define MGP_BUDGET_DEFAULT 8
void mgp_set_launch_budget(int cic, int grid);
/* Per-launch scalars of the fused MtoParticles + Kick + Drift kernel. */
typedef struct {
  float scale;        /* N / Box */
  float inv_scale;    /* Box / N */
  float kick_disp;    /* -1.5 * Omega * dda */
  float kick_d1;      /* -UseCOLA * ddD(A) / A * dda */
  float kick_d2;      /* -UseCOLA * ddD2(A) / A * dda */
  float dyyy;         /* Sq(A, AFF, AF) */
  float dD1;          /* UseCOLA * (D(AFF) - D(A)) */
  float dD2;          /* UseCOLA * (D2(AFF) - D2(A)) */
  int do_drift;
  double dda_omega;   /* 1.5 * Omega * dda for the velocity offset */
  double dyyy_d;
  /* layout of D1/D2: component c of particle (i, j, k) is at
   * c * lpt_stride + (i*Ns + j) * lpt_pitch + k (Np and Ns for the particle
   * arrays, the slot grid size and Ps for the scale-dependent slots) */
  long long lpt_stride;
  int lpt_pitch;
} mgp_kd_args;

extern long long g_kernel_launches;
int mgp_blocks_for(long long n, int per_sm);

/* the y pass of 1024^3 transforms and the fused force pass (mgp_fft.cu) */
int mgp_fft_supported(const mgp_ctx *c);
int mgp_fft_setup(mgp_ctx *c);
void mgp_fft_free(mgp_ctx *c);
int mgp_fft_r2c(mgp_ctx *c, float *in, float *out);
int mgp_fft_c2r(mgp_ctx *c, float *grid);
int mgp_fft_forces(mgp_ctx *c, const float *spec, float mult, int t_x, int t_rest);
int mgp_fft_c2r_filtered(mgp_ctx *c, const float *in, float *out, int kind, int filter, float kR1, float norm);
/* learned force closure (mgp_nn.cu): adds its residual to the force grids */
int mgp_closure_apply(struct mgp_closure *cl, mgp_ctx *c, double A);
/* waits for a pending snapshot write and frees the output buffers (mgp_destroy) */
int mgp_run_release(mgp_ctx *c);

/* scale-dependent growth (mgp_sd.cu) */
int mgp_sd_alloc(mgp_ctx *c);
void mgp_sd_free(mgp_ctx *c);
/* keep delta(k) and the complex 2LPT source S(k) of the IC (stored as
 * delta and -S, src/2LPT.c:301-309, 1336-1344) */
int mgp_sd_store(mgp_ctx *c, const float *deltak, const float *source2k);
/* fields of `types` (one per slot) at A (and AFF for deltaD) */
int mgp_sd_fields(mgp_ctx *c, double A, double AFF, int n, const int *types);
/* IC particle state from the D (slot 0) and dDdy (slot 2) fields */
int mgp_sd_init_particles(mgp_ctx *c);

int mgp_launch_fill(float *p, long long n, float value, cudaStream_t st);
int mgp_launch_cic(const float *s, const mgp_dstate *st, long long np, int Ns, int N, double box,
                   float wpar, float *rho, long long P, cudaStream_t stream, int nbox = 1, long long g_bs = 0);
int mgp_launch_cic_range(const float *s, const mgp_dstate *st, long long np, long long p0, long long p1, int Ns, int N,
                         double box, float wpar, float *rho, long long P, cudaStream_t stream);
int mgp_launch_pofk(const float *dk, int N, const int *rk_bin, const float *win, int nbins,
                    double *block_part, int nblocks, double *sums, cudaStream_t st);
int mgp_launch_pofk_thr(const float *dk, int N, const int *thr, const float *win, int nbins, int bintype, double kmin,
                        double kmax, double *block_part, int nblocks, double *sums, int fuse_kind, int filter,
                        float *fuse_out, float fuse_a, float fuse_b, cudaStream_t st, int nbox = 1,
                        long long g_bs = 0, long long sum_bs = 0);
int mgp_launch_forces(const float *dk, const float *mgk, float mg_coupling, float mg_mass2, int mg_kind,
                      int N, double box, float *frc, long long grid_floats, cudaStream_t st, int nbox = 1,
                      const mgp_box_scalars *bs = NULL);
int mgp_launch_ikd(const float *frc, long long grid_floats, int N, long long P, int Ns, long long np,
                   float *s, float *v, const float *D1, const float *D2, mgp_dstate *dst,
                   double *partials, int nblocks, const mgp_kd_args *a, cudaStream_t st, int nbox = 1,
                   const mgp_box_scalars *bs = NULL, const unsigned *qlat = NULL);
int mgp_ikd_blocks(long long np);
/* cell-tile order (mgp_tiles.cu) */
int mgp_tile_side(int N, long long np);
int mgp_tiles_check(const mgp_ctx *c, int T);
int mgp_tiles_alloc(mgp_ctx *c, int T);
void mgp_tiles_free(mgp_ctx *c);
int mgp_tiles_sort(mgp_ctx *c, int T);
int mgp_cic_tiles(mgp_ctx *c, float wpar, int per_sm = 0);
/* single-box tile deposit writing every cell itself (no pre-set mesh) */
int mgp_cic_tiles_own(mgp_ctx *c, float wpar);
/* kick + drift in the order of the last mgp_tiles_sort, the particle
 * arrays rewritten in that order */
int mgp_ikd_tiles(mgp_ctx *c, const mgp_kd_args *a, int *nblocks_out);
/* lattice order of the particle arrays (no-op unless permuted) */
int mgp_particles_canonical(mgp_ctx *c);
int mgp_launch_nu_table(float *tab, int nrk, double kfac, double fac, const double *x, const double *val,
                        const double *dval, int nx, const double *den, cudaStream_t st);
int mgp_launch_nu_add(float *dk, const float *dk0, int N, double cdmfac, const float *nufac, cudaStream_t st);
int mgp_launch_cic_unit(const double *pos, long long n, int N, long long P, float wpar, float *rho, cudaStream_t st);
int mgp_launch_ic_from_density(float *dk, int N, int Ns, double normfac, const double *gc, const double *rescale,
                               cudaStream_t st);
long long mgp_kernel_launches(void);

/* MG real-space and k-space passes */
int mgp_launch_div_laplacian(const float *dk, float *out, int N, float norm, cudaStream_t st, int nbox = 1,
                             long long g_bs = 0);
int mgp_launch_smooth(const float *dk, float *out, int N, int filter, float kR_per_sqrtRK, float norm, cudaStream_t st,
                      int nbox = 1, long long g_bs = 0);
int mgp_launch_screen_potential(float *rho, const float *phi, long long n, float phicrit, cudaStream_t st,
                                int nbox = 1, const mgp_box_scalars *bs = NULL);
int mgp_launch_screen_density(float *rho, const float *dsm, long long n, float coupling, float pref,
                              cudaStream_t st, int nbox = 1, const mgp_box_scalars *bs = NULL, float base = 0.0f);
int mgp_launch_scale_complex(float *c, long long ncomplex, float factor, cudaStream_t st);
/* a user's screening function from its per-step table (mgp_model_hooks) */
#define MGP_SCREEN_TABLE 16384
int mgp_launch_screen_table(float *rho, const float *arg, long long n, float mult, const float *tab, int nt, double us,
                            double t0, double dt, cudaStream_t st);

/* IC */
int mgp_launch_ic_delta(const uint32_t *seedtable, const double *amp_rk, const unsigned char *cut1d,
                        int N, int Ns, double box, int fixed, int inverted, int sphere, float *dk,
                        cudaStream_t st);
int mgp_launch_ic_grad6(const float *dk, float *out6, long long grid_floats, int N, cudaStream_t st);
int mgp_launch_ic_source(float *g6, long long grid_floats, int N, long long P, cudaStream_t st);
int mgp_launch_ic_disp(const float *dk, const float *src, float *out6, long long grid_floats, int N, double box,
                       cudaStream_t st);
int mgp_launch_cic_rsd(const float *s, const float *v, const float *D1, const float *D2, long long lpt_stride,
                       int lpt_pitch, const mgp_dstate *st, long long np, int Ns, int N, double box, float wpar,
                       int axis, float vnorm, float g1, float g2, float *rho, long long P, cudaStream_t stream);
int mgp_launch_pofk_mu(const float *dk, int N, const int *rk_bin, const float *win, int nbins, double *block_part,
                       int nblocks, double *sums, cudaStream_t st);
int mgp_launch_aos_to_soa(const float *in, float *out, long long np, cudaStream_t st);
int mgp_launch_output(const float *s, const float *v, const float *D1, const float *D2, long long lpt_stride,
                      int lpt_pitch, const mgp_dstate *dst, long long np, int Ns, double box, double lengthfac,
                      double vfac, double dDdy, double dD2dy, double cola, float *pos, float *vel, cudaStream_t st);
int mgp_launch_ic_readout(const float *g6, long long grid_floats, int N, long long P, int Ns,
                          float *D1, float *D2, double *partials, int nblocks, cudaStream_t st);
int mgp_launch_ic_finish(float *D1, float *D2, float *s, float *v, long long np, const double *partials,
                         int nblocks, float Di, float Di2, float vD, float vD2, cudaStream_t st);
int mgp_launch_finalize_kd(mgp_dstate *dst, const double *partials, int nblocks, long long np,
                           double dda_omega, double dyyy, int do_drift, cudaStream_t st);
int mgp_launch_positions(const float *s, const mgp_dstate *dst, long long np, int Ns, double box,
                         float *out_pos, float *out_vel, const float *v, cudaStream_t st);
int mgp_launch_set_state(float *s, float *v, const float *pos, const float *vel, long long np, int Ns,
                         double box, cudaStream_t st);
int mgp_launch_set_state_range(float *s, float *v, const float *pos, const float *vel, long long np, int Ns,
                               double box, long long p0, long long p1, cudaStream_t st);

#endif
