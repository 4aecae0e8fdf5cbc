/*
 * mgpicola.h -- C ABI of the GB300 COLA particle-mesh step and 2LPT IC path.
 *
 * Drop-in boundary for MG-PICOLA's hot path.  Every entry point is extern "C",
 * takes plain pointers and sizes, and returns an int status (MGP_OK = 0,
 * negative MGP_E* on failure; mgp_last_error() gives the message).  The
 * reference aborts the whole MPI job instead (FatalError, src/auxPM.c:668-673).
 *
 * Ownership: the library owns all device memory of a context; the caller owns
 * every host buffer it passes.  One context per host thread; each context
 * owns one CUDA stream and every call is stream-ordered and synchronous on
 * return unless stated otherwise.
 *
 * Reference interfaces replaced (paths within MG-PICOLA-PUBLIC):
 *   mgp_params                 <- parameter-file globals, src/vars.h:60-472,
 *                                 read by read_parameterfile src/read_param.c:107-445
 *   mgp_read_parameterfile     <- read_parameterfile + read_mg_parameters
 *                                 (src/read_param.c:107-445,
 *                                 src/user_defined_functions.h:227-406)
 *   mgp_create                 <- the start-up of main (src/main.c:33-200):
 *                                 set_units, initialize_powerspectrum,
 *                                 initialize_ffts, init_modified_version
 *   mgp_displacement_fields    <- displacement_fields (src/2LPT.c:185-1519) +
 *                                 the particle assignment of src/main.c:231-309
 *   mgp_get_displacements      <- GetDisplacements (src/auxPM.c:37-103):
 *                                 PtoMesh + ComputeFifthForce + Forces
 *   mgp_kick_drift             <- MtoParticles (src/auxPM.c:560-644) +
 *                                 Kick (src/main.c:688-742) + Drift
 *                                 (src/main.c:747-787), fused
 *   mgp_pofk                   <- compute_power_spectrum (src/compute_pofk.c:71-271)
 *   mgp_run                    <- the time loop of main (src/main.c:394-611)
 *   mgp_get_particles          <- the particle data read by Output
 *                                 (src/main.c:792-1061)
 */
#ifndef MGPICOLA_H
#define MGPICOLA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status */
#define MGP_OK 0
#define MGP_EINVAL -1       /* invalid argument or parameter value */
#define MGP_ECUDA -2        /* CUDA runtime error */
#define MGP_ECUFFT -3       /* cuFFT error */
#define MGP_ENOMEM -4       /* allocation failed */
#define MGP_EIO -5          /* file could not be read or written */
#define MGP_EPARAM -6       /* parameter file: unknown, duplicate or missing key */
#define MGP_ESTATE -7       /* call out of order (e.g. forces before density) */
#define MGP_ENUMERIC -8     /* ODE / numerical failure */

/* ------------------------------------------------------------ models */
/* The reference picks the model at compile time (Makefile:61-106). */
#define MGP_MODEL_LCDM 0
#define MGP_MODEL_FOFR 1        /* Hu-Sawicki f(R), potential screening */
#define MGP_MODEL_DGP 2         /* normal-branch DGP, density screening */
#define MGP_MODEL_BRANSDICKE 3  /* JBD: Geff(a) rescaling of the density */
#define MGP_MODEL_MBETA 4       /* general m(a), beta(a) (symmetron example) */

#define MGP_FILTER_NONE 0
#define MGP_FILTER_GAUSSIAN 1
#define MGP_FILTER_TOPHAT 2
#define MGP_FILTER_SHARPK 3

/* Run parameters.  Field names are the parameter-file keys of the
 * reference (src/read_param.c:167-265, src/user_defined_functions.h:233-405,
 * paramfiles/additions_compute_pofk.txt). */
typedef struct mgp_params {
  /* model selection (compile-time in the reference) */
  int model;
  int smoothing_filter;            /* GAUSSIANFILTER etc. (src/mg.h:318-338) */
  int use_w0wa;                    /* EQUATIONOFSTATE_PARAMETRIZATION */
  int scaledependent;              /* SCALEDEPENDENT build */

  /* modified gravity */
  int modified_gravity_active;
  int include_screening;
  int use_lcdm_growth_factors;
  int input_pofk_is_for_lcdm;
  int input_sigma8_is_for_lcdm;
  int inverted_initial_condition;
  int amplitude_fixed_initial_condition;
  double fofr0, nfofr;             /* FOFR */
  double Rsmooth, rcH0_DGP;        /* DGP */
  double wBD, Omegah2, Omegarh2, Omegavh2;   /* BRANSDICKE */
  double range_symm, assb_symm, beta_symm;  /* MBETA */
  double w_0, w_a;

  /* P(k) */
  int pofk_compute_every_step;
  int pofk_compute_rsd_pofk;
  int pofk_nbins;
  int pofk_bintype;
  int pofk_subtract_shotnoise;
  double pofk_kmin, pofk_kmax;

  /* outputs */
  char OutputDir[500];
  char FileBase[500];
  char OutputRedshiftFile[500];
  int NumFilesWrittenInParallel;

  /* simulation */
  int UseCOLA;
  double Buffer;
  int Nmesh;
  int Nsample;
  double Box;
  double Init_Redshift;
  int Seed;
  int SphereMode;
  int WhichSpectrum;
  int WhichTransfer;
  char FileWithInputSpectrum[500];
  char FileWithInputTransfer[500];

  /* cosmology */
  double Omega;
  double OmegaBaryon;
  double HubbleParam;
  double Sigma8;
  double PrimordialIndex;

  /* units */
  double UnitLength_in_cm;
  double UnitMass_in_g;
  double UnitVelocity_in_cm_per_s;
  double InputSpectrum_UnitLength_in_cm;

  /* output list (read_outputs, src/read_param.c:32-89); descending z */
  int Noutputs;
  double output_redshift[64];
  int output_nsteps[64];

  /* k grid of the scale-dependent growth tables (not parameter-file keys;
   * src/cosmo.c:803-805 hard-codes them): number of log-spaced k and the
   * range in h/Mpc.  0 selects the reference's grid, 1000 points in
   * [pi/Box, 4 pi sqrt(3) Nmesh/Box]. */
  int sd_nk;
  double sd_kmin, sd_kmax;
  /* initial conditions from particle files (src/readICfromfile.c, the
   * READICFROMFILE build): when ReadParticlesFromFile is set,
   * mgp_displacement_fields deposits the particles of NumInputParticleFiles
   * files, takes their density as the LCDM linear field at Init_Redshift and
   * runs the 2LPT IC from it.  TypeInputParticleFiles: 1 RAMSES
   * (<dir>/part_<RamsesOutputNumber %05d>.out<n %05d>, n = 1..), 2 ASCII
   * (<dir>/<prefix>.<n>, n = 1.., "npart" then "x y z mass" in [0,1)),
   * 3 GADGET-1 (<dir>/<prefix>.<n>, n = 0.., type-1 positions in Box units).
   * Setting ReadParticlesFromFile before mgp_read_parameterfile makes the six
   * keys required, as the READICFROMFILE build does. */
  int ReadParticlesFromFile, NumInputParticleFiles, RamsesOutputNumber, TypeInputParticleFiles;
  char InputParticleFileDir[500], InputParticleFilePrefix[500];
  /* massive neutrinos (the MASSIVE_NEUTRINOS build, which needs
   * scaledependent = 1): massive_neutrinos plays the build flag (the three
   * nu_ keys are read from a parameter file when it is set before
   * mgp_read_parameterfile); nu_include_massive_neutrinos switches them on,
   * Omega_nu = nu_SumMassNuEV / (93.14 h^2), and nu_FilenameTransferInfofile
   * names "<dir> <n>" followed by n lines "<file> <z>" of CAMB transfer
   * files (one header line, 13 columns: k/h, T_cdm, T_b, T_g, T_nu,
   * T_massive_nu, T_tot, ...), z increasing.  The linear P(k) is then the
   * CDM+baryon spectrum of those files and every step adds the neutrino
   * density to delta(k) (src/auxPM.c:383-428). */
  int massive_neutrinos, nu_include_massive_neutrinos;
  double nu_SumMassNuEV;
  char nu_FilenameTransferInfofile[500];
} mgp_params;

typedef struct mgp_ctx mgp_ctx;

/* Fill *p with the defaults used by the reference's example parameter
 * files (paramfiles/example_*.txt). */
int mgp_params_default(mgp_params *p);

/* read_parameterfile (src/read_param.c:107-445) for `model`: every key the
 * reference registers for that model is mandatory, unknown or repeated keys
 * are errors, '%' starts a comment.  Also reads OutputRedshiftFile
 * (read_outputs, src/read_param.c:32-89) unless read_outputs == 0, and the
 * tabulated spectrum for WhichSpectrum == 1 at mgp_create time. */
int mgp_read_parameterfile(const char *fname, int model, int pofk_keys, int read_outputs, mgp_params *p);

/* Start-up: validate parameters, solve the growth ODEs, normalise the power
 * spectrum, allocate device memory on `device` and plan the FFTs. */
int mgp_create(const mgp_params *p, int device, mgp_ctx **out);

/* User model hooks: the functions a user of the reference edits in
 * src/user_defined_functions.h to define a gravity model (lines 413-904),
 * as host FP64 callbacks.  Every member is optional: NULL keeps the built-in
 * model that mgp_params selects, and the built-in functions call the other
 * hooks through the same table (the built-in GeffoverG of f(R) uses a user
 * mass2_of_a, as in the reference).  `user` is passed to every call.  The
 * library calls them on the host only: while the growth tables are solved
 * at mgp_create, and once per step for the step's scalars (coupling, mass
 * term, phi_crit, Factor_2LPT) and screening tables.
 *   hubble, dhubbleda     H(a)/H0 and its a-derivative          (:413-452)
 *   GeffoverG             mu(a, k), k in h/Mpc                  (:618-660)
 *   beta_of_a, mass2_of_a, dmass2_of_ada
 *                         coupling strength, m^2(a)/H0^2 and d/da (:462-560)
 *   coupling_function     the coupling of the fifth-force equation (:587-611)
 *   phi_of_a              phi_crit(a) of the potential screening (:571-579,
 *                         the f(R) form of :725-750 for FOFR)
 *   screening_factor_potential / screening_factor_density
 *                         the screening factors as functions of the Newtonian
 *                         potential or the smoothed density (:725-773); the
 *                         device applies them through a table of 16384
 *                         values per step over asinh-spaced arguments
 *                         (linear interpolation, ~1e-6 relative), where the
 *                         built-in forms are evaluated exactly
 *   Factor_2LPT           the 2LPT source factor (:814-838)
 *   second_order_kernel   gamma_2(k, k1, k2, cos theta, a) of the
 *                         scale-dependent 2LPT growth (:862-904) */
typedef struct mgp_model_hooks {
  void *user;
  double (*hubble)(double a, void *user);
  double (*dhubbleda)(double a, void *user);
  double (*GeffoverG)(double a, double k, void *user);
  double (*beta_of_a)(double a, void *user);
  double (*mass2_of_a)(double a, void *user);
  double (*dmass2_of_ada)(double a, void *user);
  double (*coupling_function)(double a, void *user);
  double (*phi_of_a)(double a, void *user);
  double (*screening_factor_potential)(double a, double phinewton, void *user);
  double (*screening_factor_density)(double a, double density, void *user);
  double (*Factor_2LPT)(double a, void *user);
  double (*second_order_kernel)(double k, double k1, double k2, double costheta, double a, void *user);
} mgp_model_hooks;

/* mgp_create with user model hooks (NULL hooks = mgp_create).  The table is
 * copied; `user` must stay valid for the context's life. */
int mgp_create_with_hooks(const mgp_params *p, const mgp_model_hooks *hooks, int device, mgp_ctx **out);
/* Host-only cosmology of a parameter set with hooks, as mgp_cosmo_eval
 * (which 0-9); `which` 10-15 give the model functions themselves at a = x
 * as the library evaluates them (10 hubble, 11 GeffoverG at k = 0.1 h/Mpc,
 * 12 coupling_function, 13 mass2_of_a, 14 phi_crit, 15 Factor_2LPT). */
int mgp_cosmo_eval_hooks(const mgp_params *p, const mgp_model_hooks *hooks, int which, const double *x, int n,
                         double *out);
int mgp_destroy(mgp_ctx *ctx);
const char *mgp_last_error(void);

/* 2LPT initial conditions on the device (displacement_fields + the particle
 * assignment of main.c:231-309): afterwards the context holds positions at
 * a_init = 1/(1+Init_Redshift), zero COLA velocities and the Lagrangian
 * displacements D1 (ZA) and D2 (2LPT, times -3/7). */
int mgp_displacement_fields(mgp_ctx *ctx);
/* displacement_fields from particles held by the caller instead of files
 * (the ReadParticlesFromFile path, src/readICfromfile.c:533-777): n
 * positions in Mpc/h, [n][3]; their CIC density at Init_Redshift is taken as
 * the LCDM linear field.  For Nmesh <= Nsample the three Nyquist planes of
 * that field are zeroed (the reference uses +N/2 there in its displacement
 * and -N/2 in its gradient pass); for Nmesh > Nsample its |k| > Nsample/2 cut
 * removes them anyway. */
int mgp_displacement_fields_from_positions(mgp_ctx *ctx, const double *pos, size_t n);
/* The IC particle files of p read on the host (readICfromfile.c:221-531):
 * *pos receives n positions in [0,1) of the box, [n][3], allocated by the
 * library; release it with mgp_free_particles. */
int mgp_read_particle_files(const mgp_params *p, double **pos, size_t *n);
void mgp_free_particles(double *pos);

/* GetDisplacements at scale factor A: CIC density, forward FFT, optional
 * P(k) (pofk_compute_every_step), fifth force, and the force grids. */
int mgp_get_displacements(mgp_ctx *ctx, double A);

/* Fused MtoParticles + Kick (AI -> AF at A) [+ Drift A -> AFF].  Requires a
 * preceding mgp_get_displacements at the same A. */
int mgp_kick_drift(mgp_ctx *ctx, double AI, double AF, double A, double AFF, int do_drift);

/* One KDK step (main.c:410-602 body for a non-output step); with
 * scale-dependent growth it also assigns that step's ddDddy and deltaD
 * fields (main.c:487-503). */
int mgp_step(mgp_ctx *ctx, double A, double AI, double AF, double AFF);

/* Scale-dependent growth (contexts created with scaledependent = 1, the
 * reference's SCALEDEPENDENT build): assign_displacment_field_to_particles
 * (src/2LPT.c:1758-2005) with from_cdisp_store_to_ZA (src/2LPT.c:1539-1735)
 * for `n` (1-3) field types at once, each for both LPT orders.  Field types
 * as src/proto.h:155-158.  The context keeps one particle slot per role, as
 * the reference's P[] members: D and ddDddy go to the slot the Kick reads
 * (P.D/P.D2), deltaD to the one the Drift reads (P.dDdy/P.dD2dy), dDdy to a
 * velocity slot for outputs and RSD (the reference puts it into P.dDdy and
 * restores deltaD afterwards, src/main.c:1051-1053, compute_pofk.c:409-500),
 * so two types of one slot in a call are MGP_EINVAL.  deltaD uses
 * D(k, AFF) - D(k, A).  Requires Nmesh to be a multiple of Nsample. */
#define MGP_FIELD_D 0
#define MGP_FIELD_dDdy 1
#define MGP_FIELD_ddDddy 2
#define MGP_FIELD_deltaD 3
int mgp_assign_displacement_fields(mgp_ctx *ctx, double A, double AFF, int n, const int *fieldtypes);

/* Full time loop with outputs (main.c:394-611).  Writes snapshot files
 * (GADGET-1 when gadget != 0, else ASCII) and pofk_* files to OutputDir. */
int mgp_run(mgp_ctx *ctx, int gadget);
/* mgp_run writes each snapshot from pinned host memory (two slots) on a host
 * thread while the next steps run; the files are complete when mgp_run
 * returns.  Statistics since the context was created, host milliseconds:
 * snapshots, writers waiting for the GPU to reach the snapshot and download
 * it, writers writing files, and the caller's thread held by output launches
 * and waits for a free slot. */
int mgp_output_stats(mgp_ctx *ctx, int *count, double *wait_ms, double *file_ms, double *blocked_ms);

/* P(k) of the most recent density (compute_power_spectrum).  Arrays of
 * capacity `cap`; *nbins receives the bin count after the reference's
 * parameter adjustment (compute_pofk.c:758-805).  k = k_from_index,
 * kmean = mean |k| of the modes, n = mode count (weights as the reference). */
int mgp_pofk(mgp_ctx *ctx, int cap, int *nbins, double *k, double *pk, double *kmean, double *n);

/* Total matter P(k) of a run with massive neutrinos (the "total" spectrum
 * of src/auxPM.c:423-426: delta(k) after the neutrino density was added in
 * the last mgp_get_displacements); without neutrinos the same as mgp_pofk. */
int mgp_pofk_total(mgp_ctx *ctx, int cap, int *nbins, double *k, double *pk, double *kmean, double *n);

/* RSD multipoles P0/P2/P4 for LOS y and z (compute_RSD_powerspectrum,
 * src/compute_pofk.c:403-512) at the current particle state.  The seven
 * output arrays (k, P0, P2, P4 averaged over y and z, and the sigma
 * columns) have capacity `cap`. */
int mgp_pofk_rsd(mgp_ctx *ctx, double A, int cap, int *nbins, double *k, double *P0, double *P2,
                 double *P4, double *s0, double *s2, double *s4, double *n);

/* Particle state, host buffers of [np][3] floats (AoS, the order of
 * struct part_data's Pos/Vel/D/D2, src/vars.h:292-321).  Positions are
 * wrapped to [0, Box); velocities are the internal COLA velocities
 * (Vel - <Vel> is what Drift uses).  Any pointer may be NULL; setting only
 * positions (velocities) leaves the velocities (positions) as they were. */
int mgp_get_particles(mgp_ctx *ctx, float *pos, float *vel, float *D1, float *D2, size_t np);
int mgp_set_particles(mgp_ctx *ctx, const float *pos, const float *vel, const float *D1,
                      const float *D2, size_t np);

/* Host-buffer step for drop-in callers that keep particles in host memory:
 * copies pos/vel/D1/D2 in, runs mgp_step, copies pos/vel back.  The
 * positions are uploaded in chunks that are deposited as they arrive; the
 * other arrays travel on a second stream while the step runs.  With
 * scale-dependent growth the step assigns its own LPT fields, so D1/D2 are
 * not read (as mgp_set_particles). */
int mgp_step_host(mgp_ctx *ctx, double A, double AI, double AF, double AFF, float *pos, float *vel,
                  const float *D1, const float *D2, size_t np);

/* Growth factors and COLA coefficients of the context's cosmology
 * (src/cosmo.c:318-403, 1114-1160). which: 0 D, 1 dD/dy, 2 d2D/dy2,
 * 3 D2, 4 dD2/dy, 5 d2D2/dy2, 6 D_LCDM. */
double mgp_growth(mgp_ctx *ctx, int which, double a);
double mgp_Sq(mgp_ctx *ctx, double ai, double af, double aref);
double mgp_Sphi(mgp_ctx *ctx, double ai, double af, double aref);
double mgp_power_spectrum(mgp_ctx *ctx, double k);

/* Host-only cosmology of a parameter set (no device needed): which 0-6 as
 * mgp_growth, 7 the linear P(k) at x = k (h/Mpc), 8 mg_pofk_ratio(k = x,
 * a = 1), 9 mg_sigma8_enhancement(a = x) (src/cosmo.c:688-756);
 * mgp_cosmo_coeff gives Sq (kind 0) or Sphi (kind 1) for n triples
 * (ai, af, aref), or SqStd (2) / SphiStd (3) of (ai, af), the coefficients
 * of a run with UseCOLA = 0 (src/cosmo.c:1165-1200). */
int mgp_cosmo_eval(const mgp_params *p, int which, const double *x, int n, double *out);
/* growth_*_scaledependent(k, a) (src/cosmo.c:987-1010) of a parameter set
 * with scaledependent = 1, host only: which 0 D, 1 dD/dy, 2 d2D/dy2, 3 D2,
 * 4 dD2/dy, 5 d2D2/dy2 at n pairs (k in h/Mpc, a), normalised at a = 1 per k. */
int mgp_growth_scaledependent(const mgp_params *p, int which, const double *k, const double *a, int n, double *out);
int mgp_cosmo_coeff(const mgp_params *p, int kind, const double *ai, const double *af, const double *aref, int n,
                    double *out);

/* Batches of independent boxes (no counterpart in the reference, which runs
 * one box per MPI job: a parameter sweep is many runs of main).  All boxes
 * share Nmesh, Nsample, Box, the model, its switches and the background;
 * each has its own seed, IC flags and, for f(R) / nDGP, its own |fR0| /
 * rcH0 (values <= 0 keep the common one).  Every kernel and FFT of the PM
 * step covers all boxes at once, and mgp_batch_run captures the whole KDK
 * loop of main.c:394-611 (one output at z_final, nsteps steps, P(k) at
 * every step when pofk_compute_every_step) into one CUDA graph launch.
 * Scale-independent growth only.  The context returned works only with the
 * mgp_batch_* calls and mgp_destroy. */
typedef struct mgp_box_params {
  int Seed;
  int inverted_initial_condition;
  int amplitude_fixed_initial_condition;
  double fofr0;
  double rcH0_DGP;
} mgp_box_params;
int mgp_batch_create(const mgp_params *p, int nbox, const mgp_box_params *boxes, int device, mgp_ctx **out);
/* 2LPT ICs of every box, then the captured loop (built on the first call
 * for this nsteps / z_final and replayed afterwards). */
int mgp_batch_run(mgp_ctx *ctx, int nsteps, double z_final);
/* P(k) of box `box` at step `step` (0 .. nsteps; step nsteps is z_final),
 * arrays as mgp_pofk. */
int mgp_batch_pofk(mgp_ctx *ctx, int box, int step, int cap, int *nbins, double *k, double *pk, double *kmean,
                   double *n);
/* Final particles of one box, as mgp_get_particles. */
int mgp_batch_get_particles(mgp_ctx *ctx, int box, float *pos, float *vel, size_t np);
/* CUDA-event milliseconds of the last mgp_batch_run: what 0 = the captured
 * loop (one graph launch), 1 = the ICs; and the captured graph's node count. */
double mgp_batch_ms(mgp_ctx *ctx, int what);
int mgp_batch_graph_nodes(mgp_ctx *ctx);
/* this library's own kernels among them (the rest are cuFFT's) */
int mgp_batch_graph_kernels(mgp_ctx *ctx);
/* Launch budgets in resident blocks per SM: [0] CIC deposit, [1] grid passes
 * (fill, forces, MG passes), [2] interp+kick+drift, [3] P(k) binning
 * (defaults 8, 8, 8, 4).  They change launch shapes only; the next run
 * captures a new graph.  mgp_batch_autotune picks them by coordinate descent,
 * timing one mgp_batch_run of nsteps per candidate, and leaves the fastest
 * set (its graph time in *best_ms). */
int mgp_batch_set_tuning(mgp_ctx *ctx, const int tune[4]);
int mgp_batch_get_tuning(mgp_ctx *ctx, int tune[4]);
/* Deposit form of a batch: 0 (default) one thread per particle in lattice
 * order; 8 or 16: every step all boxes' particles are bucketed by the
 * side^3-cell tile of their CIC base cell (a counting sort inside the
 * graph) and each tile is summed in shared memory before one float2
 * reduction per pair of mesh cells.  side must divide Nmesh.  The density
 * agrees up to the order of float sums; the next run captures a new graph.
 * get returns the side (or a negative error code). */
int mgp_batch_set_deposit_tiles(mgp_ctx *ctx, int side);
int mgp_batch_get_deposit_tiles(mgp_ctx *ctx);
/* The autotuner also picks the deposit form (after the grid budget, before
 * the deposit budget), timing each side that applies. */
int mgp_batch_autotune(mgp_ctx *ctx, int nsteps, double z_final, double *best_ms);

/* Learned force closure (no counterpart in the reference): a 3D CNN on the
 * PM mesh -- four periodic 3x3x3 convolutions, 16 channels, ReLU, BF16
 * weights and activations with FP32 accumulation on the tensor cores --
 * that maps [asinh(delta), Phi_N/1e-5, screening factor] to a
 * residual force added to the mesh force.  Trained on the GPU against the
 * force of a finer mesh for the same particles (Nmesh_fine = r Nmesh), with
 * this library's forward and backward kernels and Adam.  Nmesh must be a
 * multiple of 16.  Weight layout: w [4][27 taps][16 out][16 in], tap =
 * 9 (di+1) + 3 (dj+1) + (dk+1), b [4][16]; the last layer has 3 live outputs. */
typedef struct mgp_closure mgp_closure;
int mgp_closure_create(int Nmesh, unsigned seed, int device, mgp_closure **out);
int mgp_closure_destroy(mgp_closure *cl);
int mgp_closure_get_weights(mgp_closure *cl, float *w, float *b, float *out_scale);
int mgp_closure_set_weights(mgp_closure *cl, const float *w, const float *b, float out_scale);
/* Working sample from the host ([V][3] features and targets, FP32; either
 * may be NULL), forward pass (out [V][3] or NULL), loss and gradients
 * without an update, one Adam step (returns the loss before it). */
int mgp_closure_set_sample(mgp_closure *cl, const float *x, const float *t);
int mgp_closure_get_sample(mgp_closure *cl, float *x, float *t);
int mgp_closure_forward(mgp_closure *cl, float *out);
int mgp_closure_gradients(mgp_closure *cl, double *loss, float *gw, float *gb);
int mgp_closure_train_step(mgp_closure *cl, float lr, double *loss);
/* Training data from contexts after mgp_get_displacements at scale factor A:
 * features of the coarse context, and the target = fine force averaged onto
 * the coarse mesh minus the coarse force (*rms its rms, may be NULL). */
int mgp_closure_features(mgp_closure *cl, mgp_ctx *coarse, double A);
int mgp_closure_target(mgp_closure *cl, mgp_ctx *fine, mgp_ctx *coarse, double *rms);
/* Particle-level target (the loss a closure is trained with for use in a
 * run): per particle, the fine context's force interpolated at the particle
 * minus the coarse context's, r_p = F_fine(x_p) - F_coarse(x_p), with the
 * particle's cell coordinates on the coarse mesh.  With such a sample the
 * loss is the mean over particles and components of (out_scale u_p - r_p)^2,
 * u_p the CIC interpolation of the network output at x_p, so the network
 * learns the correction as the kick will use it; its gradient is the CIC
 * deposit of the residuals.  A sample made from contexts takes its own rms
 * as the scale and its loss relative to that rms squared (the network
 * predicts the residual in units of its rms, so every time step weighs the
 * same); host samples use out_scale and an unnormalised loss.  The contexts hold the same particles.  band:
 * restrict the fine force to the modes of the coarse mesh first (|k_i| below
 * its Nyquist frequency), which drops the sub-grid force.  Host
 * form: np particles, cells and t [np][3] (cells in mesh units, [0, Nmesh));
 * get returns the working sample's np (0 for a grid target). */
int mgp_closure_target_particles(mgp_closure *cl, mgp_ctx *fine, mgp_ctx *coarse, int band, double *rms);
int mgp_closure_set_particle_sample(mgp_closure *cl, long long np, const float *cells, const float *t);
int mgp_closure_get_particle_sample(mgp_closure *cl, long long *np, float *cells, float *t);
/* Device training set: reserve n slots (np = 0: grid targets; np > 0:
 * particle samples of np particles), store / load the working sample. */
int mgp_closure_reserve(mgp_closure *cl, int n, long long np);
int mgp_closure_store(mgp_closure *cl, int slot);
int mgp_closure_load(mgp_closure *cl, int slot);
/* Use the closure in every later mgp_get_displacements of ctx (NULL detaches):
 * the network output, high-passed (modes of wavelength >= lambda mesh cells
 * and the mean removed; default lambda 0: the mean only) and scaled by
 * out_scale, is added
 * to the force transforms before their C2R.  The particle loss trains the
 * same high-passed output; mgp_closure_forward returns the raw output. */
int mgp_set_closure(mgp_ctx *ctx, mgp_closure *cl);
int mgp_closure_set_highpass(mgp_closure *cl, double lambda_cells);
/* The in-step output scale: a table of the residual rms s(a) of the training
 * snapshots (n points, a increasing), interpolated log-log at the step's
 * scale factor; without a table (n = 0) out_scale is used.  scale_at returns
 * the value the step uses. */
int mgp_closure_set_scale_table(mgp_closure *cl, int n, const double *a, const double *s);
double mgp_closure_scale_at(mgp_closure *cl, double A);
double mgp_closure_get_highpass(mgp_closure *cl);

/* Copy an internal grid to a host buffer (diagnostics and parity tests).
 * which: 0 density (real padded [N][N][2(N/2+1)] float; after the fifth
 * force the MG source, which reuses it), 1 delta(k) (complex [N][N][N/2+1]
 * float pairs; the total matter field once massive neutrinos were added),
 * 2..4 force grids x,y,z (real padded), 5 as 0, 6 the filtered density of
 * the MG solver, 7 the stored IC delta(k) of the scale-dependent build
 * (cdelta_cdm).  `count` is the number of floats. */
int mgp_copy_grid(mgp_ctx *ctx, int which, float *host, size_t count);

/* Kernel timing: CUDA-event milliseconds of the named kernels launched by
 * the last call (names: "cic", "r2c", "pofk", "forces", "c2r", "interp_kick_drift",
 * "mg", "step" = the whole mgp_step); returns -1 if not timed.  Timing is on when enable != 0. */
int mgp_set_timing(mgp_ctx *ctx, int enable);
double mgp_kernel_ms(mgp_ctx *ctx, const char *name);
/* Caller marks (no counterpart in the reference, whose timer.c reads the
 * host clock): mgp_mark records event `slot` (0..3) on the context's stream;
 * mgp_mark_ms waits for mark `to` and returns the device milliseconds from
 * mark `from` to it (-1 on error).  Brackets whole runs without per-step
 * synchronisation. */
int mgp_mark(mgp_ctx *ctx, int slot);
/* Particle order of the deposit and the kick (no counterpart in the
 * reference).  Every step the particles are bucketed by the 16^3-cell (or
 * 8^3) tile of the mesh holding their CIC base cell and deposited per tile
 * in shared memory (tiles = 1 or 2).  tiles = 2 (the default for single
 * boxes): the kick also runs per tile -- the three force grids over the
 * tile staged in shared memory -- and writes the particles back in the
 * tile order, so the arrays follow the particles (with scale-independent
 * growth; the scale-dependent LPT fields keep the array-order kick); entry
 * points that hand particles to the caller, or take them, restore the
 * lattice order first.  tiles = 1: the arrays stay in lattice order and the
 * kick walks them in that order.  tiles = 0: deposit and kick in lattice
 * order.  All give the same results up to the order of float sums. */
int mgp_set_particle_order(mgp_ctx *ctx, int tiles);
/* Transforms of a single box with Nmesh = 1024 (no counterpart in the
 * reference, whose FFTW calls are src/wrappers.c:26-96).  mode 1 (the
 * default there): the z rows with cuFFT's batched 1D transforms and the
 * strided y and x passes with this library's kernels, the force pass of
 * Forces (src/auxPM.c:437-555) fused into the inverse passes; mode 0: cuFFT's
 * 3D plans and the separate force pass.  Both give the same fields up to
 * float rounding.  Other sizes and batches always use the 3D plans (mode 1
 * is accepted and has no effect). */
int mgp_set_fft_mode(mgp_ctx *ctx, int mode);
/* With mgp_set_timing(ctx, n) for n > 1 the stage events of the last n
 * mgp_step calls are kept: milliseconds of stage `name` in step `step`
 * (counted from that mgp_set_timing call), -1 if not kept or not timed. */
double mgp_kernel_ms_step(mgp_ctx *ctx, const char *name, int step);
double mgp_mark_ms(mgp_ctx *ctx, int from, int to);
/* P(k) binning for callers that cannot allocate (no counterpart in the
 * reference): for code running inside another framework's memory pool or
 * allocator hooks, or that must not let cudaMalloc/cudaFree synchronise the
 * device.  Bins the caller's delta(k) grid (device pointer, complex
 * [Nmesh][Nmesh][Nmesh/2+1] float pairs, the R2C of a CIC density) exactly as
 * mgp_pofk does, with every scratch buffer in one fixed-size device array
 * owned by the library (about 11.4 MB, held on each device that loads the
 * library until exit); it calls no cudaMalloc, cudaFree or other allocating
 * routine.  Results are bit-reproducible from call to call.  Limits: even Nmesh <= 1024, at most 2048 bins after the
 * reference's parameter adjustment; larger requests return MGP_EINVAL.  Runs
 * on the current device and on `stream` (NULL = legacy default stream) and
 * returns after the results are in the host arrays.  The first call on a
 * device looks up the array's device address and keeps it for the process,
 * so do not call it on a device after cudaDeviceReset.  All calls share the
 * array: calls whose GPU work overlaps race and must be serialised by the
 * caller. */
int mgp_pofk_noalloc(const float *d_deltak, int Nmesh, int Nsample, double Box, int nbins, int bintype,
                     int subtract_shotnoise, double kmin, double kmax, int cap, int *nbins_out, double *k,
                     double *pk, double *kmean, double *n, void *stream);

/* Process-wide number of this library's own kernel launches so far (cuFFT
 * launches are not included). */
long long mgp_launch_count(mgp_ctx *ctx);

/* Page-lock (pin) a caller-owned host buffer for fast copies, and release it
 * (cudaHostRegister / cudaHostUnregister). */
int mgp_host_register(void *ptr, size_t bytes);
int mgp_host_unregister(void *ptr);
/* Page-locked host allocations (cudaMallocHost / cudaFreeHost) for the
 * particle arrays of the host-buffer step.  Copies from them stayed at the
 * link rate on a busy host, where copies from registered pageable memory
 * (mgp_host_register) slowed down several-fold. */
int mgp_host_alloc(void **ptr, size_t bytes);
int mgp_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif
