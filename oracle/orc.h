/*
 * FP64 CPU oracle for the MG-PICOLA COLA particle-mesh step and 2LPT initial
 * conditions.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; it is the oracle that the CUDA path is compared against
 * (tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
 * bench.py).  Every routine restates one reference routine in double
 * precision and cites it (paths are relative to the MG-PICOLA-PUBLIC tree).
 *
 * Conventions shared with the reference (src/vars.h:292-353 with MEMORY_MODE
 * off, SINGLE_PRECISION off):
 *   - particle arrays are AoS [np][3] doubles (P[i].Pos[3] etc.);
 *   - real grids use the FFTW in-place padded layout [N][N][2(N/2+1)];
 *   - complex grids are [N][N][N/2+1] interleaved (re, im);
 *   - FFTs are unnormalised, forward sign -1, backward sign +1.
 *
 * Parity status: pinned against the reference's own sources compiled with
 * project-written single-rank shims (oracle/ref_shim, output in oracle/_ref)
 * where that build succeeds; see tests/golden/make_golden.py.
 */
#ifndef MGP_ORACLE_H
#define MGP_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- RNG */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Used as the
 * project-defined stand-in for gsl_rng_ranlxd1 in the IC generator. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* One uniform double in [0,1): draw number `n` of the stream seeded by `seed`. */
double orc_stream_uniform(uint32_t seed, uint64_t n);

/* ---------------------------------------------------------------- FFT */
/* In-place 3D real FFTs on an [N][N][2(N/2+1)] double grid, FFTW semantics.
 * Backward (c2r) uses only Re of the kz=0 and kz=N/2 entries after the x/y
 * passes, as a real-output half-complex transform does. */
void orc_fft_r2c(int N, double *grid);
void orc_fft_c2r(int N, double *grid);
/* 1D complex FFT helper for tests (sign -1 forward, +1 backward). */
void orc_fft1d(int n, double *data_interleaved, int sign);

/* ------------------------------------------------------------ PM step */
/* PtoMesh (src/auxPM.c:280-357): density = -1 + CIC(pos) * (N/Ns)^3. */
void orc_cic(const double *pos, long np, int N, int Ns, double box, double *grid);
/* CIC with positions taken as q + disp (lattice q) -- same arithmetic as
 * orc_cic on pos = wrap(q + disp); convenience for tests. */
void orc_lattice_positions(const double *disp, int Ns, double box, double *pos);

/* Forces k-space pass (src/auxPM.c:437-535): from delta(k) (+ optional MG
 * source added first, auxPM.c:450-455) produce the three complex force grids. */
void orc_forces_kspace(const double *deltak, const double *mgk, int N, double box,
                       double *f1, double *f2, double *f3);
/* MtoParticles (src/auxPM.c:560-644); returns per-particle Disp and mean. */
void orc_interp(const double *f1, const double *f2, const double *f3, int N, double box,
                const double *pos, long np, double *disp, double mean_out[3]);
/* Kick (src/main.c:688-742) for scale-independent growth. */
void orc_kick(long np, double *vel, double *disp, const double *D1, const double *D2,
              const double sumD[3], double omega, double dda, double ddD, double ddD2,
              double A, int usecola, double sumv_out[3]);
/* Drift (src/main.c:747-787) for scale-independent growth. */
void orc_drift(long np, double *pos, const double *vel, const double *D1, const double *D2,
               const double sumv[3], double dyyy, double dD, double dD2, int usecola, double box);
double orc_periodic_wrap(double x, double box);

/* compute_power_spectrum (src/compute_pofk.c:71-271).  kmin/kmax in h/Mpc as
 * in the parameter file; the k_bin/P/k_mean/n arrays have `nbins` entries
 * (after adjust_pofk_parameters, compute_pofk.c:758-805, which may change
 * nbins: pass capacity in *nbins_io, get the used count back). */
int orc_pofk(const double *deltak, int N, int Ns, double box, int *nbins_io, int bintype,
             int subtract_shotnoise, double kmin_hmpc, double kmax_hmpc,
             double *kbin, double *pk, double *kmean, double *nmodes);

/* RSD multipoles of one line of sight (compute_pofk.c:518-753).  The
 * LOS axis must be 1 (y) or 2 (z).  vel_los_extra is the per-particle LPT
 * velocity added for COLA (main.c:959-967 form), may be NULL. */
int orc_pofk_rsd_axis(const double *pos, const double *vel, const double *vel_extra, long np,
                      int axis, int N, int Ns, double box, double vnorm,
                      int *nbins_io, int bintype, int subtract_shotnoise,
                      double kmin_hmpc, double kmax_hmpc,
                      double *k, double *P0, double *P2, double *P4, double *n);

/* ------------------------------------------------------- MG screening */
/* Model ids (compile-time MODEL switch in the reference Makefile:61-106). */
enum { ORC_LCDM = 0, ORC_FOFR = 1, ORC_DGP = 2, ORC_JBD_GEFF = 3, ORC_MBETA = 4 };

typedef struct {
  int model;
  int mg_active, include_screening, use_lcdm_growth;
  double omega;            /* Omega_m */
  double fofr0, nfofr;     /* Hu-Sawicki (user_defined_functions.h:490-500) */
  double rcH0, rsmooth;    /* nDGP (user_defined_functions.h:453, mg.h:197-260) */
  double geff_const;       /* Geff/G(a) for the time-dependent-Geff path */
  double w0, wa; int use_w0wa;
  /* m(a)/beta(a) symmetron example (user_defined_functions.h:462-484) */
  double beta_symm, assb_symm, range_symm;
  int smoothing_filter;    /* 0 none, 1 gaussian, 2 tophat, 3 sharpk */
  /* Brans-Dicke background parameters (src/jbd.c) */
  double wBD, Omegah2, Omegarh2, Omegavh2;
  /* SCALEDEPENDENT build: growth factors D(k, a) from 2D tables
   * (src/cosmo.c:798-1010).  sd_nk/sd_kmin/sd_kmax (h/Mpc) override the
   * reference's k grid (1000 points in [pi/Box, 4 pi sqrt(3) N/Box]) when
   * nonzero. */
  int scaledependent;
  int sd_nk;
  double sd_kmin, sd_kmax;
  /* MASSIVE_NEUTRINOS build: transfer tables and Omega's (orc_nu.c), or NULL */
  const struct orc_nu_s *nu;
} orc_mg;

/* Brans-Dicke background (src/jbd.c) and the m(a), beta(a) phi_crit(a)
 * integral (src/cosmo.c:104-190): solved into oracle-global splines used by
 * the hooks below; orc_jbd_solve returns h and writes Omega = Omegah2/h^2. */
double orc_jbd_solve(orc_mg *m);
void orc_phia_solve(const orc_mg *m, double init_redshift);
double orc_phicrit(const orc_mg *m, double a);

double orc_hubble(const orc_mg *m, double a);
double orc_dhubbleda(const orc_mg *m, double a);
double orc_beta_dgp(const orc_mg *m, double a);
double orc_beta_of_a(const orc_mg *m, double a);
double orc_mass2_of_a(const orc_mg *m, double a);
double orc_coupling(const orc_mg *m, double a);
double orc_geff(const orc_mg *m, double a, double k);
double orc_factor_2lpt(const orc_mg *m, double a);
/* dmass2_of_ada (user_defined_functions.h:527-560) and the second-order
 * kernel gamma_2(k, k1, k2, cos theta, a) (user_defined_functions.h:848-904) */
double orc_dmass2_of_ada(const orc_mg *m, double a);
double orc_second_order_kernel(const orc_mg *m, double k, double k1, double k2, double costheta, double a);
double orc_screen_potential(const orc_mg *m, double a, double phinewton);
double orc_screen_density(const orc_mg *m, double a, double density);

/* ComputeFifthForce (user_defined_functions.h:687-719 + src/mg.h).
 * density_x: real-space density copy (CopyDensityArray), deltak: P3D.
 * Writes the complex MG source to mgk (P3D_mgarray_two) when the model uses
 * MG arrays; multiplies deltak in place for the time-dependent Geff path. */
void orc_fifth_force(const orc_mg *m, double a, int N, double box,
                     const double *density_x, double *deltak, double *mgk);

/* ------------------------------------------------- 2D bicubic tables */
/* GSL gsl_interp2d_bicubic restated (orc_interp2d.c); z[j * nx + i]. */
typedef struct {
  int nx, ny;
  double *x, *y, *z, *zx, *zy, *zxy;
} orc_bicubic;
void orc_bicubic_init(orc_bicubic *b, const double *x, const double *y, const double *z, int nx, int ny);
double orc_bicubic_eval(const orc_bicubic *b, double x, double y);
void orc_bicubic_free(orc_bicubic *b);

/* ------------------------------------------------- massive neutrinos */
/* orc_nu.c: CAMB transfer tables over (ln k, z) read from the info file
 * (src/read_CAMB_data.h), OmegaNu = sum m_nu / (93.14 h^2) and OmegaCDM as
 * init_modified_version sets them, the growth-equation factors, the CDM+
 * baryon P(k) and the per-step k-space density add.  which: 0 massive nu,
 * 1 CDM, 2 baryon, 3 total. */
typedef struct orc_nu_s orc_nu;
orc_nu *orc_nu_create(const char *infofile, double omega, double omega_b, double h, double ns, double sum_mnu_ev,
                      int include);
void orc_nu_free(orc_nu *nu);
double orc_nu_omega_nu(const orc_nu *nu);
double orc_nu_omega_cdm(const orc_nu *nu);
double orc_nu_transfer(const orc_nu *nu, int which, double k, double a);
double orc_nu_Tcb(const orc_nu *nu, double k, double a, double omega_cdm);
double orc_nu_mu1(const orc_nu *nu, double a, double k);
double orc_nu_mu2(const orc_nu *nu);
double orc_nu_pofk_cb(const orc_nu *nu, double k, double omega_cdm);
void orc_nu_add_density(const orc_nu *nu, double a, int N, double box, double *grid, const double *cdelta);

/* ----------------------------------------------------------- cosmology */
struct orc_power_s;
typedef struct orc_cosmo orc_cosmo;
/* Growth ODEs (src/cosmo.c:206-643) on a fine fixed-step RK4 grid. */
orc_cosmo *orc_cosmo_create(const orc_mg *m, double init_redshift);
void orc_cosmo_free(orc_cosmo *c);
double orc_growth_D(orc_cosmo *c, double a);
double orc_growth_dDdy(orc_cosmo *c, double a);
double orc_growth_ddDddy(orc_cosmo *c, double a);
double orc_growth_D2(orc_cosmo *c, double a);
double orc_growth_dD2dy(orc_cosmo *c, double a);
double orc_growth_ddD2ddy(orc_cosmo *c, double a);
double orc_growth_DLCDM(orc_cosmo *c, double a);
/* Scale-dependent build: the growth ODEs per k on the reference's k grid
 * (needs Box and Nmesh for that grid).  orc_cosmo_create is this with the
 * tables off. */
orc_cosmo *orc_cosmo_create_sd(const orc_mg *m, double init_redshift, double box, int nmesh);
/* growth_*_scaledependent (src/cosmo.c:987-1010): which 0 D, 1 dDdy,
 * 2 ddDddy, 3 D2, 4 dD2dy, 5 ddD2ddy; k in h/Mpc, normalised at a = 1 per k. */
double orc_growth_sd(orc_cosmo *c, int which, double k, double a);
/* mg_pofk_ratio (src/cosmo.c:688-706) and mg_sigma8_enhancement
 * (src/cosmo.c:713-756), both build variants. */
double orc_mg_pofk_ratio(orc_cosmo *c, double k, double a);
double orc_mg_sigma8_enh(orc_cosmo *c, const struct orc_power_s *pw, double a);

/* COLA coefficients (src/cosmo.c:1114-1160), nLPT = -2.5, fullT = 1. */
double orc_Sq(orc_cosmo *c, double ai, double af, double aref);
double orc_Sphi(orc_cosmo *c, double ai, double af, double aref);
/* non-COLA (UseCOLA = 0): SqStd, SphiStd (src/cosmo.c:1165-1200) */
double orc_SqStd(orc_cosmo *c, double ai, double af);
double orc_SphiStd(orc_cosmo *c, double ai, double af);
/* LCDM fitting functions (src/cosmo.c:1291-1398) -- known-answer checks. */
double orc_growthD_fit(double omega, double a);

/* Linear power spectrum (src/power.c:373-498). */
typedef struct orc_power_s {
  int which_spectrum;       /* 0 transfer-function, 1 tabulated, else EH */
  double omega, omega_b, h, ns, sigma8;
  int ntab; const double *tab_logk, *tab_logP;   /* log10 table for type 1 */
  double norm;              /* filled by orc_power_init */
  /* MASSIVE_NEUTRINOS build: the CDM+baryon spectrum of the CAMB tables,
   * with the OmegaCDM it is evaluated at (orc_power_init sets it) */
  const struct orc_nu_s *nu;
  double nu_ocdm;
} orc_power;
void orc_power_init(orc_power *p);
double orc_power_spec(const orc_power *p, double k);
double orc_tophat_sigma2(const orc_power *p, double R);
double orc_transfer_eh(const orc_power *p, double k);

/* ------------------------------------------------------------------ IC */
typedef struct {
  int N, Ns; double box; uint32_t seed; int sphere_mode;
  int fixed_amplitude, inverted;
  double pofk_rescale;      /* mg_pofk_ratio * sigma8 factor, scale-independent */
} orc_ic_params;
/* Seed table exactly in the order of src/2LPT.c:262-271. */
void orc_seedtable(int N, uint32_t seed, uint32_t *table);
/* displacement_fields() Gaussian + 2LPT (src/2LPT.c:185-495,1209-1519):
 * writes ZA (D1) and 2LPT (D2, already times -3/7) displacements per
 * particle [Ns^3][3], means removed.  Also returns delta(k) and the 2LPT
 * source(k) (cdelta_cdm / cdelta_cdm2 of the SCALEDEPENDENT build) if the
 * pointers are non-NULL. */
void orc_ic_2lpt(const orc_ic_params *ip, const orc_power *pw, double *D1, double *D2,
                 double *deltak_out, double *source2k_out);
/* The same from particles read from files (ReadParticlesFromFile,
 * src/readICfromfile.c:133-777): pos01 [n][3] in [0,1), normfac =
 * D_LCDM(1)/D_LCDM(a_i)/N^3, rescale_rk[|d|^2] the P(k) rescaling per integer
 * |k|^2 (sqrt(mg_pofk_ratio(k, 1)) / sigma8 enhancement as applicable). */
void orc_ic_2lpt_from_particles(const orc_ic_params *ip, const double *pos01, long n, double normfac,
                                const double *rescale_rk, double *D1, double *D2, double *deltak_out,
                                double *source2k_out);

/* Scale-dependent displacement fields (SCALEDEPENDENT build).  Field types
 * as src/proto.h:153-158. */
enum { ORC_FIELD_D = 0, ORC_FIELD_dDdy = 1, ORC_FIELD_ddDddy = 2, ORC_FIELD_deltaD = 3 };
/* from_cdisp_store_to_ZA (src/2LPT.c:1539-1735) for one LPT order (1 or 2):
 * disp(k) = i k/k^2 stored(k) G(k), three c2r, trilinear read-out at the
 * Lagrangian lattice, mean removed.  stored is delta(k) for order 1 and
 * -source(k) for order 2 (orc_ic_2lpt outputs).  out [Ns^3][3]. */
void orc_sd_field(orc_cosmo *c, const double *stored, int N, int Ns, double box, double A, double AFF,
                  int fieldtype, int order, double *out);

/* --------------------------------------------------------- full run */
typedef struct {
  orc_mg mg; orc_power pw; orc_ic_params ic;
  double init_redshift;
  int nsteps; double final_redshift;       /* one output at the end */
  int pofk_nbins, pofk_bintype, pofk_subtract_shotnoise;
  double pofk_kmin, pofk_kmax;
  int usecola;
  /* ReadParticlesFromFile: the IC from these particles (positions in [0,1),
   * [n][3]) and the P(k) rescaling per integer |k|^2, instead of the
   * Gaussian field; NULL for the Gaussian IC */
  const double *ic_pos01;
  long ic_n;
  const double *ic_rescale_rk;
  /* > 0: stop at the start of step stop_step of the schedule, after its
   * density and P(k); pos/vel out are then the particles there (vel = the
   * COLA velocity minus its mean, without the LPT part) */
  int stop_step;
} orc_run_params;
/* Runs IC + the KDK loop of src/main.c:394-611 for one output redshift.
 * pos/vel out [Ns^3][3] at the final time (vel incl. LPT part as written by
 * Output, main.c:959-967, in code units before velfac*fac); pk arrays sized
 * pofk_nbins.  Returns number of P(k) bins. */
int orc_run(const orc_run_params *rp, double *pos_out, double *vel_out,
            double *kbin, double *pk, double *kmean, double *nmodes);

/* CPU baseline timing: seconds per KDK step after an untimed IC. */
double orc_time_steps(const orc_run_params *rp, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
