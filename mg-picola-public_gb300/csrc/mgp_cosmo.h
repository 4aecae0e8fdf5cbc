/*
 * Host FP64 cosmology of the GB300 library: model hooks, growth factors,
 * COLA time-step coefficients and the linear power spectrum.  Everything here
 * runs on the host in double precision; kernels receive per-step scalars.
 */
#ifndef MGP_COSMO_H
#define MGP_COSMO_H
#include "mgpicola.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;
  double *x, *y, *y2;
} mgp_spline;

/* bicubic table over (x, y), z[j * nx + i], with node derivatives */
typedef struct {
  int nx, ny;
  double *x, *y, *z, *zx, *zy, *zxy;
} mgp_bicubic;

typedef struct mgp_cosmo {
  mgp_params p;
  /* user model hooks (NULL members: the built-in model) */
  mgp_model_hooks hooks;
  /* growth splines over x = ln a (src/cosmo.c:54-95) */
  mgp_spline D, dDdy, ddDddy, D2, dD2dy, ddD2ddy;
  mgp_spline DL, dDLdy, ddDLddy, D2L, dD2Ldy, ddD2Lddy;
  /* Brans-Dicke background (src/jbd.c): H(a)/H0, dH/da, Geff/G over ln a */
  int have_jbd;
  mgp_spline jbdH, jbddH, jbdG;
  /* m(a), beta(a) models: phi_crit(a) over ln a (src/cosmo.c:104-190) */
  int have_phia;
  mgp_spline phia;
  /* scale-dependent growth (src/cosmo.c:798-1010): D, dDdy, ddDddy, D2,
   * dD2dy, ddD2ddy over (ln a, ln k) */
  int sd;
  mgp_bicubic sd_tab[6];
  /* massive neutrinos (MASSIVE_NEUTRINOS build): Omega_nu, Omega_cdm
   * (user_defined_functions.h:59-66); CAMB transfer functions over
   * (ln k, z) for nu, cdm, baryon, total (read_CAMB_data.h:41-170); the
   * LCDM growth D(k, a) with the neutrino factor (cosmo.c:829-884) */
  int nu;          /* neutrino density added to delta(k) every step */
  int nu_growth;   /* neutrino factors in the growth equations */
  double OmegaNu, OmegaCDM;
  mgp_bicubic nuT[4];
  double *nu_rows0;   /* the four transfer functions at z = 0 as rows over ln k */
  mgp_bicubic sd_lcdm;
  /* power spectrum */
  double norm;
  int ntab;
  double *tab_logk, *tab_logv; /* log10 k and log10 P (or T) */
} mgp_cosmo;

int mgp_cosmo_init(mgp_cosmo *c, const mgp_params *p, char *err, size_t errlen);
/* the same with user model hooks (NULL = none) */
int mgp_cosmo_init_hooks(mgp_cosmo *c, const mgp_params *p, const mgp_model_hooks *hooks, char *err, size_t errlen);
/* the user's screening functions, when given (else NULL) */
int mgp_cosmo_user_screening(const mgp_cosmo *c, int density);
/* Massive-neutrino density factors per integer |k|^2 = rk of an N^3 mesh
 * (src/auxPM.c:383-421), OmegaNu/Omega N^3 T_nu(k, a) / T_cb(k, 1):
 * mgp_cosmo_nu_den fills den[rk] = T_cb(k, 1), the step-independent
 * denominators; mgp_cosmo_nu_row gives the massive-nu transfer function at
 * z = 1/a - 1 as value and d/d ln k on the table's ln k nodes
 * (mgp_cosmo_nu_lnk; clamped lookups use the cubic Hermite between nodes)
 * and returns the node count. */
void mgp_cosmo_nu_den(const mgp_cosmo *c, int N, int nrk, double *den);
int mgp_cosmo_nu_row(const mgp_cosmo *c, double a, double *val, double *dval);
const double *mgp_cosmo_nu_lnk(const mgp_cosmo *c, int *nx);
void mgp_cosmo_free(mgp_cosmo *c);

/* hooks, src/user_defined_functions.h:413-904 */
double mgp_hubble(const mgp_cosmo *c, double a);
double mgp_dhubbleda(const mgp_cosmo *c, double a);
double mgp_beta_dgp(const mgp_cosmo *c, double a);
double mgp_beta_of_a(const mgp_cosmo *c, double a);
double mgp_mass2_of_a(const mgp_cosmo *c, double a);
double mgp_coupling(const mgp_cosmo *c, double a);
double mgp_geff(const mgp_cosmo *c, double a, double k);
double mgp_factor_2lpt(const mgp_cosmo *c, double a);
/* phi_crit(a) of screening_factor_potential (user_defined_functions.h:725-750) */
double mgp_phicrit(const mgp_cosmo *c, double a);
/* prefactor C(a) with fac = C(a)(1+delta) in screening_factor_density
 * (user_defined_functions.h:757-773) */
double mgp_dgp_screen_prefactor(const mgp_cosmo *c, double a);

/* growth lookups (src/cosmo.c:318-403), normalised at a = 1 */
double mgp_cosmo_growth(const mgp_cosmo *c, int which, double a);
double mgp_cosmo_Sq(const mgp_cosmo *c, double ai, double af, double aref);
double mgp_cosmo_Sphi(const mgp_cosmo *c, double ai, double af, double aref);
double mgp_cosmo_SqStd(const mgp_cosmo *c, double ai, double af);
double mgp_cosmo_SphiStd(const mgp_cosmo *c, double ai, double af);
double mgp_cosmo_step_da(const mgp_params *p, double A, double aout, int nsteps);
double mgp_cosmo_step_mid(const mgp_params *p, double A, double da);
double mgp_cosmo_step_end(const mgp_params *p, double A, double da);
double mgp_cosmo_kick_dda(const mgp_cosmo *c, double ai, double af, double a);
double mgp_cosmo_drift_dyyy(const mgp_cosmo *c, double a, double aff, double af);

/* PowerSpec (src/power.c:373-394) in (Mpc/h)^3, k in h/Mpc */
double mgp_cosmo_power(const mgp_cosmo *c, double k);
/* mg_pofk_ratio(k, a) and mg_sigma8_enhancement(a) (src/cosmo.c:688-756) */
double mgp_cosmo_pofk_ratio(const mgp_cosmo *c, double k, double a);
void mgp_cosmo_pofk_ratio_many(const mgp_cosmo *c, double a, int n, const double *k, double *out);
double mgp_cosmo_sigma8_enh(const mgp_cosmo *c, double a);
/* Scale-dependent growth: growth_*_scaledependent (src/cosmo.c:987-1010),
 * which 0-5 = D, dDdy, ddDddy, D2, dD2dy, ddD2ddy, k in h/Mpc; and the
 * table restricted to x = ln a (clamped): value and d/d ln k at the ln k
 * nodes sd_tab[which].y. */
double mgp_cosmo_growth_sd(const mgp_cosmo *c, int which, double k, double a);
int mgp_cosmo_sd_column(const mgp_cosmo *c, int which, double a, double *val, double *dval);
double mgp_dmass2_of_ada(const mgp_cosmo *c, double a);

#ifdef __cplusplus
}
#endif
#endif
