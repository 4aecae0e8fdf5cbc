/*
 * Oracle cosmology (test infrastructure only): model hooks of
 * src/user_defined_functions.h, growth ODEs of src/cosmo.c, COLA time-step
 * coefficients and the linear power spectrum of src/power.c, all FP64.
 *
 * Third-party numerics the reference takes from GSL are replaced here by
 * textbook methods: the growth ODE (GSL odeiv2 rk2, eps 1e-7, cosmo.c:460-463)
 * is integrated with a fixed-step classical RK4 at 64 sub-steps per knot;
 * quadratures (GSL qag) use adaptive 20-point Gauss-Legendre bisection to a
 * 1e-12 relative tolerance; splines are natural cubic (GSL cspline).
 */
#include "orc.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define INVERSE_H0_MPCH 2997.92458 /* src/vars.h:65 */

/* ---------------------------------------------------- JBD / phi(a) state */
typedef struct { int n; double *x, *y, *y2; } spl;
static void spl_init(spl *s, const double *x, const double *y, int n);
static double spl_eval(const spl *s, double x);
static int g_jbd = 0, g_phia = 0;
static spl g_jbdH, g_jbddH, g_jbdG, g_phia_s;

/* ---------------------------------------------------------------- hooks */
/* hubble: user_defined_functions.h:413-429 */
double orc_hubble(const orc_mg *m, double a) {
  if (m->model == ORC_JBD_GEFF && g_jbd) return spl_eval(&g_jbdH, log(a));
  if (m->use_w0wa)
    return sqrt(m->omega / (a * a * a) + (1.0 - m->omega) * exp(3.0 * m->wa * (a - 1) - 3 * (1 + m->w0 + m->wa) * log(a)));
  return sqrt(m->omega / (a * a * a) + 1.0 - m->omega);
}
/* dhubbleda: user_defined_functions.h:431-447 */
double orc_dhubbleda(const orc_mg *m, double a) {
  if (m->model == ORC_JBD_GEFF && g_jbd) return spl_eval(&g_jbddH, log(a));
  if (m->use_w0wa)
    return 1.0 / (2.0 * orc_hubble(m, a)) *
           (-3.0 * m->omega / (a * a * a * a) - 3.0 * (1.0 - m->omega) * (1.0 + m->w0 + m->wa * (1 - a)) / a);
  return 1.0 / (2.0 * orc_hubble(m, a)) * (-3.0 * m->omega / (a * a * a * a));
}
/* beta_DGP: user_defined_functions.h:453-455 */
double orc_beta_dgp(const orc_mg *m, double a) {
  return 1.0 + 2.0 * m->rcH0 * (orc_hubble(m, a) + a * orc_dhubbleda(m, a) / 3.0);
}
/* beta_of_a: user_defined_functions.h:462-484 */
double orc_beta_of_a(const orc_mg *m, double a) {
  if (m->model == ORC_FOFR) return 1.0 / sqrt(6.0);
  if (m->model == ORC_MBETA) {
    if (a > m->assb_symm) return m->beta_symm * sqrt(1.0 - pow(m->assb_symm / a, 3));
    return 0.0;
  }
  return 0.0;
}
/* mass2_of_a: user_defined_functions.h:490-522 */
double orc_mass2_of_a(const orc_mg *m, double a) {
  if (m->model == ORC_FOFR) {
    double a3 = a * a * a;
    double fac = m->omega / a3 + 4.0 * (1.0 - m->omega);
    double fac0 = m->omega + 4.0 * (1.0 - m->omega);
    return fac0 * pow(fac / fac0, m->nfofr + 2.0) / ((1.0 + m->nfofr) * m->fofr0);
  }
  if (m->model == ORC_MBETA) {
    if (a > m->assb_symm) return 0.5 * pow(2998.0 / m->range_symm, 2) * (1.0 - pow(m->assb_symm / a, 3));
    return 1.0;
  }
  return 0.0;
}
/* coupling_function: user_defined_functions.h:587-611 */
double orc_coupling(const orc_mg *m, double a) {
  if (m->model == ORC_FOFR || m->model == ORC_MBETA) return 2.0 * orc_beta_of_a(m, a) * orc_beta_of_a(m, a);
  if (m->model == ORC_DGP) return 1.0 / (3.0 * orc_beta_dgp(m, a));
  if (m->model == ORC_JBD_GEFF) return g_jbd ? spl_eval(&g_jbdG, log(a)) - 1.0 : m->geff_const - 1.0;
  return 0.0;
}
/* GeffoverG: user_defined_functions.h:618-652 */
double orc_geff(const orc_mg *m, double a, double k) {
  double mu = 1.0;
  if (!m->mg_active) return mu;
  if (m->use_lcdm_growth) return mu;
  if (m->model == ORC_FOFR || m->model == ORC_MBETA) {
    double mass2a2 = a * a * orc_mass2_of_a(m, a);
    double k2 = pow(k * INVERSE_H0_MPCH, 2);
    if (k2 == 0) return mu;
    mu *= 1.0 + 2.0 * orc_beta_of_a(m, a) * orc_beta_of_a(m, a) * k2 / (k2 + mass2a2);
    return mu;
  }
  if (m->model == ORC_DGP) return mu * (1.0 + 1.0 / (3.0 * orc_beta_dgp(m, a)));
  if (m->model == ORC_JBD_GEFF) return mu * (1.0 + orc_coupling(m, a));
  return mu;
}
/* Factor_2LPT: user_defined_functions.h:814-838 */
double orc_factor_2lpt(const orc_mg *m, double a) {
  if (!m->mg_active || m->use_lcdm_growth) return 1.0;
  if (m->model == ORC_DGP) {
    double b = orc_beta_dgp(m, a);
    return 1.0 - (2.0 * m->rcH0 * m->rcH0 * m->omega) / (9.0 * a * a * a * pow(b, 3) * (1 + 1.0 / (3.0 * b)));
  }
  return 1.0;
}
/* dmass2_of_ada: user_defined_functions.h:527-560 (dm^2/da / H0^2) */
double orc_dmass2_of_ada(const orc_mg *m, double a) {
  if (m->model == ORC_FOFR) {
    double a3 = a * a * a;
    double fac = m->omega / a3 + 4.0 * (1.0 - m->omega);
    double fac0 = m->omega + 4.0 * (1.0 - m->omega);
    double mass2 = fac0 * (m->nfofr + 2.0) * pow(fac / fac0, m->nfofr + 1.0) / ((1.0 + m->nfofr) * m->fofr0 * fac0);
    return mass2 * (-3.0 * m->omega / a3 / a);
  }
  if (m->model == ORC_MBETA) {
    if (a > m->assb_symm) return 0.5 * pow(2998.0 / m->range_symm, 2) * (3.0 * pow(m->assb_symm / a, 3) / a);
    return 0.0;
  }
  return 0.0;
}
/* fofr_pi_factor: user_defined_functions.h:848-854 */
static double fofr_pi(const orc_mg *m, double k, double a) {
  double a3 = a * a * a;
  double fac = m->omega / a3 + 4.0 * (1.0 - m->omega);
  double fac0 = m->omega + 4.0 * (1.0 - m->omega);
  return pow(k * INVERSE_H0_MPCH / a, 2) + fac0 * pow(fac / fac0, m->nfofr + 2.0) / (1.0 + m->nfofr) / m->fofr0;
}
/* second_order_kernel: user_defined_functions.h:862-904 */
double orc_second_order_kernel(const orc_mg *m, double k, double k1, double k2, double cost, double a) {
  if (!m->mg_active || m->use_lcdm_growth) return 0.0;
  double g = 0.0, H = orc_hubble(m, a), a3 = a * a * a;
  if (m->model == ORC_FOFR) {
    double fac = m->omega / a3 + 4.0 * (1.0 - m->omega);
    double fac0 = m->omega + 4.0 * (1.0 - m->omega);
    double n = m->nfofr;
    g = -(3.0 * (n + 2.0) / (12.0 * (1.0 + n) * (1.0 + n))) * pow(k * INVERSE_H0_MPCH / (a * H), 2) *
        pow(m->omega / a3, 2) * fac0 * pow(fac / fac0, 2.0 * n + 3.0) / pow(m->fofr0, 2);
    g /= fofr_pi(m, k, a) * fofr_pi(m, k1, a) * fofr_pi(m, k2, a);
  } else if (m->model == ORC_DGP) {
    g = -1.0 / 6.0 / pow(orc_beta_dgp(m, a), 3) * pow(m->rcH0 / H, 2) * pow(m->omega / a3, 2) * (1.0 - cost * cost);
  } else if (m->model == ORC_MBETA) {
    double m2 = orc_mass2_of_a(m, a), dm2da = orc_dmass2_of_ada(m, a);
    double pk = pow(k * INVERSE_H0_MPCH / a, 2) + m2;
    double pk1 = pow(k1 * INVERSE_H0_MPCH / a, 2) + m2;
    double pk2 = pow(k2 * INVERSE_H0_MPCH / a, 2) + m2;
    double b = orc_beta_of_a(m, a);
    g = (dm2da / m2) * b * b * m->omega / (2.0 * a * a) * (m2 / pk1) * (m2 / pk2) * (1.0 - m2 / pk) / (H * H);
  }
  if (k2 > 1e-3 && k1 > 1e-3) {
    double mk = orc_geff(m, a, k);
    g += 1.5 * m->omega / (a3 * H * H) *
         ((mk - orc_geff(m, a, k1)) * (k1 / k2) + (mk - orc_geff(m, a, k2)) * (k2 / k1)) * cost / 2.0;
  }
  return g;
}
/* screening_factor_potential: user_defined_functions.h:725-750 (f(R)) */
double orc_screen_potential(const orc_mg *m, double a, double phinewton) {
  if (!m->include_screening) return 1.0;
  if (phinewton >= 0.0) return 1.0;
  if (m->model == ORC_FOFR) {
    double phicrit = 1.5 * m->fofr0 *
                     pow((m->omega + 4.0 * (1.0 - m->omega)) / (1.0 / (a * a * a) * m->omega + 4.0 * (1.0 - m->omega)), m->nfofr + 1.0);
    double s = fabs(phicrit / phinewton);
    return s > 1.0 ? 1.0 : s;
  }
  if (m->model == ORC_MBETA) {
    double s = fabs(orc_phicrit(m, a) / phinewton);
    return s > 1.0 ? 1.0 : s;
  }
  return 1.0;
}
/* screening_factor_density: user_defined_functions.h:757-773 (nDGP) */
double orc_screen_density(const orc_mg *m, double a, double density) {
  if (!m->include_screening) return 1.0;
  if (m->model == ORC_DGP) {
    double fac = 8.0 / 9.0 * m->omega * pow(m->rcH0 / orc_beta_dgp(m, a), 2) * (1.0 + density);
    if (fac < 1e-5) return 1.0;
    return 2.0 * (sqrt(1.0 + fac) - 1.0) / fac;
  }
  return 1.0;
}

/* ------------------------------------------------------------- splines */
typedef struct { int n; double *x, *y, *y2; } spline1;

static void spline_init(spline1 *s, const double *x, const double *y, int n) {
  s->n = n;
  s->x = malloc(8 * n); s->y = malloc(8 * n); s->y2 = calloc(n, 8);
  memcpy(s->x, x, 8 * n); memcpy(s->y, y, 8 * n);
  double *u = calloc(n, 8);
  /* natural cubic spline, tridiagonal solve */
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * s->y2[i - 1] + 2.0;
    s->y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  s->y2[n - 1] = 0.0;
  for (int k = n - 2; k >= 0; k--) s->y2[k] = s->y2[k] * s->y2[k + 1] + u[k];
  free(u);
}

/* Clamped lookup as Lookup_GSL_Spline (src/wrappers.c:162-167). */
static double spline_eval(const spline1 *s, double x) {
  if (x < s->x[0]) x = s->x[0];
  if (x > s->x[s->n - 1]) x = s->x[s->n - 1];
  int lo = 0, hi = s->n - 1;
  while (hi - lo > 1) { int mid = (hi + lo) / 2; if (s->x[mid] > x) hi = mid; else lo = mid; }
  double h = s->x[hi] - s->x[lo];
  double A = (s->x[hi] - x) / h, B = (x - s->x[lo]) / h;
  return A * s->y[lo] + B * s->y[hi] + ((A * A * A - A) * s->y2[lo] + (B * B * B - B) * s->y2[hi]) * (h * h) / 6.0;
}
static void spline_free(spline1 *s) { free(s->x); free(s->y); free(s->y2); }

/* ---------------------------------------------------------- quadrature */
static const double GL20_X[10] = {0.0765265211334973, 0.2277858511416451, 0.3737060887154195,
                                  0.5108670019508271, 0.6360536807265150, 0.7463319064601508,
                                  0.8391169718222188, 0.9122344282513259, 0.9639719272779138,
                                  0.9931285991850949};
static const double GL20_W[10] = {0.1527533871307258, 0.1491729864726037, 0.1420961093183820,
                                  0.1316886384491766, 0.1181945319615184, 0.1019301198172404,
                                  0.0832767415767048, 0.0626720483341091, 0.0406014298003869,
                                  0.0176140071391521};
/* Nodes above are printed to 16 digits; refine them by Newton on P_20. */
static double glx[10], glw[10];
static int gl_ready = 0;
static void gl_init(void) {
  if (gl_ready) return;
  for (int i = 0; i < 10; i++) {
    double x = GL20_X[i], dp = 0;
    for (int it = 0; it < 8; it++) {
      double p0 = 1.0, p1 = x;
      for (int n = 2; n <= 20; n++) { double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n; p0 = p1; p1 = p2; }
      dp = 20 * (x * p1 - p0) / (x * x - 1.0);
      x -= p1 / dp;
    }
    glx[i] = x;
    glw[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  (void)GL20_W;
  gl_ready = 1;
}
typedef double (*fn1)(double, void *);
static double gl20(fn1 f, void *par, double a, double b) {
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0;
  for (int i = 0; i < 10; i++) s += glw[i] * (f(c - h * glx[i], par) + f(c + h * glx[i], par));
  return s * h;
}
static double adapt(fn1 f, void *par, double a, double b, double whole, double abstol, int depth) {
  double c = 0.5 * (a + b);
  double l = gl20(f, par, a, c), r = gl20(f, par, c, b);
  if (depth >= 16 || fabs(l + r - whole) <= abstol) return l + r;
  return adapt(f, par, a, c, l, 0.5 * abstol, depth + 1) + adapt(f, par, c, b, r, 0.5 * abstol, depth + 1);
}
static double integrate(fn1 f, void *par, double a, double b) {
  gl_init();
  /* 8 starting panels so oscillatory integrands are resolved; the absolute
   * tolerance is 1e-13 of the first estimate of the whole integral */
  double est[8], tot = 0;
  for (int i = 0; i < 8; i++) {
    est[i] = gl20(f, par, a + (b - a) * i / 8.0, a + (b - a) * (i + 1) / 8.0);
    tot += fabs(est[i]);
  }
  double s = 0, tol = 1e-13 * tot / 8.0 + 1e-300;
  for (int i = 0; i < 8; i++)
    s += adapt(f, par, a + (b - a) * i / 8.0, a + (b - a) * (i + 1) / 8.0, est[i], tol, 0);
  return s;
}

/* --------------------------------------------------------- growth ODEs */
struct orc_cosmo {
  orc_mg m;
  spline1 D, dDdy, ddDddy, D2, dD2dy, ddD2ddy, DLCDM;
  /* SCALEDEPENDENT: D, dDdy, ddDddy, D2, dD2dy, ddD2ddy over (ln a, ln k) */
  int sd;
  orc_bicubic tab[6];
  /* massive neutrinos: the LCDM D(k, a) of the same build (cosmo.c:829-884) */
  int sd_lcdm;
  orc_bicubic tab_lcdm;
};

/* ode_growth_D (cosmo.c:206-239); lcdm = 1 gives ode_growth_DLCDM
 * (cosmo.c:245-268).  modfac is Factor_2LPT(a) in the scale-independent
 * build and 1 + 2 (a^2 H)^2 gamma_2(k, k/sqrt2, k/sqrt2, 0, a) / (1.5 Omega a
 * mu) in the SCALEDEPENDENT build (cosmo.c:215-223).  The 1D tables use
 * k = 1e-3 h/Mpc (solve_for_growth_factors, cosmo.c:456). */
static void growth_rhs(const orc_mg *m, int lcdm, double k, double x, const double *D, double *dD) {
  double a = exp(x);
  double mu = lcdm ? 1.0 : orc_geff(m, a, k);
  double H = orc_hubble(m, a), dH = orc_dhubbleda(m, a);
  double betafac = 1.5 * m->omega * mu / (a * a * a * H * H);
  double alphafac = 2.0 + a * dH / H;
  double modfac = 1.0;
  if (!lcdm) {
    if (m->scaledependent)
      modfac = 1.0 + 2.0 * pow(a * a * H, 2) * orc_second_order_kernel(m, k, k / sqrt(2.0), k / sqrt(2.0), 0.0, a) /
                         (1.5 * m->omega * a * mu);
    else
      modfac = orc_factor_2lpt(m, a);
  }
  /* massive neutrinos (cosmo.c:224-236, 253-265): mu_nu multiplies the
   * source terms */
  double mu1 = orc_nu_mu1(m->nu, a, k), mu2 = orc_nu_mu2(m->nu);
  dD[0] = D[1];
  dD[1] = -alphafac * D[1] + betafac * mu1 * D[0];
  dD[2] = D[3];
  dD[3] = -alphafac * D[3] + betafac * mu2 * (D[2] - modfac * D[0] * D[0]);
}

static void rk4(const orc_mg *m, int lcdm, double k, double x0, double x1, int nsub, double *y) {
  double h = (x1 - x0) / nsub;
  for (int s = 0; s < nsub; s++) {
    double x = x0 + s * h, k1[4], k2[4], k3[4], k4[4], t[4];
    growth_rhs(m, lcdm, k, x, y, k1);
    for (int i = 0; i < 4; i++) t[i] = y[i] + 0.5 * h * k1[i];
    growth_rhs(m, lcdm, k, x + 0.5 * h, t, k2);
    for (int i = 0; i < 4; i++) t[i] = y[i] + 0.5 * h * k2[i];
    growth_rhs(m, lcdm, k, x + 0.5 * h, t, k3);
    for (int i = 0; i < 4; i++) t[i] = y[i] + h * k3[i];
    growth_rhs(m, lcdm, k, x + h, t, k4);
    for (int i = 0; i < 4; i++) y[i] += h / 6.0 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
  }
}

static double Qfactor(const orc_mg *m, double a) { return orc_hubble(m, a) * a * a * a; }

/* calculate_scale_dependent_growth_factor (cosmo.c:798-981): the growth
 * ODEs for each of nk log-spaced k, stored as 2D tables over (ln a, ln k). */
static void solve_sd(orc_cosmo *c, double xini, double xend, int npts, double box, int nmesh) {
  const orc_mg *m = &c->m;
  int nk = m->sd_nk > 0 ? m->sd_nk : 1000;
  double kmin = m->sd_kmin > 0 ? m->sd_kmin : 2.0 * M_PI / box * 0.5;
  double kmax = m->sd_kmax > 0 ? m->sd_kmax : 2.0 * M_PI / box * nmesh * sqrt(3.0) * 2.0;
  double *logk = malloc(8 * nk), *x = malloc(8 * npts);
  double *T[6];
  for (int f = 0; f < 6; f++) T[f] = malloc(sizeof(double) * npts * nk);
  for (int i = 0; i < nk; i++) logk[i] = log(kmin) + log(kmax / kmin) * i / (double)(nk - 1);
  for (int i = 0; i < npts; i++) x[i] = xini + (xend - xini) * i / (double)(npts - 1);
#pragma omp parallel for schedule(dynamic)
  for (int ik = 0; ik < nk; ik++) {
    double know = exp(log(kmin) + log(kmax / kmin) * ik / (double)(nk - 1));
    double y[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0};
    for (int i = 0; i < npts; i++) {
      if (i > 0) rk4(m, 0, know, x[i - 1], x[i], 16, y);
      double anow = exp(x[i]), mu = orc_geff(m, anow, know);
      size_t c0 = (size_t)ik * npts + i;
      T[0][c0] = y[0];
      T[1][c0] = y[1] * Qfactor(m, anow) / anow;
      const double mu1 = orc_nu_mu1(m->nu, anow, know), mu2 = orc_nu_mu2(m->nu);
      T[2][c0] = 1.5 * mu * mu1 * m->omega * anow * y[0];
      T[3][c0] = y[2];
      T[4][c0] = y[3] * Qfactor(m, anow) / anow;
      T[5][c0] = 1.5 * mu * mu2 * m->omega * anow * (y[2] - y[0] * y[0]);
    }
  }
  if (m->nu) {
    /* the LCDM growth per k with the neutrino factors (gravity switched off:
     * mu = 1 and no second-order kernel); only D is looked up later */
    double *L = malloc(sizeof(double) * npts * nk);
#pragma omp parallel for schedule(dynamic)
    for (int ik = 0; ik < nk; ik++) {
      double know = exp(log(kmin) + log(kmax / kmin) * ik / (double)(nk - 1));
      double y[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0};
      for (int i = 0; i < npts; i++) {
        if (i > 0) rk4(m, 1, know, x[i - 1], x[i], 16, y);
        L[(size_t)ik * npts + i] = y[0];
      }
    }
    orc_bicubic_init(&c->tab_lcdm, x, logk, L, npts, nk);
    free(L);
    c->sd_lcdm = 1;
  }
  for (int f = 0; f < 6; f++) {
    orc_bicubic_init(&c->tab[f], x, logk, T[f], npts, nk);
    free(T[f]);
  }
  free(logk);
  free(x);
  c->sd = 1;
}

/* Lookup_GSL_2D_Spline (src/wrappers.c:129-136): clamp, then evaluate */
static double lookup2d(const orc_bicubic *b, double x, double y) {
  if (x < b->x[0]) x = b->x[0];
  if (x > b->x[b->nx - 1]) x = b->x[b->nx - 1];
  if (y < b->y[0]) y = b->y[0];
  if (y > b->y[b->ny - 1]) y = b->y[b->ny - 1];
  return orc_bicubic_eval(b, x, y);
}

orc_cosmo *orc_cosmo_create(const orc_mg *m, double init_redshift) {
  return orc_cosmo_create_sd(m, init_redshift, 0.0, 0);
}

/* solve_for_growth_factors (cosmo.c:409-643) */
orc_cosmo *orc_cosmo_create_sd(const orc_mg *m, double init_redshift, double box, int nmesh) {
  orc_cosmo *c = calloc(1, sizeof(orc_cosmo));
  c->m = *m;
  const int npts = 1000;
  double zini = init_redshift > 200.0 ? init_redshift : 200.0, zend = -0.5;
  double aini = 1.0 / (1.0 + zini), xini = log(aini), xend = log(1.0 / (1.0 + zend));
  double dx = (xend - xini) / (double)(npts - 1);
  double *x = malloc(8 * npts), *D = malloc(8 * npts), *dD = malloc(8 * npts), *ddD = malloc(8 * npts);
  double *D2 = malloc(8 * npts), *dD2 = malloc(8 * npts), *ddD2 = malloc(8 * npts), *DL = malloc(8 * npts);
  double y[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0}, yl[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0};
  for (int i = 0; i < npts; i++) {
    double xnow = xini + i * dx;
    if (i > 0) {
      rk4(m, 0, 1e-3, xini + (i - 1) * dx, xnow, 64, y);
      rk4(m, 1, 1e-3, xini + (i - 1) * dx, xnow, 64, yl);
    }
    double anow = exp(xnow), mu = orc_geff(m, anow, 1e-3);
    x[i] = xnow;
    D[i] = y[0];
    dD[i] = y[1] * Qfactor(m, anow) / anow;
    ddD[i] = 1.5 * mu * m->omega * anow * y[0];
    D2[i] = y[2];
    dD2[i] = y[3] * Qfactor(m, anow) / anow;
    ddD2[i] = 1.5 * mu * m->omega * anow * (y[2] - y[0] * y[0] * orc_factor_2lpt(m, anow));
    DL[i] = yl[0];
  }
  spline_init(&c->D, x, D, npts); spline_init(&c->dDdy, x, dD, npts); spline_init(&c->ddDddy, x, ddD, npts);
  spline_init(&c->D2, x, D2, npts); spline_init(&c->dD2dy, x, dD2, npts); spline_init(&c->ddD2ddy, x, ddD2, npts);
  spline_init(&c->DLCDM, x, DL, npts);
  free(x); free(D); free(dD); free(ddD); free(D2); free(dD2); free(ddD2); free(DL);
  if (m->scaledependent && box > 0 && nmesh > 0) solve_sd(c, xini, xend, npts, box, nmesh);
  return c;
}
void orc_cosmo_free(orc_cosmo *c) {
  if (!c) return;
  spline_free(&c->D); spline_free(&c->dDdy); spline_free(&c->ddDddy);
  spline_free(&c->D2); spline_free(&c->dD2dy); spline_free(&c->ddD2ddy); spline_free(&c->DLCDM);
  if (c->sd)
    for (int f = 0; f < 6; f++) orc_bicubic_free(&c->tab[f]);
  if (c->sd_lcdm) orc_bicubic_free(&c->tab_lcdm);
  free(c);
}
/* growth_*_scaledependent (cosmo.c:987-1010) */
double orc_growth_sd(orc_cosmo *c, int which, double k, double a) {
  const orc_bicubic *norm = &c->tab[which < 3 ? 0 : 3];
  return lookup2d(&c->tab[which], log(a), log(k)) / lookup2d(norm, 0.0, log(k));
}
/* mg_pofk_ratio (cosmo.c:688-706), no massive neutrinos */
double orc_mg_pofk_ratio(orc_cosmo *c, double k, double a) {
  if (!c->m.mg_active) return 1.0;
  if (c->sd_lcdm) {  /* cosmo.c:692-695 */
    double q = lookup2d(&c->tab[0], log(a), log(k)) / lookup2d(&c->tab_lcdm, log(a), log(k));
    return q * q;
  }
  double r = c->sd ? lookup2d(&c->tab[0], log(a), log(k)) / spline_eval(&c->DLCDM, log(a))
                   : spline_eval(&c->D, log(a)) / spline_eval(&c->DLCDM, log(a));
  return r * r;
}
/* mg_sigma8_enhancement (cosmo.c:713-756) */
double orc_mg_sigma8_enh(orc_cosmo *c, const struct orc_power_s *pw, double a) {
  if (!c->m.mg_active) return 1.0;
  if (!c->sd) return spline_eval(&c->D, log(a)) / spline_eval(&c->DLCDM, log(a));
  const double kmin = 0.001, kmax = 100.0;
  const int npts = 1000;
  double s = 0.0, sl = 0.0, dlogk = log(kmax / kmin) / (double)(npts - 1);
  for (int i = 0; i < npts; i++) {
    double know = exp(log(kmin) + log(kmax / kmin) * i / (double)(npts - 1));
    double kR8 = know * 8.0;
    double w = 3.0 / (kR8 * kR8 * kR8) * (sin(kR8) - kR8 * cos(kR8));
    double D = lookup2d(&c->tab[0], log(a), log(know));
    double DL = c->sd_lcdm ? lookup2d(&c->tab_lcdm, log(a), log(know)) : spline_eval(&c->DLCDM, log(a));
    double power = orc_power_spec((const orc_power *)pw, know);
    s += power * w * w * D * D * know * know * know * dlogk / (2.0 * M_PI * M_PI);
    sl += power * w * w * DL * DL * know * know * know * dlogk / (2.0 * M_PI * M_PI);
  }
  return sqrt(s) / sqrt(sl);
}
/* growth_* lookups (cosmo.c:318-403), normalised at a = 1 */
double orc_growth_D(orc_cosmo *c, double a) { return spline_eval(&c->D, log(a)) / spline_eval(&c->D, 0.0); }
double orc_growth_dDdy(orc_cosmo *c, double a) { return spline_eval(&c->dDdy, log(a)) / spline_eval(&c->D, 0.0); }
double orc_growth_ddDddy(orc_cosmo *c, double a) { return spline_eval(&c->ddDddy, log(a)) / spline_eval(&c->D, 0.0); }
double orc_growth_D2(orc_cosmo *c, double a) { return spline_eval(&c->D2, log(a)) / spline_eval(&c->D2, 0.0); }
double orc_growth_dD2dy(orc_cosmo *c, double a) { return spline_eval(&c->dD2dy, log(a)) / spline_eval(&c->D2, 0.0); }
double orc_growth_ddD2ddy(orc_cosmo *c, double a) { return spline_eval(&c->ddD2ddy, log(a)) / spline_eval(&c->D2, 0.0); }
double orc_growth_DLCDM(orc_cosmo *c, double a) { return spline_eval(&c->DLCDM, log(a)) / spline_eval(&c->DLCDM, 0.0); }

/* COLA coefficients, cosmo.c:1114-1160 with nLPT = -2.5, fullT = 1
 * (main.c:82-85). */
static double gpQ(double a) { return pow(a, -2.5); }
static double DERgpQ(double a) { return -2.5 * pow(a, -3.5); }
static double sq_integrand(double a, void *p) { return gpQ(a) / Qfactor((const orc_mg *)p, a); }
double orc_Sq(orc_cosmo *c, double ai, double af, double aref) {
  return integrate(sq_integrand, &c->m, ai, af) / gpQ(aref);
}
double orc_Sphi(orc_cosmo *c, double ai, double af, double aref) {
  return (gpQ(af) - gpQ(ai)) * aref / Qfactor(&c->m, aref) / DERgpQ(aref);
}
/* SqStd / SphiStd (src/cosmo.c:1165-1200): the Quinn et al. coefficients of
 * the non-COLA run (StdDA = 2, main.c:75-81) */
static double sqstd_integrand(double a, void *m) { return 1.0 / Qfactor((const orc_mg *)m, a); }
static double sphistd_integrand(double a, void *m) { return a / Qfactor((const orc_mg *)m, a); }
double orc_SqStd(orc_cosmo *c, double ai, double af) { return integrate(sqstd_integrand, &c->m, ai, af); }
double orc_SphiStd(orc_cosmo *c, double ai, double af) { return integrate(sphistd_integrand, &c->m, ai, af); }

/* Gauss hypergeometric series 2F1(a,b;c;z), |z| < 1. */
static double hyp2f1(double a, double b, double c, double z) {
  double term = 1.0, sum = 1.0;
  for (int n = 0; n < 2000000; n++) {
    term *= (a + n) * (b + n) / ((c + n) * (n + 1.0)) * z;
    sum += term;
    if (fabs(term) < 1e-17 * fabs(sum)) break;
  }
  return sum;
}
/* growthDtemp, cosmo.c:1307-1356 (LCDM closed form). */
static double growthDtemp(double Omega, double a) {
  double hyperP = 0.0, hyperM = 0.0;
  double x = -Omega / (Omega - 1.0) / (a * a * a);
  if (fabs(x - 1.0) < 1.e-3) {
    double t = -1.0 + x;
    hyperP = 0.859596768064608 - 0.1016599912520404 * t + 0.025791094277821357 * pow(t, 2) -
             0.008194025861121475 * pow(t, 3) + 0.0029076305993447644 * pow(t, 4) -
             0.0011025426387159761 * pow(t, 5) + 0.00043707304964624546 * pow(t, 6) -
             0.0001788889964687831 * pow(t, 7);
    hyperM = 1.1765206505266006 + 0.15846194123099624 * t - 0.014200487494738975 * pow(t, 2) +
             0.002801728034399257 * pow(t, 3) - 0.0007268267888593511 * pow(t, 4) +
             0.00021801569226706922 * pow(t, 5) - 0.00007163321597397065 * pow(t, 6) +
             0.000025063737576245116 * pow(t, 7);
  } else {
    if (x < 1.0) {
      hyperP = hyp2f1(1.0 / 2.0, 2.0 / 3.0, 5.0 / 3.0, -x);
      hyperM = hyp2f1(-1.0 / 2.0, 2.0 / 3.0, 5.0 / 3.0, -x);
    }
    x = 1.0 / x;
    if ((x < 1.0) && (x > 1.0 / 30.0)) {
      hyperP = hyp2f1(-1.0 / 6.0, 0.5, 5.0 / 6.0, -x);
      hyperP *= 4 * sqrt(x);
      hyperP += -3.4494794123063873799 * pow(x, 2.0 / 3.0);
      hyperM = hyp2f1(-7.0 / 6.0, -0.5, -1.0 / 6.0, -x);
      hyperM *= 4.0 / 7.0 / sqrt(x);
      hyperM += pow(x, 2.0 / 3.0) * (-1.4783483195598803057);
    }
    if (x <= 1.0 / 30.0) {
      hyperP = 4.0 * sqrt(x) - 3.4494794123063865 * pow(x, 2.0 / 3.0) + 0.4 * pow(x, 1.5) -
               0.13636363636363635 * pow(x, 2.5) + 0.07352941176470587 * pow(x, 3.5) -
               0.04755434782608695 * pow(x, 4.5) + 0.033943965517241374 * pow(x, 5.5) -
               0.02578125 * pow(x, 6.5) + 0.020436356707317072 * pow(x, 7.5) -
               0.01671324384973404 * pow(x, 8.5) + 0.013997779702240564 * pow(x, 9.5) -
               0.011945562847590041 * pow(x, 10.5) + 0.01035003662109375 * pow(x, 11.5) -
               0.009080577904069926 * pow(x, 12.5);
      hyperM = 0.5714285714285715 / sqrt(x) + 2.0 * sqrt(x) - 1.4783483195598794 * pow(x, 2.0 / 3.0) +
               0.1 * pow(x, 1.5) - 0.022727272727272735 * pow(x, 2.5) + 0.009191176470588237 * pow(x, 3.5) -
               0.004755434782608697 * pow(x, 4.5) + 0.002828663793103449 * pow(x, 5.5) -
               0.0018415178571428578 * pow(x, 6.5) + 0.0012772722942073172 * pow(x, 7.5) -
               0.0009285135472074472 * pow(x, 8.5) + 0.0006998889851120285 * pow(x, 9.5) -
               0.0005429801294359111 * pow(x, 10.5) + 0.0004312515258789064 * pow(x, 11.5) -
               0.00034925299631038194 * pow(x, 12.5);
    }
  }
  if (a > 0.2) {
    return sqrt(1.0 + (-1.0 + pow(a, -3)) * Omega) *
           (3.4494794123063873799 * pow(-1.0 + 1.0 / Omega, 2.0 / 3.0) +
            (hyperP * (4 * pow(a, 3) * (-1.0 + Omega) - Omega) - 7.0 * pow(a, 3) * hyperM * (-1.0 + Omega)) /
                (pow(a, 5) * (-1.0 + Omega) - pow(a, 2) * Omega));
  }
  return (a * pow(1 - Omega, 1.5) *
          (1291467969 * pow(a, 12) * pow(-1 + Omega, 4) + 1956769650 * pow(a, 9) * pow(-1 + Omega, 3) * Omega +
           8000000000 * pow(a, 3) * (-1 + Omega) * pow(Omega, 3) + 37490640625 * pow(Omega, 4))) /
         (1.5625e10 * pow(Omega, 5));
}
double orc_growthD_fit(double omega, double a) { return growthDtemp(omega, a) / growthDtemp(omega, 1.0); }

/* -------------------------------------------------------- power spectrum */
/* TransferFunc_EH, src/power.c:447-476 (UnitLength = Mpc/h). */
double orc_transfer_eh(const orc_power *p, double k) {
  double hubble = p->h, omegam = p->omega, ombh2 = p->omega_b * p->h * p->h;
  if (p->omega_b == 0) ombh2 = 0.04 * p->h * p->h;
  double theta = 2.728 / 2.7;
  double ommh2 = omegam * hubble * hubble;
  double s = 44.5 * log(9.83 / ommh2) / sqrt(1. + 10. * exp(0.75 * log(ombh2))) * hubble;
  double a = 1. - 0.328 * log(431. * ommh2) * ombh2 / ommh2 + 0.380 * log(22.3 * ommh2) * (ombh2 / ommh2) * (ombh2 / ommh2);
  double gamma = a + (1. - a) / (1. + exp(4 * log(0.43 * k * s)));
  gamma *= omegam * hubble;
  double q = k * theta * theta / gamma;
  double L0 = log(2. * exp(1.) + 1.8 * q);
  double C0 = 14.2 + 731. / (1. + 62.5 * q);
  return L0 / (L0 + C0 * q * q);
}
/* PowerSpec_Tabulated, src/power.c:399-435 */
static double pk_tab(const orc_power *p, double k) {
  double logk = log10(k);
  if (logk < p->tab_logk[0] || logk > p->tab_logk[p->ntab - 1]) return 0;
  int lo = 0, hi = p->ntab - 1;
  while (hi - lo > 1) { int mid = (hi + lo) / 2; if (logk < p->tab_logk[mid]) hi = mid; else lo = mid; }
  double u = (logk - p->tab_logk[lo]) / (p->tab_logk[hi] - p->tab_logk[lo]);
  return p->norm * pow(10.0, (1 - u) * p->tab_logP[lo] + u * p->tab_logP[hi]);
}
/* PowerSpec, src/power.c:373-394 */
double orc_power_spec(const orc_power *p, double k) {
  if (p->nu) return p->norm * orc_nu_pofk_cb(p->nu, k, p->nu_ocdm);  /* power.c:376-380 */
  if (p->which_spectrum == 1) return pk_tab(p, k);
  double T = orc_transfer_eh(p, k);
  return p->norm * pow(k, p->ns) * T * T;
}
struct th_par { const orc_power *p; double R; };
/* sigma2_int, src/power.c:503-516 */
static double sigma2_int(double k, void *v) {
  struct th_par *t = v;
  double kr = t->R * k, kr2 = kr * kr, kr3 = kr2 * kr;
  if (kr < 1e-8) return 0;
  double w = 3 * (sin(kr) / kr3 - cos(kr) / kr2);
  return k * k * w * w * orc_power_spec(t->p, k);
}
/* TopHatSigma2, src/power.c:481-498 */
double orc_tophat_sigma2(const orc_power *p, double R) {
  struct th_par t = {p, R};
  /* split [0, 500/R] into many panels: the integrand oscillates */
  double s = 0, b = 500.0 / R;
  int np = 256;
  for (int i = 0; i < np; i++) s += integrate(sigma2_int, &t, b * i / np, b * (i + 1) / np);
  return s / (2.0 * M_PI * M_PI);
}
/* initialize_powerspectrum, src/power.c:226-257 */
void orc_power_init(orc_power *p) {
  p->norm = 1.0;
  /* with massive neutrinos the normalisation runs before
   * init_modified_version has set OmegaCDM (main.c:153-162), so the
   * CDM+baryon transfer function is the baryon one there */
  p->nu_ocdm = 0.0;
  double res = orc_tophat_sigma2(p, 8.0);
  p->norm = p->sigma8 * p->sigma8 / res;
  if (p->nu) p->nu_ocdm = orc_nu_omega_cdm(p->nu);
}

/* ------------------------------------------------------------ splines */
static void spl_init(spl *s, const double *x, const double *y, int n) {
  s->n = n;
  s->x = malloc(8 * n); s->y = malloc(8 * n); s->y2 = calloc(n, 8);
  memcpy(s->x, x, 8 * n); memcpy(s->y, y, 8 * n);
  double *u = calloc(n, 8);
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * s->y2[i - 1] + 2.0;
    s->y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  for (int k = n - 2; k >= 0; k--) s->y2[k] = s->y2[k] * s->y2[k + 1] + u[k];
  free(u);
}
static double spl_eval(const spl *s, double x) {
  if (x < s->x[0]) x = s->x[0];
  if (x > s->x[s->n - 1]) x = s->x[s->n - 1];
  int lo = 0, hi = s->n - 1;
  while (hi - lo > 1) { int mid = (hi + lo) / 2; if (s->x[mid] > x) hi = mid; else lo = mid; }
  double h = s->x[hi] - s->x[lo], A = (s->x[hi] - x) / h, B = (x - s->x[lo]) / h;
  return A * s->y[lo] + B * s->y[hi] + ((A * A * A - A) * s->y2[lo] + (B * B * B - B) * s->y2[hi]) * (h * h) / 6.0;
}
static void spl_free(spl *s) { free(s->x); free(s->y); free(s->y2); s->x = s->y = s->y2 = NULL; }

/* ----------------------------------------- JBD background, src/jbd.c */
static double jw, jom, jor, jov;
static double jH(double x, double y, double dy) {
  return sqrt(exp(-y) * (jor * exp(-4 * x) + jom * exp(-3 * x) + jov) / (1.0 + dy - jw / 6 * dy * dy));
}
static double jdHdx(double x, double y, double dy) {
  double H = jH(x, y, dy);
  double om = jom * exp(-y - 3.0 * x) / (H * H), ov = jov * exp(-y) / (H * H), ora = jor * exp(-y - 4.0 * x) / (H * H);
  return H / 2.0 * (-3.0 - ora - jw / 2.0 * dy * dy + dy - 3.0 * (om + 4.0 * ov) / (3.0 + 2.0 * jw) + 3.0 * ov);
}
static double jHz(double x, double y, double z) {
  return sqrt(exp(-y) * (jor * exp(-4 * x) + jom * exp(-3 * x) + jov) + z * z / 12.0 * (2.0 * jw + 3.0) * exp(-2 * y - 6 * x)) -
         z / 2.0 * exp(-y - 3 * x);
}
static void jrhs(double x, const double *u, double *f) {
  double hubb = jHz(x, u[0], u[1]);
  f[0] = u[1] * exp(-u[0] - 3 * x) / hubb;
  f[1] = 3.0 * exp(3.0 * x) / (2 * jw + 3) / hubb * (jom * exp(-3 * x) + 4.0 * jov);
}
double orc_jbd_solve(orc_mg *m) {
  const int npts = 10000, nsub = 16;
  jw = m->wBD; jom = m->Omegah2; jor = m->Omegarh2; jov = m->Omegavh2;
  double xini = log(1.0 / (1.0 + 1e6)), dx = -xini / (double)(npts - 1);
  double *x = malloc(8 * npts), *y = malloc(8 * npts), *dy = malloc(8 * npts);
  double lo = 0.0, hi = 1.0;
  for (int it = 0; it < 200; it++) {
    double ph = 0.5 * (lo + hi), u[2] = {log(ph), 0.0};
    x[0] = xini; y[0] = u[0]; dy[0] = 0.0;
    for (int i = 1; i < npts; i++) {
      double h = dx / nsub;
      for (int s = 0; s < nsub; s++) {
        double xx = xini + (i - 1) * dx + s * h, k1[2], k2[2], k3[2], k4[2], t[2];
        jrhs(xx, u, k1);
        for (int q = 0; q < 2; q++) t[q] = u[q] + 0.5 * h * k1[q];
        jrhs(xx + 0.5 * h, t, k2);
        for (int q = 0; q < 2; q++) t[q] = u[q] + 0.5 * h * k2[q];
        jrhs(xx + 0.5 * h, t, k3);
        for (int q = 0; q < 2; q++) t[q] = u[q] + h * k3[q];
        jrhs(xx + h, t, k4);
        for (int q = 0; q < 2; q++) u[q] += h / 6.0 * (k1[q] + 2 * k2[q] + 2 * k3[q] + k4[q]);
      }
      double xn = xini + i * dx;
      x[i] = xn; y[i] = u[0];
      dy[i] = u[1] / jHz(xn, u[0], u[1]) * exp(-3.0 * xn - u[0]);
    }
    double r = exp(y[npts - 1]);
    if (fabs(r - 1.0) < 1e-6) break;
    if (r < 1.0) lo = ph; else hi = ph;
  }
  double h = jH(0.0, y[npts - 1], dy[npts - 1]);
  double *G = malloc(8 * npts), *H = malloc(8 * npts), *dH = malloc(8 * npts);
  for (int i = 0; i < npts; i++) {
    G[i] = exp(-y[i]);
    H[i] = jH(x[i], y[i], dy[i]) / h;
    dH[i] = jdHdx(x[i], y[i], dy[i]) / h * exp(-x[i]);
  }
  if (g_jbd) { spl_free(&g_jbdG); spl_free(&g_jbdH); spl_free(&g_jbddH); }
  spl_init(&g_jbdG, x, G, npts); spl_init(&g_jbdH, x, H, npts); spl_init(&g_jbddH, x, dH, npts);
  g_jbd = 1;
  free(x); free(y); free(dy); free(G); free(H); free(dH);
  m->omega = m->Omegah2 / (h * h);
  return h;
}

/* ------------------------------------- phi_crit(a), src/cosmo.c:104-190 */
static double phia_int(double x, void *p) {
  const orc_mg *m = p;
  double a = exp(x), b = orc_beta_of_a(m, a);
  if (b == 0.0) return 0.0;
  return 9.0 * m->omega * b / (orc_mass2_of_a(m, a) * a * a * a);
}
void orc_phia_solve(const orc_mg *m, double init_redshift) {
  const int npts = 1000;
  double zini = init_redshift > 200.0 ? init_redshift : 200.0;
  double xmin = log(1.0 / (1.0 + zini)), xmax = log(1.0 / (1.0 - 0.5)), dx = (xmax - xmin) / (npts - 1);
  double *x = malloc(8 * npts), *ph = malloc(8 * npts);
  x[0] = xmin; ph[0] = 0.0;
  for (int i = 1; i < npts; i++) {
    x[i] = xmin + i * dx;
    ph[i] = ph[i - 1] + integrate(phia_int, (void *)m, xmin + (i - 1) * dx, x[i]);
  }
  for (int i = 0; i < npts; i++) {
    double b = orc_beta_of_a(m, exp(x[i]));
    if (b != 0.0) ph[i] /= 2.0 * b;
  }
  if (g_phia) spl_free(&g_phia_s);
  spl_init(&g_phia_s, x, ph, npts);
  g_phia = 1;
  free(x); free(ph);
}
double orc_phicrit(const orc_mg *m, double a) {
  (void)m;
  return g_phia ? spl_eval(&g_phia_s, log(a)) : 0.0;
}
