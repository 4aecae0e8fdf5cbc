/*
 * Host FP64 cosmology for the GB300 COLA library.
 *
 * Growth factors: the coupled first/second-order growth ODEs of
 * src/cosmo.c:206-268 in x = ln a, from z = max(200, z_init) to z = -0.5,
 * stored at 1000 knots and interpolated by natural cubic splines with clamped
 * lookup (src/cosmo.c:409-520, src/wrappers.c:102-167).  The reference uses
 * GSL's rk2 driver at eps 1e-7; here an adaptive Dormand-Prince 5(4) pair
 * (J. R. Dormand, P. J. Prince, J. Comp. Appl. Math. 6 (1980) 19) at a
 * relative tolerance of 1e-11 integrates between knots.
 *
 * Quadratures (COLA Sq, sigma_8 normalisation) use adaptive 16-point
 * Gauss-Legendre bisection; nodes are computed by Newton iteration on the
 * Legendre polynomial.
 */
#include "mgp_cosmo.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define INVERSE_H0_MPCH 2997.92458 /* 1/H0 in Mpc/h, src/vars.h:65 */

int mgp_set_error(int code, const char *fmt, ...);

static double spline_eval(const mgp_spline *s, double x);

/* ------------------------------------------------------------------ hooks */
/* Each function below is the built-in model of mgp_params unless the user's
 * hook table replaces it (the hook replaces the whole function, including
 * its modified_gravity_active checks). */
#define HOOK1(name, a) \
  if (c->hooks.name) return c->hooks.name((a), c->hooks.user)

double mgp_hubble(const mgp_cosmo *c, double a) {
  HOOK1(hubble, a);
  const double om = c->p.Omega;
  if (c->have_jbd) return spline_eval(&c->jbdH, log(a));
  if (c->p.use_w0wa)
    return sqrt(om / (a * a * a) + (1.0 - om) * exp(3.0 * c->p.w_a * (a - 1) - 3 * (1 + c->p.w_0 + c->p.w_a) * log(a)));
  return sqrt(om / (a * a * a) + 1.0 - om);
}

double mgp_dhubbleda(const mgp_cosmo *c, double a) {
  HOOK1(dhubbleda, a);
  const double om = c->p.Omega;
  if (c->have_jbd) return spline_eval(&c->jbddH, log(a));
  double rhs = -3.0 * om / (a * a * a * a);
  if (c->p.use_w0wa) rhs += -3.0 * (1.0 - om) * (1.0 + c->p.w_0 + c->p.w_a * (1 - a)) / a;
  return rhs / (2.0 * mgp_hubble(c, a));
}

double mgp_beta_dgp(const mgp_cosmo *c, double a) {
  return 1.0 + 2.0 * c->p.rcH0_DGP * (mgp_hubble(c, a) + a * mgp_dhubbleda(c, a) / 3.0);
}

double mgp_beta_of_a(const mgp_cosmo *c, double a) {
  HOOK1(beta_of_a, a);
  switch (c->p.model) {
    case MGP_MODEL_FOFR: return 1.0 / sqrt(6.0);
    case MGP_MODEL_MBETA: {
      double r = c->p.assb_symm / a;
      return a > c->p.assb_symm ? c->p.beta_symm * sqrt(1.0 - r * r * r) : 0.0;
    }
    default: return 0.0;
  }
}

double mgp_mass2_of_a(const mgp_cosmo *c, double a) {
  HOOK1(mass2_of_a, a);
  if (c->p.model == MGP_MODEL_FOFR) {
    const double om = c->p.Omega, n = c->p.nfofr;
    double fac = om / (a * a * a) + 4.0 * (1.0 - om);
    double fac0 = om + 4.0 * (1.0 - om);
    return fac0 * pow(fac / fac0, n + 2.0) / ((1.0 + n) * c->p.fofr0);
  }
  if (c->p.model == MGP_MODEL_MBETA) {
    double r = c->p.assb_symm / a;
    if (a > c->p.assb_symm) return 0.5 * pow(2998.0 / c->p.range_symm, 2) * (1.0 - r * r * r);
    return 1.0;
  }
  return 0.0;
}

double mgp_coupling(const mgp_cosmo *c, double a) {
  HOOK1(coupling_function, a);
  switch (c->p.model) {
    case MGP_MODEL_FOFR:
    case MGP_MODEL_MBETA: {
      double b = mgp_beta_of_a(c, a);
      return 2.0 * b * b;
    }
    case MGP_MODEL_DGP: return 1.0 / (3.0 * mgp_beta_dgp(c, a));
    case MGP_MODEL_BRANSDICKE: return c->have_jbd ? spline_eval(&c->jbdG, log(a)) - 1.0 : 0.0;
    default: return 0.0;
  }
}

double mgp_geff(const mgp_cosmo *c, double a, double k) {
  if (c->hooks.GeffoverG) return c->hooks.GeffoverG(a, k, c->hooks.user);
  if (!c->p.modified_gravity_active || c->p.use_lcdm_growth_factors) return 1.0;
  switch (c->p.model) {
    case MGP_MODEL_FOFR:
    case MGP_MODEL_MBETA: {
      double k2 = (k * INVERSE_H0_MPCH) * (k * INVERSE_H0_MPCH);
      if (k2 == 0) return 1.0;
      double b = mgp_beta_of_a(c, a);
      return 1.0 + 2.0 * b * b * k2 / (k2 + a * a * mgp_mass2_of_a(c, a));
    }
    case MGP_MODEL_DGP: return 1.0 + 1.0 / (3.0 * mgp_beta_dgp(c, a));
    case MGP_MODEL_BRANSDICKE: return 1.0 + mgp_coupling(c, a);
    default: return 1.0;
  }
}

double mgp_factor_2lpt(const mgp_cosmo *c, double a) {
  HOOK1(Factor_2LPT, a);
  if (!c->p.modified_gravity_active || c->p.use_lcdm_growth_factors) return 1.0;
  if (c->p.model == MGP_MODEL_DGP) {
    double b = mgp_beta_dgp(c, a), r = c->p.rcH0_DGP;
    return 1.0 - (2.0 * r * r * c->p.Omega) / (9.0 * a * a * a * b * b * b * (1 + 1.0 / (3.0 * b)));
  }
  return 1.0;
}

/* dm^2/da / H0^2 (user_defined_functions.h:527-560) */
double mgp_dmass2_of_ada(const mgp_cosmo *c, double a) {
  HOOK1(dmass2_of_ada, a);
  const double om = c->p.Omega;
  if (c->p.model == MGP_MODEL_FOFR) {
    double a3 = a * a * a, fac = om / a3 + 4.0 * (1.0 - om), fac0 = om + 4.0 * (1.0 - om), n = c->p.nfofr;
    double m2 = fac0 * (n + 2.0) * pow(fac / fac0, n + 1.0) / ((1.0 + n) * c->p.fofr0 * fac0);
    return m2 * (-3.0 * om / a3 / a);
  }
  if (c->p.model == MGP_MODEL_MBETA) {
    if (a > c->p.assb_symm) {
      double r = 2998.0 / c->p.range_symm, q = c->p.assb_symm / a;
      return 0.5 * r * r * (3.0 * q * q * q / a);
    }
    return 0.0;
  }
  return 0.0;
}

/* The a-dependent factors of GeffoverG(a, k) and second_order_kernel(k, k1,
 * k2, cos theta, a) (user_defined_functions.h:618-652, 848-904), split so that
 * the scale-dependent growth ODE evaluates them once per a for all k. */
typedef struct {
  double H, alpha, beta0;  /* H/H0, 2 + a H'/H, 1.5 Omega / (a^3 H^2) */
  double geff_const;       /* mu for k-independent models */
  int kdep;                /* mu(k) = 1 + mu_b k2 / (k2 + mu_m) with k2 = (k c/H0)^2 */
  double mu_b, mu_m;
  int g2kind;              /* 0 none, 1 f(R), 2 DGP, 3 m(a)/beta(a) */
  double g2_pref, g2_pi0;  /* f(R): prefactor and pi(k) = (k c/(H0 a))^2 + pi0; MBETA: pi0 = m2 */
  double inv_a2;           /* (c/H0 / a)^2 multiplier of k^2 in pi(k) */
  const mgp_model_hooks *h; /* user GeffoverG / second_order_kernel, called per k */
  double a;
} mgp_sd_apart;

static void sd_apart(const mgp_cosmo *c, double a, mgp_sd_apart *o) {
  const double om = c->p.Omega, a3 = a * a * a;
  memset(o, 0, sizeof(*o));
  o->H = mgp_hubble(c, a);
  o->alpha = 2.0 + a * mgp_dhubbleda(c, a) / o->H;
  o->beta0 = 1.5 * om / (a3 * o->H * o->H);
  o->geff_const = 1.0;
  o->inv_a2 = (INVERSE_H0_MPCH / a) * (INVERSE_H0_MPCH / a);
  o->a = a;
  if (c->hooks.GeffoverG || c->hooks.second_order_kernel) o->h = &c->hooks;
  if (!c->p.modified_gravity_active || c->p.use_lcdm_growth_factors) return;
  switch (c->p.model) {
    case MGP_MODEL_FOFR:
    case MGP_MODEL_MBETA: {
      double b = mgp_beta_of_a(c, a);
      o->kdep = 1;
      o->mu_b = 2.0 * b * b;
      o->mu_m = a * a * mgp_mass2_of_a(c, a);
      if (c->p.model == MGP_MODEL_FOFR) {
        double fac = om / a3 + 4.0 * (1.0 - om), fac0 = om + 4.0 * (1.0 - om), n = c->p.nfofr;
        double cH = INVERSE_H0_MPCH / (a * o->H);
        o->g2kind = 1;
        o->g2_pref = -(3.0 * (n + 2.0) / (12.0 * (1.0 + n) * (1.0 + n))) * cH * cH * (om / a3) * (om / a3) * fac0 *
                     pow(fac / fac0, 2.0 * n + 3.0) / (c->p.fofr0 * c->p.fofr0);
        o->g2_pi0 = fac0 * pow(fac / fac0, n + 2.0) / (1.0 + n) / c->p.fofr0;
      } else {
        double m2 = mgp_mass2_of_a(c, a);
        o->g2kind = 3;
        o->g2_pi0 = m2;
        o->g2_pref = (mgp_dmass2_of_ada(c, a) / m2) * b * b * om / (2.0 * a * a) / (o->H * o->H);
      }
      break;
    }
    case MGP_MODEL_DGP: {
      double bd = mgp_beta_dgp(c, a), r = c->p.rcH0_DGP / o->H;
      o->geff_const = mgp_geff(c, a, 1.0);
      o->g2kind = 2;
      o->g2_pref = -1.0 / 6.0 / (bd * bd * bd) * r * r * (om / a3) * (om / a3);
      break;
    }
    default: o->geff_const = mgp_geff(c, a, 1.0); break;
  }
}

static double sd_mu(const mgp_sd_apart *o, double k) {
  if (o->h && o->h->GeffoverG) return o->h->GeffoverG(o->a, k, o->h->user);
  if (!o->kdep) return o->geff_const;
  double k2 = (k * INVERSE_H0_MPCH) * (k * INVERSE_H0_MPCH);
  if (k2 == 0) return 1.0;
  return 1.0 + o->mu_b * k2 / (k2 + o->mu_m);
}

/* second_order_kernel(k, k/sqrt2, k/sqrt2, 0, a): the cos(theta) term of the
 * reference vanishes at cos(theta) = 0. */
static double sd_gamma2(const mgp_sd_apart *o, double k) {
  if (o->h && o->h->second_order_kernel)
    return o->h->second_order_kernel(k, k / sqrt(2.0), k / sqrt(2.0), 0.0, o->a, o->h->user);
  double k2 = k * k * o->inv_a2, k12 = 0.5 * k2;
  switch (o->g2kind) {
    case 1: return o->g2_pref * k * k / ((k2 + o->g2_pi0) * (k12 + o->g2_pi0) * (k12 + o->g2_pi0));
    case 2: return o->g2_pref;
    case 3: {
      double m2 = o->g2_pi0, p1 = k12 + m2;
      return o->g2_pref * (m2 / p1) * (m2 / p1) * (1.0 - m2 / (k2 + m2));
    }
    default: return 0.0;
  }
}

/* modfac of ode_growth_D in the SCALEDEPENDENT build (src/cosmo.c:215-219) */
static double sd_modfac(const mgp_sd_apart *o, double a, double k, double mu, double omega) {
  double a2H = a * a * o->H;
  return 1.0 + 2.0 * a2H * a2H * sd_gamma2(o, k) / (1.5 * omega * a * mu);
}

double mgp_phicrit(const mgp_cosmo *c, double a) {
  HOOK1(phi_of_a, a);
  const double om = c->p.Omega;
  if (c->p.model == MGP_MODEL_MBETA) return c->have_phia ? spline_eval(&c->phia, log(a)) : 0.0;
  return 1.5 * c->p.fofr0 * pow((om + 4.0 * (1.0 - om)) / (om / (a * a * a) + 4.0 * (1.0 - om)), c->p.nfofr + 1.0);
}

double mgp_dgp_screen_prefactor(const mgp_cosmo *c, double a) {
  double r = c->p.rcH0_DGP / mgp_beta_dgp(c, a);
  return 8.0 / 9.0 * c->p.Omega * r * r;
}

/* ---------------------------------------------------------------- splines */
static void spline_init(mgp_spline *s, const double *x, const double *y, int n) {
  s->n = n;
  s->x = (double *)malloc(sizeof(double) * n);
  s->y = (double *)malloc(sizeof(double) * n);
  s->y2 = (double *)calloc(n, sizeof(double));
  double *u = (double *)calloc(n, sizeof(double));
  memcpy(s->x, x, sizeof(double) * n);
  memcpy(s->y, y, sizeof(double) * n);
  for (int i = 1; i + 1 < n; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double pp = sig * s->y2[i - 1] + 2.0;
    double d = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    s->y2[i] = (sig - 1.0) / pp;
    u[i] = (6.0 * d / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / pp;
  }
  for (int k = n - 2; k >= 0; k--) s->y2[k] = s->y2[k] * s->y2[k + 1] + u[k];
  free(u);
}

static double spline_eval(const mgp_spline *s, double x) {
  if (x < s->x[0]) x = s->x[0];
  if (x > s->x[s->n - 1]) x = s->x[s->n - 1];
  int lo = 0, hi = s->n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (s->x[mid] > x) hi = mid; else lo = mid;
  }
  double h = s->x[hi] - s->x[lo], A = (s->x[hi] - x) / h, B = 1.0 - A;
  return A * s->y[lo] + B * s->y[hi] + ((A * A * A - A) * s->y2[lo] + (B * B * B - B) * s->y2[hi]) * h * h / 6.0;
}

static void spline_free(mgp_spline *s) {
  free(s->x); free(s->y); free(s->y2);
  memset(s, 0, sizeof(*s));
}

/* ------------------------------------------------------------- quadrature */
static double gx[8], gw[8];
static int g_ready = 0;
static void gl16_init(void) {
  if (g_ready) return;
  for (int i = 0; i < 8; i++) {
    double x = cos(M_PI * (i + 0.75) / 16.5), dp = 1.0;
    for (int it = 0; it < 50; it++) {
      double p0 = 1.0, p1 = x;
      for (int n = 2; n <= 16; n++) { double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n; p0 = p1; p1 = p2; }
      dp = 16 * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    gx[i] = x;
    gw[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  g_ready = 1;
}
typedef double (*qfn)(double, const void *);
static double gl16(qfn f, const void *par, double a, double b) {
  double m = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
  for (int i = 0; i < 8; i++) s += gw[i] * (f(m - h * gx[i], par) + f(m + h * gx[i], par));
  return s * h;
}
static double qadapt(qfn f, const void *par, double a, double b, double whole, double tol, int depth) {
  double m = 0.5 * (a + b), l = gl16(f, par, a, m), r = gl16(f, par, m, b);
  if (depth >= 18 || fabs(l + r - whole) <= tol) return l + r;
  return qadapt(f, par, a, m, l, 0.5 * tol, depth + 1) + qadapt(f, par, m, b, r, 0.5 * tol, depth + 1);
}
static double quad(qfn f, const void *par, double a, double b, int panels) {
  gl16_init();
  double tot = 0.0, s = 0.0;
  double *est = (double *)malloc(sizeof(double) * panels);
  for (int i = 0; i < panels; i++) {
    est[i] = gl16(f, par, a + (b - a) * i / panels, a + (b - a) * (i + 1) / panels);
    tot += fabs(est[i]);
  }
  double tol = 1e-13 * tot / panels + 1e-300;
  for (int i = 0; i < panels; i++)
    s += qadapt(f, par, a + (b - a) * i / panels, a + (b - a) * (i + 1) / panels, est[i], tol, 0);
  free(est);
  return s;
}

/* massive-neutrino factors of the growth equations (defined below) */
typedef struct {
  int nx;
  double *rows; /* 8 nx: value and d/d ln k of the four transfer functions */
} nu_rows;
static void nu_rows_at(const mgp_cosmo *c, double a, nu_rows *o);
static double nu_mu1(const mgp_cosmo *c, const nu_rows *o, double k);
static double nu_mu2(const mgp_cosmo *c);

/* ------------------------------------------------------------ growth ODE */
typedef struct { const mgp_cosmo *c; int lcdm; } ode_par;

static void growth_rhs(const ode_par *op, double x, const double *y, double *f) {
  const mgp_cosmo *c = op->c;
  double a = exp(x), H = mgp_hubble(c, a), dH = mgp_dhubbleda(c, a);
  double mu = op->lcdm ? 1.0 : mgp_geff(c, a, 1e-3);
  double beta = 1.5 * c->p.Omega * mu / (a * a * a * H * H);
  double alpha = 2.0 + a * dH / H;
  double mod = 1.0;
  if (!op->lcdm) {
    if (c->p.scaledependent) {
      mgp_sd_apart o;
      sd_apart(c, a, &o);
      mod = sd_modfac(&o, a, 1e-3, mu, c->p.Omega);
    } else {
      mod = mgp_factor_2lpt(c, a);
    }
  }
  double mu1 = 1.0;
  if (c->nu_growth) {
    /* ode_growth_D / ode_growth_DLCDM at k_value = 1e-3 (cosmo.c:227-236,
     * 256-265, 459) */
    double *buf = (double *)malloc(sizeof(double) * 8 * c->nuT[0].nx);
    nu_rows nr = {0, buf};
    nu_rows_at(c, a, &nr);
    mu1 = nu_mu1(c, &nr, 1e-3);
    free(buf);
  }
  f[0] = y[1];
  f[1] = -alpha * y[1] + beta * mu1 * y[0];
  f[2] = y[3];
  f[3] = -alpha * y[3] + beta * nu_mu2(c) * (y[2] - mod * y[0] * y[0]);
}

/* Dormand-Prince 5(4) coefficients (Dormand & Prince 1980, Table 2). */
static const double DP_C[7] = {0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1, 1};
static const double DP_A[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
static const double DP_B5[7] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0};
static const double DP_B4[7] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};

/* Integrate y from x0 to x1 (adaptive); returns 0 on success. */
static int dp45(const ode_par *op, double x0, double x1, double *y, double *hguess) {
  double x = x0, h = *hguess;
  int steps = 0;
  while (x < x1) {
    if (x + h > x1) h = x1 - x;
    double k[7][4], yt[4], y5[4], err = 0.0;
    for (int s = 0; s < 7; s++) {
      for (int i = 0; i < 4; i++) {
        double acc = y[i];
        for (int j = 0; j < s; j++) acc += h * DP_A[s][j] * k[j][i];
        yt[i] = acc;
      }
      growth_rhs(op, x + DP_C[s] * h, yt, k[s]);
    }
    for (int i = 0; i < 4; i++) {
      double s5 = y[i], s4 = y[i];
      for (int s = 0; s < 7; s++) { s5 += h * DP_B5[s] * k[s][i]; s4 += h * DP_B4[s] * k[s][i]; }
      y5[i] = s5;
      double sc = 1e-11 * (fabs(y[i]) > fabs(s5) ? fabs(y[i]) : fabs(s5)) + 1e-14;
      double e = fabs(s5 - s4) / sc;
      if (e > err) err = e;
    }
    if (err <= 1.0) {
      x += h;
      memcpy(y, y5, sizeof(y5));
    }
    double fac = err > 0 ? 0.9 * pow(err, -0.2) : 5.0;
    if (fac > 5.0) fac = 5.0;
    if (fac < 0.2) fac = 0.2;
    h *= fac;
    if (++steps > 10000000 || !(h > 1e-14)) return -1;
  }
  *hguess = h;
  return 0;
}

static double Qfactor(const mgp_cosmo *c, double a) { return mgp_hubble(c, a) * a * a * a; }

static int solve_growth(mgp_cosmo *c, char *err, size_t errlen) {
  const int npts = 1000;
  double zini = c->p.Init_Redshift > 200.0 ? c->p.Init_Redshift : 200.0;
  double xini = log(1.0 / (1.0 + zini)), xend = log(1.0 / (1.0 - 0.5));
  double dx = (xend - xini) / (double)(npts - 1);
  double *buf = (double *)malloc(sizeof(double) * npts * 13);
  double *x = buf, *v[12];
  for (int i = 0; i < 12; i++) v[i] = buf + npts * (i + 1);
  double y[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0}, yl[4] = {1.0, 1.0, -3.0 / 7.0, -6.0 / 7.0};
  double h = 1e-4, hl = 1e-4;
  ode_par op = {c, 0}, opl = {c, 1};
  for (int i = 0; i < npts; i++) {
    double xn = xini + i * dx;
    if (i > 0) {
      if (dp45(&op, xini + (i - 1) * dx, xn, y, &h) || dp45(&opl, xini + (i - 1) * dx, xn, yl, &hl)) {
        snprintf(err, errlen, "growth ODE integration failed at x = %f", xn);
        free(buf);
        return MGP_ENUMERIC;
      }
    }
    double a = exp(xn), mu = mgp_geff(c, a, 1e-3), qa = Qfactor(c, a) / a, om = c->p.Omega;
    x[i] = xn;
    v[0][i] = y[0];
    v[1][i] = y[1] * qa;
    v[2][i] = 1.5 * mu * om * a * y[0];
    v[3][i] = y[2];
    v[4][i] = y[3] * qa;
    v[5][i] = 1.5 * mu * om * a * (y[2] - y[0] * y[0] * mgp_factor_2lpt(c, a));
    v[6][i] = yl[0];
    v[7][i] = yl[1] * qa;
    v[8][i] = 1.5 * om * a * yl[0];
    v[9][i] = yl[2];
    v[10][i] = yl[3] * qa;
    v[11][i] = 1.5 * om * a * (yl[2] - yl[0] * yl[0]);
  }
  mgp_spline *sp[12] = {&c->D, &c->dDdy, &c->ddDddy, &c->D2, &c->dD2dy, &c->ddD2ddy,
                        &c->DL, &c->dDLdy, &c->ddDLddy, &c->D2L, &c->dD2Ldy, &c->ddD2Lddy};
  for (int i = 0; i < 12; i++) spline_init(sp[i], x, v[i], npts);
  free(buf);
  return MGP_OK;
}

/* ------------------------------------------- scale-dependent growth tables */
/* Bicubic interpolation on the (ln a, ln k) grid as GSL's
 * gsl_interp2d_bicubic (src/wrappers.c:101-136): node derivatives from
 * natural cubic splines along the grid lines (z_x along x, z_y along y,
 * z_xy = d/dx of z_y), tensor-product cubic Hermite cells. */
static void node_derivs(const double *x, const double *y, long ys, int n, double *d, long ds, double *M, double *u) {
  M[0] = u[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]), p = sig * M[i - 1] + 2.0;
    M[i] = (sig - 1.0) / p;
    double r = (y[(i + 1) * ys] - y[i * ys]) / (x[i + 1] - x[i]) - (y[i * ys] - y[(i - 1) * ys]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * r / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  M[n - 1] = 0.0;
  for (int k = n - 2; k >= 0; k--) M[k] = M[k] * M[k + 1] + u[k];
  for (int i = 0; i < n - 1; i++) {
    double h = x[i + 1] - x[i];
    d[i * ds] = (y[(i + 1) * ys] - y[i * ys]) / h - h * (2.0 * M[i] + M[i + 1]) / 6.0;
  }
  double h = x[n - 1] - x[n - 2];
  d[(n - 1) * ds] = (y[(n - 1) * ys] - y[(n - 2) * ys]) / h + h * (M[n - 2] + 2.0 * M[n - 1]) / 6.0;
}

static void bicubic_init(mgp_bicubic *b, const double *x, const double *y, double *z, int nx, int ny) {
  size_t nn = (size_t)nx * ny;
  b->nx = nx;
  b->ny = ny;
  b->x = (double *)malloc(sizeof(double) * nx);
  b->y = (double *)malloc(sizeof(double) * ny);
  memcpy(b->x, x, sizeof(double) * nx);
  memcpy(b->y, y, sizeof(double) * ny);
  b->z = z;
  b->zx = (double *)malloc(sizeof(double) * nn);
  b->zy = (double *)malloc(sizeof(double) * nn);
  b->zxy = (double *)malloc(sizeof(double) * nn);
  int m = nx > ny ? nx : ny;
  double *M = (double *)malloc(sizeof(double) * 2 * m);
  for (int j = 0; j < ny; j++) node_derivs(b->x, z + (size_t)j * nx, 1, nx, b->zx + (size_t)j * nx, 1, M, M + m);
  for (int i = 0; i < nx; i++) node_derivs(b->y, z + i, nx, ny, b->zy + i, nx, M, M + m);
  for (int j = 0; j < ny; j++)
    node_derivs(b->x, b->zy + (size_t)j * nx, 1, nx, b->zxy + (size_t)j * nx, 1, M, M + m);
  free(M);
}

static void bicubic_free(mgp_bicubic *b) {
  free(b->x); free(b->y); free(b->z); free(b->zx); free(b->zy); free(b->zxy);
  memset(b, 0, sizeof(*b));
}

static int grid_cell(const double *x, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int m = (lo + hi) / 2;
    if (x[m] > v) hi = m;
    else lo = m;
  }
  return lo;
}

/* value and d/dy of the bicubic along x = xv (clamped) at every y node: the
 * cubic Hermite in x of z and z_y (exact restriction of the bicubic) */
static void bicubic_column(const mgp_bicubic *b, double xv, double *val, double *dval) {
  if (xv < b->x[0]) xv = b->x[0];
  if (xv > b->x[b->nx - 1]) xv = b->x[b->nx - 1];
  int i = grid_cell(b->x, b->nx, xv);
  double dx = b->x[i + 1] - b->x[i], t = (xv - b->x[i]) / dx;
  double h0 = (1 + 2 * t) * (1 - t) * (1 - t), h1 = t * t * (3 - 2 * t), g0 = t * (1 - t) * (1 - t) * dx,
         g1 = t * t * (t - 1) * dx;
  for (int j = 0; j < b->ny; j++) {
    size_t c0 = (size_t)j * b->nx + i, c1 = c0 + 1;
    val[j] = h0 * b->z[c0] + h1 * b->z[c1] + g0 * b->zx[c0] + g1 * b->zx[c1];
    dval[j] = h0 * b->zy[c0] + h1 * b->zy[c1] + g0 * b->zxy[c0] + g1 * b->zxy[c1];
  }
}

/* cubic Hermite in y of a column (val, dval on the y nodes), y clamped */
static double column_eval(const mgp_bicubic *b, const double *val, const double *dval, double yv) {
  if (yv < b->y[0]) yv = b->y[0];
  if (yv > b->y[b->ny - 1]) yv = b->y[b->ny - 1];
  int j = grid_cell(b->y, b->ny, yv);
  double dy = b->y[j + 1] - b->y[j], u = (yv - b->y[j]) / dy;
  return (1 + 2 * u) * (1 - u) * (1 - u) * val[j] + u * u * (3 - 2 * u) * val[j + 1] +
         u * (1 - u) * (1 - u) * dy * dval[j] + u * u * (u - 1) * dy * dval[j + 1];
}

/* value and d/dx of the bicubic along y = yv (clamped) at every x node: the
 * cubic Hermite in y of z and z_x */
static void bicubic_row(const mgp_bicubic *b, double yv, double *val, double *dval) {
  if (yv < b->y[0]) yv = b->y[0];
  if (yv > b->y[b->ny - 1]) yv = b->y[b->ny - 1];
  int j = grid_cell(b->y, b->ny, yv);
  double dy = b->y[j + 1] - b->y[j], u = (yv - b->y[j]) / dy;
  double h0 = (1 + 2 * u) * (1 - u) * (1 - u), h1 = u * u * (3 - 2 * u), g0 = u * (1 - u) * (1 - u) * dy,
         g1 = u * u * (u - 1) * dy;
  for (int i = 0; i < b->nx; i++) {
    size_t c0 = (size_t)j * b->nx + i, c1 = c0 + b->nx;
    val[i] = h0 * b->z[c0] + h1 * b->z[c1] + g0 * b->zy[c0] + g1 * b->zy[c1];
    dval[i] = h0 * b->zx[c0] + h1 * b->zx[c1] + g0 * b->zxy[c0] + g1 * b->zxy[c1];
  }
}

/* cubic Hermite in x of a row (val, dval on the x nodes), x clamped */
static double row_eval(const mgp_bicubic *b, const double *val, const double *dval, double xv) {
  if (xv < b->x[0]) xv = b->x[0];
  if (xv > b->x[b->nx - 1]) xv = b->x[b->nx - 1];
  int i = grid_cell(b->x, b->nx, xv);
  double dx = b->x[i + 1] - b->x[i], t = (xv - b->x[i]) / dx;
  return (1 + 2 * t) * (1 - t) * (1 - t) * val[i] + t * t * (3 - 2 * t) * val[i + 1] +
         t * (1 - t) * (1 - t) * dx * dval[i] + t * t * (t - 1) * dx * dval[i + 1];
}

/* ------------------------------------------------------ massive neutrinos */
/* The CAMB transfer functions at one redshift z = 1/a - 1 as rows over ln k
 * (Lookup_GSL_2D_Spline(spline, ln k, z), clamped, src/wrappers.c:132-139):
 * rows[2 q], rows[2 q + 1] value and d/d ln k of table q (nu, cdm, baryon,
 * total).  Every file shares the same k nodes. */
static void nu_rows_at(const mgp_cosmo *c, double a, nu_rows *o) {
  o->nx = c->nuT[0].nx;
  for (int q = 0; q < 4; q++)
    bicubic_row(&c->nuT[q], 1.0 / a - 1.0, o->rows + 2 * q * o->nx, o->rows + (2 * q + 1) * o->nx);
}
static double nu_T(const mgp_cosmo *c, const nu_rows *o, int q, double k) {
  return row_eval(&c->nuT[q], o->rows + 2 * q * o->nx, o->rows + (2 * q + 1) * o->nx, log(k));
}
/* get_cdm_baryon_transfer_function (read_CAMB_data.h:198-201) */
static double nu_Tcb(const mgp_cosmo *c, const nu_rows *o, double k, double ocdm) {
  const double ob = c->p.OmegaBaryon;
  return (ob * nu_T(c, o, 2, k) + ocdm * nu_T(c, o, 1, k)) / (ob + ocdm);
}
/* GeffoverG_neutrino_1LPT / _2LPT (user_defined_functions.h:664-684) */
static double nu_mu1(const mgp_cosmo *c, const nu_rows *o, double k) {
  if (!c->nu_growth) return 1.0;
  const double om = c->p.Omega;
  return (om - c->OmegaNu) / om + c->OmegaNu / om * nu_T(c, o, 0, k) / nu_Tcb(c, o, k, c->OmegaCDM);
}
static double nu_mu2(const mgp_cosmo *c) { return c->nu_growth ? (c->p.Omega - c->OmegaNu) / c->p.Omega : 1.0; }

/* read_and_spline_transfer_functions + read_single_transfer_function_file
 * (src/read_CAMB_data.h:41-170, 238-278) */
static int read_camb(mgp_cosmo *c, char *err, size_t errlen) {
  FILE *fp = fopen(c->p.nu_FilenameTransferInfofile, "r");
  if (!fp) {
    snprintf(err, errlen, "Error read_and_spline_transfer_functions: cannot read [%s]", c->p.nu_FilenameTransferInfofile);
    return MGP_EIO;
  }
  char dir[500];
  int nz = 0;
  if (fscanf(fp, "%499s %d", dir, &nz) != 2 || nz < 2) {
    fclose(fp);
    snprintf(err, errlen, "transfer info file '%s': need '<dir> <n>' with n >= 2", c->p.nu_FilenameTransferInfofile);
    return MGP_EPARAM;
  }
  double *zs = (double *)malloc(sizeof(double) * nz), *logk = NULL, *T[4] = {NULL, NULL, NULL, NULL};
  int nk = 0, rc = MGP_OK;
  const int col[4] = {5, 1, 2, 6}; /* T_massive_nu, T_cdm, T_b, T_tot */
  for (int i = 0; i < nz && rc == MGP_OK; i++) {
    char fn[500], path[1100];
    if (fscanf(fp, "%499s %lf", fn, &zs[i]) != 2) {
      snprintf(err, errlen, "transfer info file: short list (%d of %d files)", i, nz);
      rc = MGP_EPARAM;
      break;
    }
    if (i > 0 && !(zs[i] > zs[i - 1])) {
      snprintf(err, errlen, "transfer files must be listed with increasing redshift");
      rc = MGP_EPARAM;
      break;
    }
    snprintf(path, sizeof(path), "%s/%s", dir, fn);
    FILE *tf = fopen(path, "r");
    if (!tf) {
      snprintf(err, errlen, "Error ed_camb_transfer_function_file: cannot open [%s]", path);
      rc = MGP_EIO;
      break;
    }
    int ch;
    while ((ch = fgetc(tf)) != EOF && ch != '\n') {
    } /* one header line */
    int cap = 256, n = 0;
    double *rows = (double *)malloc(sizeof(double) * 13 * cap), v[13];
    for (;;) {
      int got = 0;
      while (got < 13 && fscanf(tf, "%lf", &v[got]) == 1) got++;
      if (got == 0) break;
      if (got < 13) {
        snprintf(err, errlen, "transfer file '%s': a row with %d of 13 columns", path, got);
        rc = MGP_EIO;
        break;
      }
      if (n == cap) {
        cap *= 2;
        rows = (double *)realloc(rows, sizeof(double) * 13 * cap);
      }
      memcpy(rows + 13 * n, v, sizeof(v));
      n++;
    }
    fclose(tf);
    if (rc == MGP_OK && i == 0) {
      nk = n;
      logk = (double *)malloc(sizeof(double) * nk);
      for (int q = 0; q < 4; q++) T[q] = (double *)malloc(sizeof(double) * (size_t)nz * nk);
      for (int j = 0; j < nk; j++) logk[j] = log(rows[13 * j]);
    }
    if (rc == MGP_OK && (n != nk || nk < 4)) {
      snprintf(err, errlen, "transfer file '%s' has %d rows where %d expected (same k nodes in every file)", path, n, nk);
      rc = MGP_EIO;
    }
    for (int j = 0; j < nk && rc == MGP_OK; j++)
      for (int q = 0; q < 4; q++) T[q][(size_t)i * nk + j] = rows[13 * j + col[q]];
    free(rows);
  }
  fclose(fp);
  if (rc == MGP_OK)
    for (int q = 0; q < 4; q++) bicubic_init(&c->nuT[q], logk, zs, T[q], nk, nz);
  else
    for (int q = 0; q < 4; q++) free(T[q]);
  free(logk);
  free(zs);
  return rc;
}

/* get_total_power_spectrum / get_cdm_baryon_power_spectrum at z = 0
 * (read_CAMB_data.h:215-228), before the normalisation */
static double nu_pofk_cb(const mgp_cosmo *c, double k, double ocdm) {
  const double h = c->p.HubbleParam;
  const nu_rows o = {c->nuT[0].nx, c->nu_rows0};
  const double Ttot = nu_T(c, &o, 3, k), Tcb = nu_Tcb(c, &o, k, ocdm);
  const double ptot = 2.0 * M_PI * M_PI * Ttot * Ttot * (k * h) * pow(k * h / 0.05, c->p.PrimordialIndex - 1.0) * h * h * h;
  return ptot * (Tcb / Ttot) * (Tcb / Ttot);
}

/* Dormand-Prince 5(4) over all k at once with one shared step size (the
 * a-dependent parts of the right-hand side are evaluated once per stage). */
typedef struct {
  const mgp_cosmo *c;
  int nk;
  const double *k;
  int lcdm;      /* mu = 1 and modfac = 1 (the LCDM growth of the neutrino build) */
  double *nubuf; /* 8 nx scratch for the neutrino rows */
} sd_ode;

static void sd_rhs(const sd_ode *o, double x, const double *y, double *f) {
  double a = exp(x), om = o->c->p.Omega;
  mgp_sd_apart ap;
  sd_apart(o->c, a, &ap);
  nu_rows nr = {0, o->nubuf};
  if (o->c->nu_growth) nu_rows_at(o->c, a, &nr);
  const double mu2 = nu_mu2(o->c);
  for (int q = 0; q < o->nk; q++) {
    const double *Y = y + 4 * q;
    double *F = f + 4 * q;
    double mu = o->lcdm ? 1.0 : sd_mu(&ap, o->k[q]);
    double beta = ap.beta0 * mu, mod = o->lcdm ? 1.0 : sd_modfac(&ap, a, o->k[q], mu, om);
    double mu1 = o->c->nu_growth ? nu_mu1(o->c, &nr, o->k[q]) : 1.0;
    F[0] = Y[1];
    F[1] = -ap.alpha * Y[1] + beta * mu1 * Y[0];
    F[2] = Y[3];
    F[3] = -ap.alpha * Y[3] + beta * mu2 * (Y[2] - mod * Y[0] * Y[0]);
  }
}

static int sd_dp45(const sd_ode *o, double x0, double x1, double *y, double *hguess, double *work) {
  const int n = 4 * o->nk;
  double *K[7], *yt = work + 7 * n, *y5 = work + 8 * n;
  for (int s = 0; s < 7; s++) K[s] = work + s * n;
  double x = x0, h = *hguess;
  int steps = 0;
  while (x < x1) {
    if (x + h > x1) h = x1 - x;
    for (int s = 0; s < 7; s++) {
      for (int i = 0; i < n; i++) {
        double acc = y[i];
        for (int j = 0; j < s; j++) acc += h * DP_A[s][j] * K[j][i];
        yt[i] = acc;
      }
      sd_rhs(o, x + DP_C[s] * h, yt, K[s]);
    }
    double err = 0.0;
    for (int i = 0; i < n; i++) {
      double s5 = y[i], s4 = y[i];
      for (int s = 0; s < 7; s++) {
        s5 += h * DP_B5[s] * K[s][i];
        s4 += h * DP_B4[s] * K[s][i];
      }
      y5[i] = s5;
      double sc = 1e-10 * (fabs(y[i]) > fabs(s5) ? fabs(y[i]) : fabs(s5)) + 1e-14;
      double e = fabs(s5 - s4) / sc;
      if (e > err) err = e;
    }
    if (err <= 1.0) {
      x += h;
      memcpy(y, y5, sizeof(double) * n);
    }
    double fac = err > 0 ? 0.9 * pow(err, -0.2) : 5.0;
    if (fac > 5.0) fac = 5.0;
    if (fac < 0.2) fac = 0.2;
    h *= fac;
    if (++steps > 1000000 || !(h > 1e-14)) return -1;
  }
  *hguess = h;
  return 0;
}

/* calculate_scale_dependent_growth_factor (src/cosmo.c:798-981); lcdm = 1
 * solves the LCDM growth of the neutrino build (cosmo.c:829-884: mu = 1,
 * modfac = 1, the neutrino factor kept) and keeps only D(k, a). */
static int solve_growth_sd(mgp_cosmo *c, int lcdm, char *err, size_t errlen) {
  const int npts = 1000;
  const int nk = c->p.sd_nk > 0 ? c->p.sd_nk : 1000;
  const double kmin = c->p.sd_kmin > 0 ? c->p.sd_kmin : 2.0 * M_PI / c->p.Box * 0.5;
  const double kmax = c->p.sd_kmax > 0 ? c->p.sd_kmax : 2.0 * M_PI / c->p.Box * c->p.Nmesh * sqrt(3.0) * 2.0;
  if (nk < 4 || !(kmax > kmin) || !(kmin > 0)) {
    snprintf(err, errlen, "scale-dependent k grid: nk = %d, kmin = %g, kmax = %g", nk, kmin, kmax);
    return MGP_EPARAM;
  }
  double zini = c->p.Init_Redshift > 200.0 ? c->p.Init_Redshift : 200.0;
  double xini = log(1.0 / (1.0 + zini)), xend = log(1.0 / (1.0 - 0.5));
  double *x = (double *)malloc(sizeof(double) * npts), *logk = (double *)malloc(sizeof(double) * nk);
  double *kk = (double *)malloc(sizeof(double) * nk);
  double *y = (double *)malloc(sizeof(double) * 4 * nk), *work = (double *)malloc(sizeof(double) * 9 * 4 * nk);
  double *T[6];
  for (int f = 0; f < 6; f++) T[f] = (double *)malloc(sizeof(double) * (size_t)npts * nk);
  for (int i = 0; i < npts; i++) x[i] = xini + (xend - xini) * i / (double)(npts - 1);
  for (int q = 0; q < nk; q++) {
    logk[q] = log(kmin) + log(kmax / kmin) * q / (double)(nk - 1);
    kk[q] = exp(logk[q]);
    y[4 * q] = 1.0;
    y[4 * q + 1] = 1.0;
    y[4 * q + 2] = -3.0 / 7.0;
    y[4 * q + 3] = -6.0 / 7.0;
  }
  double *nubuf = c->nu_growth ? (double *)malloc(sizeof(double) * 8 * c->nuT[0].nx) : NULL;
  sd_ode o = {c, nk, kk, lcdm, nubuf};
  double h = 1e-4;
  int rc = MGP_OK;
  for (int i = 0; i < npts && rc == MGP_OK; i++) {
    if (i > 0 && sd_dp45(&o, x[i - 1], x[i], y, &h, work)) {
      snprintf(err, errlen, "scale-dependent growth ODE integration failed at x = %f", x[i]);
      rc = MGP_ENUMERIC;
      break;
    }
    double a = exp(x[i]), qa = Qfactor(c, a) / a, om = c->p.Omega;
    mgp_sd_apart ap;
    sd_apart(c, a, &ap);
    nu_rows nr = {0, nubuf};
    if (c->nu_growth) nu_rows_at(c, a, &nr);
    const double mu2 = nu_mu2(c);
    for (int q = 0; q < nk; q++) {
      const double *Y = y + 4 * q;
      double mu = lcdm ? 1.0 : sd_mu(&ap, kk[q]), mu1 = c->nu_growth ? nu_mu1(c, &nr, kk[q]) : 1.0;
      size_t cc = (size_t)q * npts + i;
      T[0][cc] = Y[0];
      T[1][cc] = Y[1] * qa;
      T[2][cc] = 1.5 * mu * mu1 * om * a * Y[0];
      T[3][cc] = Y[2];
      T[4][cc] = Y[3] * qa;
      T[5][cc] = 1.5 * mu * mu2 * om * a * (Y[2] - Y[0] * Y[0]);
    }
  }
  if (rc == MGP_OK && lcdm) {
    bicubic_init(&c->sd_lcdm, x, logk, T[0], npts, nk);
    for (int f = 1; f < 6; f++) free(T[f]);
  } else if (rc == MGP_OK) {
    for (int f = 0; f < 6; f++) bicubic_init(&c->sd_tab[f], x, logk, T[f], npts, nk);
    c->sd = 1;
  } else {
    for (int f = 0; f < 6; f++) free(T[f]);
  }
  free(x); free(logk); free(kk); free(y); free(work); free(nubuf);
  return rc;
}

int mgp_cosmo_sd_column(const mgp_cosmo *c, int which, double a, double *val, double *dval) {
  if (!c->sd || which < 0 || which > 5) return MGP_ESTATE;
  bicubic_column(&c->sd_tab[which], log(a), val, dval);
  return MGP_OK;
}

/* growth_*_scaledependent (src/cosmo.c:987-1010): which 0-5 as
 * D, dDdy, ddDddy, D2, dD2dy, ddD2ddy, normalised at a = 1 per k. */
double mgp_cosmo_growth_sd(const mgp_cosmo *c, int which, double k, double a) {
  if (!c->sd || which < 0 || which > 5) return NAN;
  const mgp_bicubic *b = &c->sd_tab[which], *nb = &c->sd_tab[which < 3 ? 0 : 3];
  int ny = b->ny;
  double *col = (double *)malloc(sizeof(double) * 4 * ny);
  bicubic_column(b, log(a), col, col + ny);
  bicubic_column(nb, 0.0, col + 2 * ny, col + 3 * ny);
  double r = column_eval(b, col, col + ny, log(k)) / column_eval(nb, col + 2 * ny, col + 3 * ny, log(k));
  free(col);
  return r;
}

double mgp_cosmo_growth(const mgp_cosmo *c, int which, double a) {
  double la = log(a);
  switch (which) {
    case 0: return spline_eval(&c->D, la) / spline_eval(&c->D, 0.0);
    case 1: return spline_eval(&c->dDdy, la) / spline_eval(&c->D, 0.0);
    case 2: return spline_eval(&c->ddDddy, la) / spline_eval(&c->D, 0.0);
    case 3: return spline_eval(&c->D2, la) / spline_eval(&c->D2, 0.0);
    case 4: return spline_eval(&c->dD2dy, la) / spline_eval(&c->D2, 0.0);
    case 5: return spline_eval(&c->ddD2ddy, la) / spline_eval(&c->D2, 0.0);
    case 6: return spline_eval(&c->DL, la) / spline_eval(&c->DL, 0.0);
    default: return NAN;
  }
}

/* COLA: gpQ(a) = a^nLPT with nLPT = -2.5 and fullT = 1 (src/main.c:82-85,
 * src/cosmo.c:1114-1160). */
static double sq_integrand(double a, const void *par) {
  return pow(a, -2.5) / Qfactor((const mgp_cosmo *)par, a);
}
double mgp_cosmo_Sq(const mgp_cosmo *c, double ai, double af, double aref) {
  return quad(sq_integrand, c, ai, af, 4) / pow(aref, -2.5);
}
double mgp_cosmo_Sphi(const mgp_cosmo *c, double ai, double af, double aref) {
  return (pow(af, -2.5) - pow(ai, -2.5)) * aref / Qfactor(c, aref) / (-2.5 * pow(aref, -3.5));
}
/* Quinn et al. time stepping of the non-COLA run (StdDA = 2, main.c:75-81):
 * SqStd = int_ai^af da / Q(a), SphiStd = int_ai^af a da / Q(a)
 * (src/cosmo.c:1165-1200) */
static double sqstd_integrand(double a, const void *par) { return 1.0 / Qfactor((const mgp_cosmo *)par, a); }
static double sphistd_integrand(double a, const void *par) { return a / Qfactor((const mgp_cosmo *)par, a); }
double mgp_cosmo_SqStd(const mgp_cosmo *c, double ai, double af) { return quad(sqstd_integrand, c, ai, af, 4); }
double mgp_cosmo_SphiStd(const mgp_cosmo *c, double ai, double af) { return quad(sphistd_integrand, c, ai, af, 4); }
/* main.c:400-455: the step in a (UseCOLA, stepDistr = 0) or in ln a
 * (stepDistr = 1 otherwise): da from A to a_out in nsteps, and AF (mid
 * point) / AFF (end) of the step starting at A */
double mgp_cosmo_step_da(const mgp_params *p, double A, double aout, int nsteps) {
  return p->UseCOLA ? (aout - A) / (double)nsteps : (log(aout) - log(A)) / (double)nsteps;
}
double mgp_cosmo_step_mid(const mgp_params *p, double A, double da) { return p->UseCOLA ? A + 0.5 * da : A * exp(0.5 * da); }
double mgp_cosmo_step_end(const mgp_params *p, double A, double da) { return p->UseCOLA ? A + da : A * exp(da); }
/* Kick and Drift coefficients of the run's StdDA (main.c:696-701, 751-757) */
double mgp_cosmo_kick_dda(const mgp_cosmo *c, double ai, double af, double a) {
  return c->p.UseCOLA ? mgp_cosmo_Sphi(c, ai, af, a) : mgp_cosmo_SphiStd(c, ai, af);
}
double mgp_cosmo_drift_dyyy(const mgp_cosmo *c, double a, double aff, double af) {
  return c->p.UseCOLA ? mgp_cosmo_Sq(c, a, aff, af) : mgp_cosmo_SqStd(c, a, aff);
}

/* -------------------------------------------------------- power spectrum */
/* Eisenstein & Hu no-wiggle transfer function (src/power.c:447-476). */
static double transfer_eh(const mgp_cosmo *c, double k) {
  const double h = c->p.HubbleParam, om = c->p.Omega;
  double ombh2 = c->p.OmegaBaryon * h * h;
  if (c->p.OmegaBaryon == 0) ombh2 = 0.04 * h * h;
  k *= 3.085678e24 / c->p.UnitLength_in_cm;
  double theta = 2.728 / 2.7, ommh2 = om * h * h;
  double s = 44.5 * log(9.83 / ommh2) / sqrt(1. + 10. * exp(0.75 * log(ombh2))) * h;
  double fb = ombh2 / ommh2;
  double alpha = 1. - 0.328 * log(431. * ommh2) * fb + 0.380 * log(22.3 * ommh2) * fb * fb;
  double gamma = (alpha + (1. - alpha) / (1. + exp(4 * log(0.43 * k * s)))) * om * h;
  double q = k * theta * theta / gamma;
  double L0 = log(2. * exp(1.) + 1.8 * q), C0 = 14.2 + 731. / (1. + 62.5 * q);
  return L0 / (L0 + C0 * q * q);
}

static double table_interp(const mgp_cosmo *c, double k) {
  double lk = log10(k * (c->p.InputSpectrum_UnitLength_in_cm / c->p.UnitLength_in_cm));
  if (c->ntab < 2 || lk < c->tab_logk[0] || lk > c->tab_logk[c->ntab - 1]) return 0.0;
  int lo = 0, hi = c->ntab - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (lk < c->tab_logk[mid]) hi = mid; else lo = mid;
  }
  double u = (lk - c->tab_logk[lo]) / (c->tab_logk[hi] - c->tab_logk[lo]);
  return pow(10.0, (1 - u) * c->tab_logv[lo] + u * c->tab_logv[hi]);
}

double mgp_cosmo_power(const mgp_cosmo *c, double k) {
  /* PowerSpec with MASSIVE_NEUTRINOS (src/power.c:376-379): the CDM+baryon
   * spectrum of the CAMB files */
  if (c->p.massive_neutrinos) return c->norm * nu_pofk_cb(c, k, c->OmegaCDM);
  switch (c->p.WhichSpectrum) {
    case 0: {
      double T = c->p.WhichTransfer == 1 ? table_interp(c, k) : transfer_eh(c, k);
      return c->norm * pow(k, c->p.PrimordialIndex) * T * T;
    }
    case 1: return c->norm * table_interp(c, k);
    default: {
      double T = transfer_eh(c, k);
      return c->norm * pow(k, c->p.PrimordialIndex) * T * T;
    }
  }
}

typedef struct { const mgp_cosmo *c; double R; } th_par;
static double sigma2_integrand(double k, const void *v) {
  const th_par *t = (const th_par *)v;
  double kr = t->R * k;
  if (kr < 1e-8) return 0.0;
  double w = 3 * (sin(kr) / (kr * kr * kr) - cos(kr) / (kr * kr));
  return k * k * w * w * mgp_cosmo_power(t->c, k);
}

static int read_table(mgp_cosmo *c, const char *fname, int transfer, char *err, size_t errlen) {
  FILE *fd = fopen(fname, "r");
  if (!fd) {
    snprintf(err, errlen, "can't read input %s in file '%s'", transfer ? "transfer function" : "power spectrum", fname);
    return MGP_EIO;
  }
  int cap = 1024, n = 0;
  double *lk = (double *)malloc(sizeof(double) * cap), *lv = (double *)malloc(sizeof(double) * cap);
  double k, v;
  while (fscanf(fd, " %lg %lg ", &k, &v) == 2) {
    if (n == cap) {
      cap *= 2;
      lk = (double *)realloc(lk, sizeof(double) * cap);
      lv = (double *)realloc(lv, sizeof(double) * cap);
    }
    lk[n] = log10(k);
    lv[n] = log10(v);
    n++;
  }
  fclose(fd);
  /* insertion sort by log k (src/power.c:337, 125) */
  for (int i = 1; i < n; i++) {
    double a = lk[i], b = lv[i];
    int j = i - 1;
    while (j >= 0 && lk[j] > a) { lk[j + 1] = lk[j]; lv[j + 1] = lv[j]; j--; }
    lk[j + 1] = a;
    lv[j + 1] = b;
  }
  if (transfer && n > 0) {
    double t0 = lv[0];
    for (int i = 0; i < n; i++) lv[i] -= t0; /* src/power.c:144-145 */
  }
  if (n < 2) {
    snprintf(err, errlen, "table '%s' has fewer than two rows", fname);
    free(lk); free(lv);
    return MGP_EIO;
  }
  c->ntab = n;
  c->tab_logk = lk;
  c->tab_logv = lv;
  return MGP_OK;
}

/* The raw LCDM growth factor: D_LCDM(k, a) of the neutrino build, else
 * D_LCDM(a) (cosmo.c:692-698, 741-745). */
static double lcdm_D(const mgp_cosmo *c, double k, double a) {
  if (!c->sd_lcdm.nx) return spline_eval(&c->DL, log(a));
  double *col = (double *)malloc(sizeof(double) * 2 * c->sd_lcdm.ny);
  bicubic_column(&c->sd_lcdm, log(a), col, col + c->sd_lcdm.ny);
  double d = column_eval(&c->sd_lcdm, col, col + c->sd_lcdm.ny, log(k));
  free(col);
  return d;
}

/* mg_pofk_ratio(k, a) (src/cosmo.c:688-706): (D/D_LCDM)^2 with the raw
 * (unnormalised) tables; D(k, a) in the scale-dependent build. */
double mgp_cosmo_pofk_ratio(const mgp_cosmo *c, double k, double a) {
  if (!c->p.modified_gravity_active) return 1.0;
  double D;
  if (c->sd) {
    const mgp_bicubic *b = &c->sd_tab[0];
    double *col = (double *)malloc(sizeof(double) * 2 * b->ny);
    bicubic_column(b, log(a), col, col + b->ny);
    D = column_eval(b, col, col + b->ny, log(k));
    free(col);
  } else {
    D = spline_eval(&c->D, log(a));
  }
  double r = D / lcdm_D(c, k, a);
  return r * r;
}
void mgp_cosmo_pofk_ratio_many(const mgp_cosmo *c, double a, int n, const double *k, double *out) {
  if (!c->p.modified_gravity_active) {
    for (int i = 0; i < n; i++) out[i] = 1.0;
    return;
  }
  double DL = spline_eval(&c->DL, log(a));
  if (!c->sd) {
    double r = spline_eval(&c->D, log(a)) / DL;
    for (int i = 0; i < n; i++) out[i] = r * r;
    return;
  }
  const mgp_bicubic *b = &c->sd_tab[0], *bl = &c->sd_lcdm;
  double *col = (double *)malloc(sizeof(double) * 2 * (b->ny + bl->ny));
  double *coll = col + 2 * b->ny;
  bicubic_column(b, log(a), col, col + b->ny);
  if (bl->nx) bicubic_column(bl, log(a), coll, coll + bl->ny);
  for (int i = 0; i < n; i++) {
    double r = column_eval(b, col, col + b->ny, log(k[i])) /
               (bl->nx ? column_eval(bl, coll, coll + bl->ny, log(k[i])) : DL);
    out[i] = r * r;
  }
  free(col);
}

/* mg_sigma8_enhancement(a) (src/cosmo.c:713-756): the ratio of growth
 * factors, or in the scale-dependent build the ratio of the sigma_8
 * integrals over 1000 log-spaced k in [1e-3, 100] h/Mpc. */
double mgp_cosmo_sigma8_enh(const mgp_cosmo *c, double a) {
  if (!c->p.modified_gravity_active) return 1.0;
  if (!c->sd) return spline_eval(&c->D, log(a)) / spline_eval(&c->DL, log(a));
  const double kmin = 0.001, kmax = 100.0;
  const int npts = 1000;
  const mgp_bicubic *b = &c->sd_tab[0];
  double *col = (double *)malloc(sizeof(double) * 2 * b->ny);
  bicubic_column(b, log(a), col, col + b->ny);
  double DL = spline_eval(&c->DL, log(a)), dlogk = log(kmax / kmin) / (double)(npts - 1), s = 0.0, sl = 0.0;
  for (int i = 0; i < npts; i++) {
    double k = exp(log(kmin) + log(kmax / kmin) * i / (double)(npts - 1)), kR8 = k * 8.0;
    double w = 3.0 / (kR8 * kR8 * kR8) * (sin(kR8) - kR8 * cos(kR8));
    double D = column_eval(b, col, col + b->ny, log(k)), pk = mgp_cosmo_power(c, k);
    double DLk = c->sd_lcdm.nx ? lcdm_D(c, k, a) : DL;
    s += pk * w * w * D * D * k * k * k * dlogk / (2.0 * M_PI * M_PI);
    sl += pk * w * w * DLk * DLk * k * k * k * dlogk / (2.0 * M_PI * M_PI);
  }
  free(col);
  return sqrt(s) / sqrt(sl);
}

/* ------------------------------------------------ Brans-Dicke background */
/* JBD_Solve_Background (src/jbd.c): y = ln(phi/phi0) and z over x = ln a
 * from z = 1e6 to a = 1 (10000 points), phi_ini found by bisection so that
 * phi(a=1) = phi0 to 1e-6; Geff/G = e^-y, H from the modified Friedmann
 * equation.  Integrated here with the Dormand-Prince pair. */
typedef struct { double w, om, orr, ov; } jbd_par;

static double jbd_H(const jbd_par *g, double x, double y, double dy) {
  return sqrt(exp(-y) * (g->orr * exp(-4 * x) + g->om * exp(-3 * x) + g->ov) / (1.0 + dy - g->w / 6 * dy * dy));
}
static double jbd_dHdx(const jbd_par *g, double x, double y, double dy) {
  double H = jbd_H(g, x, y, dy);
  double om = g->om * exp(-y - 3.0 * x) / (H * H), ov = g->ov * exp(-y) / (H * H);
  double ora = g->orr * exp(-y - 4.0 * x) / (H * H);
  return H / 2.0 * (-3.0 - ora - g->w / 2.0 * dy * dy + dy - 3.0 * (om + 4.0 * ov) / (3.0 + 2.0 * g->w) + 3.0 * ov);
}
static double jbd_H_of_z(const jbd_par *g, double x, double y, double z) {
  return sqrt(exp(-y) * (g->orr * exp(-4 * x) + g->om * exp(-3 * x) + g->ov) +
              z * z / 12.0 * (2.0 * g->w + 3.0) * exp(-2 * y - 6 * x)) -
         z / 2.0 * exp(-y - 3 * x);
}
static void jbd_rhs(const jbd_par *g, double x, const double *u, double *f) {
  double hubb = jbd_H_of_z(g, x, u[0], u[1]);
  f[0] = u[1] * exp(-u[0] - 3 * x) / hubb;
  f[1] = 3.0 * exp(3.0 * x) / (2 * g->w + 3) / hubb * (g->om * exp(-3 * x) + 4.0 * g->ov);
}
/* generic 2-component Dormand-Prince step driver */
static int dp45_2(const jbd_par *g, double x0, double x1, double *u, double *hguess) {
  double x = x0, h = *hguess;
  int steps = 0;
  while (x < x1) {
    if (x + h > x1) h = x1 - x;
    double k[7][2], ut[2], u5[2], err = 0.0;
    for (int s = 0; s < 7; s++) {
      for (int i = 0; i < 2; i++) {
        double acc = u[i];
        for (int j = 0; j < s; j++) acc += h * DP_A[s][j] * k[j][i];
        ut[i] = acc;
      }
      jbd_rhs(g, x + DP_C[s] * h, ut, k[s]);
    }
    for (int i = 0; i < 2; i++) {
      double s5 = u[i], s4 = u[i];
      for (int s = 0; s < 7; s++) { s5 += h * DP_B5[s] * k[s][i]; s4 += h * DP_B4[s] * k[s][i]; }
      u5[i] = s5;
      double sc = 1e-11 * (fabs(u[i]) > fabs(s5) ? fabs(u[i]) : fabs(s5)) + 1e-13;
      double e = fabs(s5 - s4) / sc;
      if (e > err) err = e;
    }
    if (err <= 1.0) { x += h; u[0] = u5[0]; u[1] = u5[1]; }
    double fac = err > 0 ? 0.9 * pow(err, -0.2) : 5.0;
    if (fac > 5.0) fac = 5.0;
    if (fac < 0.2) fac = 0.2;
    h *= fac;
    if (++steps > 10000000 || !(h > 1e-15)) return -1;
  }
  *hguess = h;
  return 0;
}

static int jbd_solve(mgp_cosmo *c, char *err, size_t errlen) {
  const int npts = 10000;
  jbd_par g = {c->p.wBD, c->p.Omegah2, c->p.Omegarh2, c->p.Omegavh2};
  double xini = log(1.0 / (1.0 + 1e6)), dx = (0.0 - xini) / (double)(npts - 1);
  double *x = (double *)malloc(sizeof(double) * npts * 4), *y = x + npts, *dy = y + npts, *t = dy + npts;
  double lo = 0.0, hi = 1.0;
  int ok = 0;
  for (int it = 0; it < 200; it++) {
    double phinow = 0.5 * (lo + hi), yi = log(phinow);
    double u[2] = {yi, jbd_H(&g, xini, yi, 0.0) * exp(3.0 * xini + yi) * 0.0}, h = 1e-4;
    x[0] = xini; y[0] = u[0]; dy[0] = u[1];
    int bad = 0;
    for (int i = 1; i < npts && !bad; i++) {
      double xn = xini + i * dx;
      if (dp45_2(&g, xini + (i - 1) * dx, xn, u, &h)) bad = 1;
      x[i] = xn;
      y[i] = u[0];
      dy[i] = u[1] / jbd_H_of_z(&g, xn, u[0], u[1]) * exp(-3.0 * xn - u[0]);
    }
    if (bad) break;
    double r = exp(y[npts - 1]);
    if (fabs(r - 1.0) < 1e-6) { ok = 1; break; }
    if (r < 1.0) lo = phinow; else hi = phinow;
  }
  if (!ok) {
    free(x);
    snprintf(err, errlen, "Brans-Dicke background: no phi_ini gives phi(a=1) = phi0");
    return MGP_ENUMERIC;
  }
  double h = jbd_H(&g, 0.0, y[npts - 1], dy[npts - 1]);
  double *G = (double *)malloc(sizeof(double) * npts * 3), *H = G + npts, *dH = H + npts;
  for (int i = 0; i < npts; i++) {
    G[i] = exp(-y[i]);
    H[i] = jbd_H(&g, x[i], y[i], dy[i]) / h;
    dH[i] = jbd_dHdx(&g, x[i], y[i], dy[i]) / h * exp(-x[i]);
  }
  spline_init(&c->jbdG, x, G, npts);
  spline_init(&c->jbdH, x, H, npts);
  spline_init(&c->jbddH, x, dH, npts);
  (void)t;
  free(x);
  free(G);
  c->have_jbd = 1;
  /* init_modified_version (user_defined_functions.h:135-143) */
  c->p.HubbleParam = h;
  c->p.Omega = c->p.Omegah2 / (h * h);
  return MGP_OK;
}

/* compute_phi_of_a (src/cosmo.c:104-190): phi(a) = int 9 Omega beta /
 * (m^2 a^3) dln a from z = max(200, z_init), then phi_crit = phi / (2 beta). */
static double phia_integrand(double x, const void *par) {
  const mgp_cosmo *c = (const mgp_cosmo *)par;
  double a = exp(x), beta = mgp_beta_of_a(c, a), m2 = mgp_mass2_of_a(c, a);
  if (beta == 0.0) return 0.0;
  return 9.0 * c->p.Omega * beta / (m2 * a * a * a);
}
static int phia_solve(mgp_cosmo *c) {
  const int npts = 1000;
  double zini = c->p.Init_Redshift > 200.0 ? c->p.Init_Redshift : 200.0;
  double xmin = log(1.0 / (1.0 + zini)), xmax = log(1.0 / (1.0 - 0.5)), dx = (xmax - xmin) / (double)(npts - 1);
  double *x = (double *)malloc(sizeof(double) * npts * 2), *ph = x + npts;
  x[0] = xmin;
  ph[0] = 0.0;
  for (int i = 1; i < npts; i++) {
    x[i] = xmin + i * dx;
    ph[i] = ph[i - 1] + quad(phia_integrand, c, xmin + (i - 1) * dx, x[i], 1);
  }
  for (int i = 0; i < npts; i++) {
    double b = mgp_beta_of_a(c, exp(x[i]));
    if (b != 0.0) ph[i] /= 2.0 * b;
  }
  spline_init(&c->phia, x, ph, npts);
  free(x);
  c->have_phia = 1;
  return MGP_OK;
}

int mgp_cosmo_init(mgp_cosmo *c, const mgp_params *p, char *err, size_t errlen) {
  return mgp_cosmo_init_hooks(c, p, NULL, err, errlen);
}

int mgp_cosmo_user_screening(const mgp_cosmo *c, int density) {
  return density ? c->hooks.screening_factor_density != NULL : c->hooks.screening_factor_potential != NULL;
}

int mgp_cosmo_init_hooks(mgp_cosmo *c, const mgp_params *p, const mgp_model_hooks *hooks, char *err, size_t errlen) {
  memset(c, 0, sizeof(*c));
  c->p = *p;
  if (hooks) c->hooks = *hooks;
  int rc;
  if (p->massive_neutrinos) {
    if (!p->scaledependent) {
      snprintf(err, errlen, "Massive neutrinos must be compiled with SCALEDEPENDENT");
      return MGP_EPARAM;
    }
    if ((rc = read_camb(c, err, errlen))) return rc;
    c->nu_rows0 = (double *)malloc(sizeof(double) * 8 * c->nuT[0].nx);
    nu_rows r0 = {0, c->nu_rows0};
    nu_rows_at(c, 1.0, &r0);
  } else if (p->WhichSpectrum == 1) {
    if ((rc = read_table(c, p->FileWithInputSpectrum, 0, err, errlen))) return rc;
  } else if (p->WhichSpectrum == 0 && p->WhichTransfer == 1) {
    if ((rc = read_table(c, p->FileWithInputTransfer, 1, err, errlen))) return rc;
  }
  /* Norm = sigma8^2 / sigma^2(R8) (src/power.c:226-257) */
  c->norm = 1.0;
  th_par t = {c, 8.0 * (3.085678e24 / p->UnitLength_in_cm)};
  double s2 = quad(sigma2_integrand, &t, 0.0, 500.0 / t.R, 256) / (2.0 * M_PI * M_PI);
  if (!(s2 > 0)) {
    snprintf(err, errlen, "sigma8 normalisation integral is not positive (%g)", s2);
    return MGP_ENUMERIC;
  }
  c->norm = p->Sigma8 * p->Sigma8 / s2;
  /* init_modified_version runs after initialize_powerspectrum in main.c
   * (main.c:153-162), so the normalisation above uses the file's Omega/h;
   * with massive neutrinos it also ran with Omega_cdm still 0, i.e. with
   * the baryon transfer function in place of the CDM+baryon one (kept) */
  if (p->massive_neutrinos) {
    /* init_modified_version (user_defined_functions.h:59-66) */
    c->OmegaNu = p->nu_SumMassNuEV / (93.14 * p->HubbleParam * p->HubbleParam);
    c->OmegaCDM = p->Omega - p->OmegaBaryon - c->OmegaNu;
    if (c->OmegaNu < 1e-6) {
      c->OmegaNu = 0.0;
      c->OmegaCDM = p->Omega - p->OmegaBaryon;
    }
    /* the growth equations see the neutrinos whenever OmegaNu survived the
     * cut (GeffoverG_neutrino_*, user_defined_functions.h:662-684); the
     * density is added only with nu_include_massive_neutrinos */
    c->nu_growth = c->OmegaNu > 0.0;
    c->nu = p->nu_include_massive_neutrinos && c->nu_growth;
  }
  if (p->model == MGP_MODEL_BRANSDICKE && (rc = jbd_solve(c, err, errlen))) return rc;
  if (p->model == MGP_MODEL_MBETA && p->modified_gravity_active) phia_solve(c);
  if ((rc = solve_growth(c, err, errlen))) return rc;
  if (p->massive_neutrinos && (rc = solve_growth_sd(c, 1, err, errlen))) return rc;
  if (p->scaledependent) return solve_growth_sd(c, 0, err, errlen);
  return MGP_OK;
}

void mgp_cosmo_free(mgp_cosmo *c) {
  mgp_spline *ex[4] = {&c->jbdH, &c->jbddH, &c->jbdG, &c->phia};
  for (int i = 0; i < 4; i++)
    if (ex[i]->x) spline_free(ex[i]);
  mgp_spline *sp[12] = {&c->D, &c->dDdy, &c->ddDddy, &c->D2, &c->dD2dy, &c->ddD2ddy,
                        &c->DL, &c->dDLdy, &c->ddDLddy, &c->D2L, &c->dD2Ldy, &c->ddD2Lddy};
  for (int i = 0; i < 12; i++)
    if (sp[i]->x) spline_free(sp[i]);
  if (c->sd)
    for (int f = 0; f < 6; f++) bicubic_free(&c->sd_tab[f]);
  c->sd = 0;
  if (c->sd_lcdm.nx) bicubic_free(&c->sd_lcdm);
  for (int q = 0; q < 4; q++)
    if (c->nuT[q].nx) bicubic_free(&c->nuT[q]);
  free(c->nu_rows0);
  c->nu_rows0 = NULL;
  free(c->tab_logk);
  free(c->tab_logv);
  c->tab_logk = c->tab_logv = NULL;
}

/* Host-only evaluation of the cosmology of a parameter set (no GPU needed):
 * which 0-6 as mgp_growth, 7 the linear power spectrum P(x) (x = k in h/Mpc).
 * Sq/Sphi are available through mgp_cosmo_coeff. */
int mgp_cosmo_eval(const mgp_params *p, int which, const double *x, int n, double *out) {
  if (which < 0 || which > 9) return mgp_set_error(MGP_EINVAL, "which = %d out of range", which);
  return mgp_cosmo_eval_hooks(p, NULL, which, x, n, out);
}

int mgp_cosmo_eval_hooks(const mgp_params *p, const mgp_model_hooks *hooks, int which, const double *x, int n,
                         double *out) {
  if (!p || which < 0 || which > 15) return mgp_set_error(MGP_EINVAL, "which = %d out of range", which);
  char err[512] = "";
  mgp_cosmo c;
  int rc = mgp_cosmo_init_hooks(&c, p, hooks, err, sizeof(err));
  if (rc) {
    mgp_cosmo_free(&c);
    return mgp_set_error(rc, "%s", err);
  }
  for (int i = 0; i < n; i++) {
    switch (which) {
      case 7: out[i] = mgp_cosmo_power(&c, x[i]); break;
      case 8: out[i] = mgp_cosmo_pofk_ratio(&c, x[i], 1.0); break;
      case 9: out[i] = mgp_cosmo_sigma8_enh(&c, x[i]); break;
      case 10: out[i] = mgp_hubble(&c, x[i]); break;
      case 11: out[i] = mgp_geff(&c, x[i], 0.1); break;
      case 12: out[i] = mgp_coupling(&c, x[i]); break;
      case 13: out[i] = mgp_mass2_of_a(&c, x[i]); break;
      case 14: out[i] = mgp_phicrit(&c, x[i]); break;
      case 15: out[i] = mgp_factor_2lpt(&c, x[i]); break;
      default: out[i] = mgp_cosmo_growth(&c, which, x[i]);
    }
  }
  mgp_cosmo_free(&c);
  return MGP_OK;
}

int mgp_growth_scaledependent(const mgp_params *p, int which, const double *k, const double *a, int n, double *out) {
  if (!p || !p->scaledependent) return mgp_set_error(MGP_EINVAL, "parameters without scaledependent = 1");
  if (which < 0 || which > 5) return mgp_set_error(MGP_EINVAL, "which = %d out of range", which);
  char err[512] = "";
  mgp_cosmo c;
  int rc = mgp_cosmo_init(&c, p, err, sizeof(err));
  if (rc) {
    mgp_cosmo_free(&c);
    return mgp_set_error(rc, "%s", err);
  }
  for (int i = 0; i < n; i++) out[i] = mgp_cosmo_growth_sd(&c, which, k[i], a[i]);
  mgp_cosmo_free(&c);
  return MGP_OK;
}

/* COLA coefficients for triples (ai, af, aref): kind 0 Sq, 1 Sphi. */
int mgp_cosmo_coeff(const mgp_params *p, int kind, const double *ai, const double *af, const double *aref, int n,
                    double *out) {
  if (kind < 0 || kind > 3) return mgp_set_error(MGP_EINVAL, "kind = %d out of range", kind);
  char err[512] = "";
  mgp_cosmo c;
  int rc = mgp_cosmo_init(&c, p, err, sizeof(err));
  if (rc) {
    mgp_cosmo_free(&c);
    return mgp_set_error(rc, "%s", err);
  }
  for (int i = 0; i < n; i++) {
    switch (kind) {
      case 0: out[i] = mgp_cosmo_Sq(&c, ai[i], af[i], aref[i]); break;
      case 1: out[i] = mgp_cosmo_Sphi(&c, ai[i], af[i], aref[i]); break;
      case 2: out[i] = mgp_cosmo_SqStd(&c, ai[i], af[i]); break;
      default: out[i] = mgp_cosmo_SphiStd(&c, ai[i], af[i]);
    }
  }
  mgp_cosmo_free(&c);
  return MGP_OK;
}

/* The neutrino term of the density at scale factor a (src/auxPM.c:383-428)
 * per integer |k|^2 (k = 2 pi/Box sqrt(rk)): Omega_nu/Omega N^3
 * T_nu(k, a) / T_cb(k, 1); out[0] unused.  Returns (Omega - Omega_nu)/Omega,
 * the factor of the CDM density, or 1 without neutrinos. */
void mgp_cosmo_nu_den(const mgp_cosmo *c, int N, int nrk, double *den) {
  (void)N;
  const nu_rows o1 = {c->nuT[0].nx, c->nu_rows0};
  den[0] = 1.0;
  for (int rk = 1; rk < nrk; rk++) den[rk] = nu_Tcb(c, &o1, 2.0 * M_PI / c->p.Box * sqrt((double)rk), c->OmegaCDM);
}

int mgp_cosmo_nu_row(const mgp_cosmo *c, double a, double *val, double *dval) {
  if (!c->nu) return 0;
  bicubic_row(&c->nuT[0], 1.0 / a - 1.0, val, dval);
  return c->nuT[0].nx;
}

const double *mgp_cosmo_nu_lnk(const mgp_cosmo *c, int *nx) {
  *nx = c->nu ? c->nuT[0].nx : 0;
  return c->nu ? c->nuT[0].x : NULL;
}
