/*
 * Single-rank implementations of the MPI, FFTW3 and GSL calls made by the
 * MG-PICOLA sources, so that the reference's own code can be compiled into a
 * test binary (oracle/_ref).  Test infrastructure only.
 *
 * Written from each call's documented semantics; none of the libraries'
 * code is reproduced.  Numerics: FFTs are the oracle's (oracle/orc_fft.c),
 * the random stream is the oracle's Philox stream (oracle/orc_rng.c), ODEs
 * are integrated with an adaptive Dormand-Prince 5(4) pair to 1e-12
 * (tighter than the tolerances the reference requests), quadrature is
 * adaptive Gauss-Legendre to 1e-13, splines are natural cubic, and 2D
 * interpolation is the bicubic method gsl_interp2d_bicubic documents (node
 * derivatives from natural cubic splines along the grid lines, Hermite
 * cells), restated in oracle/orc_interp2d.c.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3-mpi.h"
#include "gsl/ref_gsl.h"
#include "mpi.h"
#include "../orc.h"

/* ------------------------------------------------------------------ MPI */
static size_t user_type_size[64];
static int n_user_types = 0;
static size_t tsize(MPI_Datatype t) {
  switch (t) {
    case MPI_BYTE: return 1;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_DOUBLE: case MPI_LONG_LONG: case MPI_UNSIGNED_LONG_LONG: return 8;
    default:
      if (t >= MPI_SHIM_FIRST_USER && t < MPI_SHIM_FIRST_USER + n_user_types) return user_type_size[t - MPI_SHIM_FIRST_USER];
      return 1;
  }
}
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code ? code : 1); }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  if (s != MPI_IN_PLACE && n > 0) memcpy(r, s, (size_t)n * tsize(t));
  return 0;
}
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)root;
  return MPI_Allreduce(s, r, n, t, op, c);
}
int MPI_Allgather(const void *s, int ns, MPI_Datatype ts, void *r, int nr, MPI_Datatype tr, MPI_Comm c) {
  (void)nr; (void)tr; (void)c;
  if (s != MPI_IN_PLACE && ns > 0) memcpy(r, s, (size_t)ns * tsize(ts));
  return 0;
}
int MPI_Sendrecv(const void *s, int ns, MPI_Datatype ts, int dest, int stag, void *r, int nr, MPI_Datatype tr,
                 int src, int rtag, MPI_Comm c, MPI_Status *st) {
  (void)stag; (void)rtag; (void)c; (void)st;
  if (dest != 0 || src != 0) return 0; /* MPI_PROC_NULL on either side */
  size_t bs = (size_t)ns * tsize(ts), br = (size_t)nr * tsize(tr);
  size_t b = bs < br ? bs : br;
  if (b > 0 && s != r) memmove(r, s, b);
  return 0;
}
int MPI_Type_match_size(int typeclass, int size, MPI_Datatype *t) {
  (void)typeclass;
  *t = size == 4 ? MPI_FLOAT : MPI_DOUBLE;
  return 0;
}
int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *off, const MPI_Datatype *types, MPI_Datatype *t) {
  size_t ext = 0;
  for (int i = 0; i < n; i++) {
    size_t e = (size_t)off[i] + (size_t)bl[i] * tsize(types[i]);
    if (e > ext) ext = e;
  }
  user_type_size[n_user_types] = ext;
  *t = MPI_SHIM_FIRST_USER + n_user_types++;
  return 0;
}
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }

/* ---------------------------------------------------------------- FFTW */
struct ref_fftw_plan_s { int dir, N; double *in, *out; };
void fftw_mpi_init(void) {}
void fftw_mpi_cleanup(void) {}
ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm c, ptrdiff_t *ln0, ptrdiff_t *s0) {
  (void)c;
  *ln0 = n0;
  *s0 = 0;
  return n0 * n1 * n2;
}
static fftw_plan mkplan(int dir, ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double *in, double *out) {
  if (n0 != n1 || n0 != n2) { fprintf(stderr, "ref shim: cubic FFTs only\n"); exit(1); }
  fftw_plan p = malloc(sizeof(*p));
  p->dir = dir; p->N = (int)n0; p->in = in; p->out = out;
  return p;
}
fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double *in, fftw_complex *out, MPI_Comm c,
                                   unsigned flags) {
  (void)c; (void)flags;
  return mkplan(-1, n0, n1, n2, in, (double *)out);
}
fftw_plan fftw_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftw_complex *in, double *out, MPI_Comm c,
                                   unsigned flags) {
  (void)c; (void)flags;
  return mkplan(+1, n0, n1, n2, (double *)in, out);
}
void fftw_execute(const fftw_plan p) {
  size_t n = (size_t)p->N * p->N * 2 * (p->N / 2 + 1);
  if (p->in != p->out) memcpy(p->out, p->in, sizeof(double) * n);
  if (p->dir < 0) orc_fft_r2c(p->N, p->out);
  else orc_fft_c2r(p->N, p->out);
}
void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ------------------------------------------------------------------ rng */
static const gsl_rng_type ranlx_t = {1};
const gsl_rng_type *gsl_rng_ranlxd1 = &ranlx_t;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) { (void)T; return calloc(1, sizeof(gsl_rng)); }
void gsl_rng_set(gsl_rng *r, unsigned long seed) { r->seed = seed; r->n = 0; }
double gsl_rng_uniform(gsl_rng *r) { return orc_stream_uniform((uint32_t)r->seed, r->n++); }
void gsl_rng_free(gsl_rng *r) { free(r); }

/* ------------------------------------------------------------ quadrature */
static double glx[10], glw[10];
static int gl_ok = 0;
static void gl_init(void) {
  if (gl_ok) return;
  for (int i = 0; i < 10; i++) {
    double x = cos(M_PI * (i + 0.75) / 20.5), dp = 1.0;
    for (int it = 0; it < 60; it++) {
      double p0 = 1.0, p1 = x;
      for (int n = 2; n <= 20; n++) { double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n; p0 = p1; p1 = p2; }
      dp = 20 * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    glx[i] = x;
    glw[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  gl_ok = 1;
}
static double gl20(const gsl_function *f, double a, double b) {
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0;
  for (int i = 0; i < 10; i++) s += glw[i] * (f->function(c - h * glx[i], f->params) + f->function(c + h * glx[i], f->params));
  return s * h;
}
static double adapt(const gsl_function *f, double a, double b, double whole, double tol, int depth) {
  double c = 0.5 * (a + b), l = gl20(f, a, c), r = gl20(f, c, b);
  if (depth >= 16 || fabs(l + r - whole) <= tol) return l + r;
  return adapt(f, a, c, l, 0.5 * tol, depth + 1) + adapt(f, c, b, r, 0.5 * tol, depth + 1);
}
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  gsl_integration_workspace *w = malloc(sizeof(*w));
  w->limit = n;
  return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *w, double *result, double *abserr) {
  (void)epsabs; (void)epsrel; (void)limit; (void)key; (void)w;
  gl_init();
  const int panels = 64;
  double est[64], tot = 0, s = 0;
  for (int i = 0; i < panels; i++) {
    est[i] = gl20(f, a + (b - a) * i / panels, a + (b - a) * (i + 1) / panels);
    tot += fabs(est[i]);
  }
  double tol = 1e-13 * tot / panels + 1e-300;
  for (int i = 0; i < panels; i++) s += adapt(f, a + (b - a) * i / panels, a + (b - a) * (i + 1) / panels, est[i], tol, 0);
  *result = s;
  *abserr = tol * panels;
  return GSL_SUCCESS;
}

/* ------------------------------------------------------------------ ODE */
static const gsl_odeiv2_step_type rk2_t = {2};
const gsl_odeiv2_step_type *gsl_odeiv2_step_rk2 = &rk2_t;
gsl_odeiv2_driver *gsl_odeiv2_driver_alloc_y_new(const gsl_odeiv2_system *sys, const gsl_odeiv2_step_type *T,
                                                 double hstart, double epsabs, double epsrel) {
  (void)T;
  gsl_odeiv2_driver *d = malloc(sizeof(*d));
  d->sys = sys; d->h = hstart; d->epsabs = epsabs; d->epsrel = epsrel;
  return d;
}
void gsl_odeiv2_driver_free(gsl_odeiv2_driver *d) { free(d); }
static const double C_[7] = {0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1, 1};
static const double A_[7][6] = {{0}, {1.0 / 5}, {3.0 / 40, 9.0 / 40}, {44.0 / 45, -56.0 / 15, 32.0 / 9},
                                {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729},
                                {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656},
                                {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
static const double B5[7] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0};
static const double B4[7] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};
int gsl_odeiv2_driver_apply(gsl_odeiv2_driver *d, double *t, double t1, double y[]) {
  const size_t n = d->sys->dimension;
  double k[7][8], yt[8], y5[8];
  double x = *t, h = d->h > 0 ? d->h : 1e-6;
  if (h < 1e-6) h = 1e-6;
  int steps = 0;
  while (x < t1) {
    if (x + h > t1) h = t1 - x;
    for (int s = 0; s < 7; s++) {
      for (size_t i = 0; i < n; i++) {
        double acc = y[i];
        for (int j = 0; j < s; j++) acc += h * A_[s][j] * k[j][i];
        yt[i] = acc;
      }
      d->sys->function(x + C_[s] * h, yt, k[s], d->sys->params);
    }
    double err = 0.0;
    for (size_t i = 0; i < n; i++) {
      double s5 = y[i], s4 = y[i];
      for (int s = 0; s < 7; s++) { s5 += h * B5[s] * k[s][i]; s4 += h * B4[s] * k[s][i]; }
      y5[i] = s5;
      double sc = 1e-12 * fmax(fabs(y[i]), fabs(s5)) + 1e-14;
      double e = fabs(s5 - s4) / sc;
      if (e > err) err = e;
    }
    if (err <= 1.0) { x += h; memcpy(y, y5, sizeof(double) * n); }
    double fac = err > 0 ? 0.9 * pow(err, -0.2) : 5.0;
    h *= fac > 5.0 ? 5.0 : (fac < 0.2 ? 0.2 : fac);
    if (++steps > 50000000 || !(h > 1e-16)) return -1;
  }
  d->h = h;
  *t = t1;
  return GSL_SUCCESS;
}

/* -------------------------------------------------------------- splines */
static const gsl_interp_type cspline_t = {1};
static const gsl_interp2d_type bicubic_t = {2};
const gsl_interp_type *gsl_interp_cspline = &cspline_t;
const gsl_interp2d_type *gsl_interp2d_bicubic = &bicubic_t;
gsl_interp_accel *gsl_interp_accel_alloc(void) { return calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n) {
  (void)T;
  gsl_spline *s = calloc(1, sizeof(*s));
  s->n = n;
  s->x = malloc(8 * n); s->y = malloc(8 * n); s->y2 = calloc(n, 8);
  return s;
}
int gsl_spline_init(gsl_spline *s, const double x[], const double y[], size_t n) {
  memcpy(s->x, x, 8 * n); memcpy(s->y, y, 8 * n);
  double *u = calloc(n, 8);
  s->y2[0] = 0.0;
  for (size_t i = 1; i + 1 < n; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]), p = sig * s->y2[i - 1] + 2.0;
    s->y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  s->y2[n - 1] = 0.0;
  for (long kk = (long)n - 2; kk >= 0; kk--) s->y2[kk] = s->y2[kk] * s->y2[kk + 1] + u[kk];
  free(u);
  return GSL_SUCCESS;
}
static size_t find_lo(const double *x, size_t n, double v) {
  size_t lo = 0, hi = n - 1;
  while (hi - lo > 1) { size_t m = (lo + hi) / 2; if (x[m] > v) hi = m; else lo = m; }
  return lo;
}
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) {
  (void)a;
  size_t lo = find_lo(s->x, s->n, x), hi = lo + 1;
  double h = s->x[hi] - s->x[lo], A = (s->x[hi] - x) / h, B = (x - s->x[lo]) / h;
  return A * s->y[lo] + B * s->y[hi] + ((A * A * A - A) * s->y2[lo] + (B * B * B - B) * s->y2[hi]) * h * h / 6.0;
}
void gsl_spline_free(gsl_spline *s) { if (!s) return; free(s->x); free(s->y); free(s->y2); free(s); }
/* gsl_interp2d_bicubic: the oracle's restatement (oracle/orc_interp2d.c) */
gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *T, size_t nx, size_t ny) {
  (void)T;
  gsl_spline2d *s = calloc(1, sizeof(*s));
  s->nx = nx; s->ny = ny;
  s->impl = calloc(1, sizeof(orc_bicubic));
  return s;
}
int gsl_spline2d_init(gsl_spline2d *s, const double x[], const double y[], const double z[], size_t nx, size_t ny) {
  orc_bicubic_init((orc_bicubic *)s->impl, x, y, z, (int)nx, (int)ny);
  return GSL_SUCCESS;
}
double gsl_spline2d_eval(const gsl_spline2d *s, double x, double y, gsl_interp_accel *xa, gsl_interp_accel *ya) {
  (void)xa; (void)ya;
  return orc_bicubic_eval((const orc_bicubic *)s->impl, x, y);
}
void gsl_spline2d_free(gsl_spline2d *s) {
  if (!s) return;
  orc_bicubic_free((orc_bicubic *)s->impl);
  free(s->impl);
  free(s);
}

/* ---------------------------------------------------------------- roots */
static const gsl_root_fsolver_type brent_t = {3};
const gsl_root_fsolver_type *gsl_root_fsolver_brent = &brent_t;
gsl_root_fsolver *gsl_root_fsolver_alloc(const gsl_root_fsolver_type *T) { (void)T; return calloc(1, sizeof(gsl_root_fsolver)); }
int gsl_root_fsolver_set(gsl_root_fsolver *s, gsl_function *f, double lo, double hi) {
  s->f = f; s->lo = lo; s->hi = hi; s->root = 0.5 * (lo + hi);
  return GSL_SUCCESS;
}
int gsl_root_fsolver_iterate(gsl_root_fsolver *s) {
  /* bisection step */
  double m = 0.5 * (s->lo + s->hi);
  double fl = s->f->function(s->lo, s->f->params), fm = s->f->function(m, s->f->params);
  if ((fl < 0) == (fm < 0)) s->lo = m; else s->hi = m;
  s->root = 0.5 * (s->lo + s->hi);
  return GSL_SUCCESS;
}
double gsl_root_fsolver_root(const gsl_root_fsolver *s) { return s->root; }
double gsl_root_fsolver_x_lower(const gsl_root_fsolver *s) { return s->lo; }
double gsl_root_fsolver_x_upper(const gsl_root_fsolver *s) { return s->hi; }
void gsl_root_fsolver_free(gsl_root_fsolver *s) { free(s); }
int gsl_root_test_interval(double lo, double hi, double epsabs, double epsrel) {
  double tol = epsabs + epsrel * fmin(fabs(lo), fabs(hi));
  return fabs(hi - lo) < tol ? GSL_SUCCESS : GSL_CONTINUE;
}

/* ------------------------------------------------------ special function */
double gsl_sf_hyperg_2F1(double a, double b, double c, double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 0; n < 2000000; n++) {
    term *= (a + n) * (b + n) / ((c + n) * (n + 1.0)) * x;
    sum += term;
    if (fabs(term) < 1e-17 * fabs(sum)) break;
  }
  return sum;
}
