/* Stand-in for the GSL interfaces used by MG-PICOLA (reference test build only).
 * Written from the documented behaviour of each call; numerics are textbook
 * methods (Philox streams, adaptive Dormand-Prince, natural cubic splines,
 * Keys cubic convolution in 2D, adaptive Gauss-Legendre, bisection, the
 * Gauss hypergeometric series). */
#ifndef REF_SHIM_GSL_H
#define REF_SHIM_GSL_H
#include <math.h>
#include <stddef.h>
#define GSL_SUCCESS 0
#define GSL_CONTINUE (-2)
#define GSL_INTEG_GAUSS41 4
#define GSL_MAX(a, b) ((a) > (b) ? (a) : (b))
#define GSL_MIN(a, b) ((a) < (b) ? (a) : (b))
/* rng */
typedef struct { int id; } gsl_rng_type;
typedef struct { unsigned long seed; unsigned long long n; } gsl_rng;
extern const gsl_rng_type *gsl_rng_ranlxd1;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(gsl_rng *r, unsigned long seed);
double gsl_rng_uniform(gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
/* functions, integration */
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *w, double *result, double *abserr);
/* ode */
typedef struct {
  int (*function)(double t, const double y[], double dydt[], void *params);
  int (*jacobian)(double t, const double y[], double *dfdy, double dfdt[], void *params);
  size_t dimension;
  void *params;
} gsl_odeiv2_system;
typedef struct { int id; } gsl_odeiv2_step_type;
extern const gsl_odeiv2_step_type *gsl_odeiv2_step_rk2;
typedef struct { const gsl_odeiv2_system *sys; double h; double epsabs, epsrel; } gsl_odeiv2_driver;
gsl_odeiv2_driver *gsl_odeiv2_driver_alloc_y_new(const gsl_odeiv2_system *sys, const gsl_odeiv2_step_type *T,
                                                 double hstart, double epsabs, double epsrel);
int gsl_odeiv2_driver_apply(gsl_odeiv2_driver *d, double *t, double t1, double y[]);
void gsl_odeiv2_driver_free(gsl_odeiv2_driver *d);
/* splines */
typedef struct { int id; } gsl_interp_type;
typedef struct { int id; } gsl_interp2d_type;
extern const gsl_interp_type *gsl_interp_cspline;
extern const gsl_interp2d_type *gsl_interp2d_bicubic;
typedef struct { size_t cache; } gsl_interp_accel;
typedef struct { size_t n; double *x, *y, *y2; } gsl_spline;
typedef struct { size_t nx, ny; void *impl; } gsl_spline2d;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n);
int gsl_spline_init(gsl_spline *s, const double x[], const double y[], size_t n);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *T, size_t nx, size_t ny);
int gsl_spline2d_init(gsl_spline2d *s, const double x[], const double y[], const double z[], size_t nx, size_t ny);
double gsl_spline2d_eval(const gsl_spline2d *s, double x, double y, gsl_interp_accel *xa, gsl_interp_accel *ya);
void gsl_spline2d_free(gsl_spline2d *s);
/* roots */
typedef struct { int id; } gsl_root_fsolver_type;
typedef struct { gsl_function *f; double lo, hi, root; } gsl_root_fsolver;
extern const gsl_root_fsolver_type *gsl_root_fsolver_brent;
gsl_root_fsolver *gsl_root_fsolver_alloc(const gsl_root_fsolver_type *T);
int gsl_root_fsolver_set(gsl_root_fsolver *s, gsl_function *f, double lo, double hi);
int gsl_root_fsolver_iterate(gsl_root_fsolver *s);
double gsl_root_fsolver_root(const gsl_root_fsolver *s);
double gsl_root_fsolver_x_lower(const gsl_root_fsolver *s);
double gsl_root_fsolver_x_upper(const gsl_root_fsolver *s);
void gsl_root_fsolver_free(gsl_root_fsolver *s);
int gsl_root_test_interval(double lo, double hi, double epsabs, double epsrel);
/* special functions */
double gsl_sf_hyperg_2F1(double a, double b, double c, double x);
#endif
