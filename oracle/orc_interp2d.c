/*
 * Bicubic interpolation on a rectilinear grid, restated from the published
 * description of GSL's gsl_interp2d_bicubic (GSL >= 2.0 manual, "2D
 * Interpolation Types"): the partial derivatives z_x, z_y and z_xy at the
 * nodes come from natural cubic splines along the grid lines (z_x along x for
 * each y, z_y along y for each x, z_xy as the x-derivative of z_y), and each
 * cell is the tensor-product cubic Hermite polynomial of the four corners.
 *
 * TEST INFRASTRUCTURE ONLY: used by the oracle's scale-dependent growth tables
 * (src/cosmo.c:798-981 via Create_GSL_2D_Spline, src/wrappers.c:101-136) and
 * by the single-rank shim that stands in for GSL when the reference sources
 * are compiled here.  z is stored as z[j * nx + i] (src/wrappers.c:115-117).
 */
#include "orc.h"
#include <stdlib.h>
#include <string.h>

/* Node derivatives of the natural cubic spline through (x[s*i], y[s*i]),
 * i = 0..n-1 (strided input and output). */
static void spline_node_derivs(const double *x, const double *y, long ys, int n, double *d, long ds) {
  if (n < 2) {
    if (n == 1) d[0] = 0.0;
    return;
  }
  double *M = calloc(n, sizeof(double)), *u = calloc(n, sizeof(double));
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * M[i - 1] + 2.0;
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
  {
    double h = x[n - 1] - x[n - 2];
    d[(n - 1) * ds] = (y[(n - 1) * ys] - y[(n - 2) * ys]) / h + h * (M[n - 2] + 2.0 * M[n - 1]) / 6.0;
  }
  free(M);
  free(u);
}

void orc_bicubic_init(orc_bicubic *b, const double *x, const double *y, const double *z, int nx, int ny) {
  b->nx = nx;
  b->ny = ny;
  size_t nn = (size_t)nx * ny;
  b->x = malloc(sizeof(double) * nx);
  b->y = malloc(sizeof(double) * ny);
  b->z = malloc(sizeof(double) * nn);
  b->zx = malloc(sizeof(double) * nn);
  b->zy = malloc(sizeof(double) * nn);
  b->zxy = malloc(sizeof(double) * nn);
  memcpy(b->x, x, sizeof(double) * nx);
  memcpy(b->y, y, sizeof(double) * ny);
  memcpy(b->z, z, sizeof(double) * nn);
  for (int j = 0; j < ny; j++) spline_node_derivs(b->x, b->z + (size_t)j * nx, 1, nx, b->zx + (size_t)j * nx, 1);
  for (int i = 0; i < nx; i++) spline_node_derivs(b->y, b->z + i, nx, ny, b->zy + i, nx);
  for (int j = 0; j < ny; j++) spline_node_derivs(b->x, b->zy + (size_t)j * nx, 1, nx, b->zxy + (size_t)j * nx, 1);
}

void orc_bicubic_free(orc_bicubic *b) {
  free(b->x); free(b->y); free(b->z); free(b->zx); free(b->zy); free(b->zxy);
  memset(b, 0, sizeof(*b));
}

/* index i with x[i] <= v < x[i+1], the last cell for v = x[n-1] */
static int cell(const double *x, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int m = (lo + hi) / 2;
    if (x[m] > v) hi = m;
    else lo = m;
  }
  return lo;
}

double orc_bicubic_eval(const orc_bicubic *b, double xv, double yv) {
  int i = cell(b->x, b->nx, xv), j = cell(b->y, b->ny, yv);
  double dx = b->x[i + 1] - b->x[i], dy = b->y[j + 1] - b->y[j];
  double t = (xv - b->x[i]) / dx, u = (yv - b->y[j]) / dy;
  /* cubic Hermite basis: value at 0, value at 1, slope at 0, slope at 1 */
  double hx[4] = {(1 + 2 * t) * (1 - t) * (1 - t), t * t * (3 - 2 * t), t * (1 - t) * (1 - t), t * t * (t - 1)};
  double hy[4] = {(1 + 2 * u) * (1 - u) * (1 - u), u * u * (3 - 2 * u), u * (1 - u) * (1 - u), u * u * (u - 1)};
  double r = 0.0;
  for (int q = 0; q < 2; q++)
    for (int p = 0; p < 2; p++) {
      size_t c = (size_t)(j + q) * b->nx + (i + p);
      r += hx[p] * hy[q] * b->z[c] + hx[2 + p] * hy[q] * b->zx[c] * dx + hx[p] * hy[2 + q] * b->zy[c] * dy +
           hx[2 + p] * hy[2 + q] * b->zxy[c] * dx * dy;
    }
  return r;
}
