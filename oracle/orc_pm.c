/*
 * Oracle particle-mesh routines (test infrastructure only).
 * Each function restates one reference routine in double precision with the
 * same loop structure and operation order; file:line citations are relative
 * to the MG-PICOLA-PUBLIC tree.
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define PI 3.14159265358979323846 /* src/vars.h:59 */

static inline size_t ridx(int N, unsigned ix, unsigned iy, unsigned iz) {
  return ((size_t)ix * N + iy) * (size_t)(2 * (N / 2 + 1)) + iz;
}

/* src/auxPM.c:649-663 (double build) */
double orc_periodic_wrap(double x, double box) {
  while (x >= box) x -= box;
  while (x < 0) x += box;
  if (x == box) x = 0.0;
  return x;
}

void orc_lattice_positions(const double *disp, int Ns, double box, double *pos) {
  long np = (long)Ns * Ns * Ns;
  for (long p = 0; p < np; p++) {
    long i = p / ((long)Ns * Ns), j = (p / Ns) % Ns, k = p % Ns;
    pos[3 * p + 0] = orc_periodic_wrap(i * (box / (double)Ns) + disp[3 * p + 0], box);
    pos[3 * p + 1] = orc_periodic_wrap(j * (box / (double)Ns) + disp[3 * p + 1], box);
    pos[3 * p + 2] = orc_periodic_wrap(k * (box / (double)Ns) + disp[3 * p + 2], box);
  }
}

/* PtoMesh, src/auxPM.c:280-357, with the reference's parallel shape: the
 * mesh is split into x slabs, one per thread as one per MPI task; the
 * particles are handed to the slab of their cell (the exchange of
 * auxPM.c:108-275), each thread deposits its particles in particle order into
 * its slab plus one ghost x-slice, and the ghost slices are then added onto
 * the next slab's first slice (auxPM.c:350-356; the last one wraps to 0). */
static void deposit_one(double *d, int N, double X, double Y, double Z, double WPAR, size_t ghost_row,
                        double *ghost) {
  unsigned IX = (unsigned)X, IY = (unsigned)Y, IZ = (unsigned)Z;
  double DX = X - (double)IX, DY = Y - (double)IY, DZ = Z - (double)IZ;
  double TX = 1.0 - DX, TY = 1.0 - DY, TZ = 1.0 - DZ;
  DY *= WPAR;
  TY *= WPAR;
  if (IX >= (unsigned)N) IX -= N; /* X == N from rounding at the box edge: slice N is slice 0 */
  if (IY >= (unsigned)N) IY = 0;
  if (IZ >= (unsigned)N) IZ = 0;
  unsigned IXn = IX + 1, IYn = IY + 1, IZn = IZ + 1;
  if (IYn >= (unsigned)N) IYn = 0;
  if (IZn >= (unsigned)N) IZn = 0;
  d[ridx(N, IX, IY, IZ)] += TX * TY * TZ;
  d[ridx(N, IX, IY, IZn)] += TX * TY * DZ;
  d[ridx(N, IX, IYn, IZ)] += TX * DY * TZ;
  d[ridx(N, IX, IYn, IZn)] += TX * DY * DZ;
  /* the next x slice: in this slab, or this thread's ghost slice */
  double *dn = IXn == ghost_row ? ghost : d + ridx(N, IXn, 0, 0);
  dn[ridx(N, 0, IY, IZ)] += DX * TY * TZ;
  dn[ridx(N, 0, IY, IZn)] += DX * TY * DZ;
  dn[ridx(N, 0, IYn, IZ)] += DX * DY * TZ;
  dn[ridx(N, 0, IYn, IZn)] += DX * DY * DZ;
}

void orc_cic(const double *pos, long np, int N, int Ns, double box, double *grid) {
  const size_t P = 2 * (size_t)(N / 2 + 1);
  const size_t slice = (size_t)N * P;
  const double scaleBox = (double)N / box;
  const double WPAR = pow((double)N / (double)Ns, 3);
  int nt = omp_get_max_threads();
  if (nt > N) nt = N;
  if (nt < 1) nt = 1;
  /* slab of every x slice, and the particles of every slab in particle order */
  int *slab_of = malloc(sizeof(int) * N);
  for (int t = 0; t < nt; t++)
    for (int x = (int)((long)N * t / nt); x < (int)((long)N * (t + 1) / nt); x++) slab_of[x] = t;
  long *count = calloc(nt + 1, sizeof(long));
  int *owner = malloc(sizeof(int) * (np > 0 ? np : 1));
  for (long i = 0; i < np; i++) {
    unsigned IX = (unsigned)(pos[3 * i] * scaleBox);
    if (IX >= (unsigned)N) IX -= N; /* as deposit_one */
    owner[i] = slab_of[IX];
    count[owner[i] + 1]++;
  }
  for (int t = 0; t < nt; t++) count[t + 1] += count[t];
  long *list = malloc(sizeof(long) * (np > 0 ? np : 1)), *fillp = malloc(sizeof(long) * nt);
  memcpy(fillp, count, sizeof(long) * nt);
  for (long i = 0; i < np; i++) list[fillp[owner[i]]++] = i;
  double *ghost = malloc(sizeof(double) * slice * nt);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    const int x0 = (int)((long)N * t / nt), x1 = (int)((long)N * (t + 1) / nt);
    for (size_t c = (size_t)x0 * slice; c < (size_t)x1 * slice; c++) grid[c] = -1.0;
    double *g = ghost + (size_t)t * slice;
    for (size_t c = 0; c < slice; c++) g[c] = 0.0;
    for (long n = count[t]; n < count[t + 1]; n++) {
      long i = list[n];
      double X = pos[3 * i + 0] * scaleBox, Y = pos[3 * i + 1] * scaleBox, Z = pos[3 * i + 2] * scaleBox;
      deposit_one(grid, N, X, Y, Z, WPAR, (size_t)x1, g);
    }
  }
  /* ghost slices onto the next slab's first slice, in slab order */
  if (np != 0)
    for (int t = 0; t < nt; t++) {
      const int x1 = (int)((long)N * (t + 1) / nt);
      double *dst = grid + (size_t)(x1 == N ? 0 : x1) * slice;
      const double *g = ghost + (size_t)t * slice;
      for (size_t c = 0; c < slice; c++) dst[c] += g[c];
    }
  free(slab_of); free(count); free(owner); free(list); free(fillp); free(ghost);
}

/* Forces, src/auxPM.c:437-535. */
void orc_forces_kspace(const double *deltak, const double *mgk, int N, double box,
                       double *f1, double *f2, double *f3) {
  const int NH = N / 2 + 1;
  const double Scale = 2. * M_PI / box;
  const size_t Total = (size_t)N * N * NH;
  double *P3D = malloc(sizeof(double) * 2 * Total);
  memcpy(P3D, deltak, sizeof(double) * 2 * Total);
  if (mgk)
    for (size_t i = 0; i < Total; i++) { P3D[2 * i] += mgk[2 * i]; P3D[2 * i + 1] += mgk[2 * i + 1]; }
  const double N3 = pow((double)N, 3);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++) {
    int iglobal = i;
    for (int j = 0; j < NH; j++) {
      int kmin = 0;
      if (iglobal == 0 && j == 0) {
        f1[0] = f1[1] = f2[0] = f2[1] = f3[0] = f3[1] = 0.0;
        kmin = 1;
      }
      for (int k = kmin; k < NH; k++) {
        int dd[3];
        size_t ind = ((size_t)i * N + j) * NH + k;
        dd[0] = iglobal > N / 2 ? iglobal - N : iglobal;
        dd[1] = j;
        dd[2] = k;
        double RK = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
        double KK = -1.0 / RK, grid_corr = 1.0;
        double dens0 = (P3D[2 * ind] * KK * grid_corr) / N3;
        double dens1 = (-1.0 * P3D[2 * ind + 1] * KK * grid_corr) / N3;
        f1[2 * ind] = dens1 * dd[0] / Scale; f1[2 * ind + 1] = dens0 * dd[0] / Scale;
        f2[2 * ind] = dens1 * dd[1] / Scale; f2[2 * ind + 1] = dens0 * dd[1] / Scale;
        f3[2 * ind] = dens1 * dd[2] / Scale; f3[2 * ind + 1] = dens0 * dd[2] / Scale;
        if (j != N / 2 && j != 0) {
          size_t ind2 = ((size_t)i * N + (N - j)) * NH + k;
          dd[1] = -j;
          dens0 = (P3D[2 * ind2] * KK * grid_corr) / N3;
          dens1 = (-1.0 * P3D[2 * ind2 + 1] * KK * grid_corr) / N3;
          f1[2 * ind2] = dens1 * dd[0] / Scale; f1[2 * ind2 + 1] = dens0 * dd[0] / Scale;
          f2[2 * ind2] = dens1 * dd[1] / Scale; f2[2 * ind2 + 1] = dens0 * dd[1] / Scale;
          f3[2 * ind2] = dens1 * dd[2] / Scale; f3[2 * ind2 + 1] = dens0 * dd[2] / Scale;
        }
      }
    }
  }
  free(P3D);
}

/* MtoParticles, src/auxPM.c:560-644 (single task: x ghost slice = slice 0). */
void orc_interp(const double *f1, const double *f2, const double *f3, int N, double box,
                const double *pos, long np, double *disp, double mean_out[3]) {
  const double scaleBox = (double)N / box;
  const double *F[3] = {f1, f2, f3};
  const int nt = omp_get_max_threads();
  double *part = calloc(3 * (size_t)nt, sizeof(double));
  /* particles in nt contiguous ranges; the sums of the ranges are added in
   * range order, so the mean does not depend on scheduling */
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    double sum[3] = {0, 0, 0};
    for (long i = np * t / nt; i < np * (t + 1) / nt; i++) {
      double X = pos[3 * i] * scaleBox, Y = pos[3 * i + 1] * scaleBox, Z = pos[3 * i + 2] * scaleBox;
      unsigned IX = (unsigned)X, IY = (unsigned)Y, IZ = (unsigned)Z;
      double DX = X - (double)IX, DY = Y - (double)IY, DZ = Z - (double)IZ;
      double TX = 1.0 - DX, TY = 1.0 - DY, TZ = 1.0 - DZ;
      if (IY >= (unsigned)N) IY = 0;
      if (IZ >= (unsigned)N) IZ = 0;
      unsigned IXn = IX + 1, IYn = IY + 1, IZn = IZ + 1;
      if (IYn >= (unsigned)N) IYn = 0;
      if (IZn >= (unsigned)N) IZn = 0;
      /* ghost slice N holds slice 0 (auxPM.c:546-551) */
      if (IX >= (unsigned)N) IX -= N;
      if (IXn >= (unsigned)N) IXn -= N;
      for (int a = 0; a < 3; a++) {
        const double *G = F[a];
        double v = G[ridx(N, IX, IY, IZ)] * TX * TY * TZ + G[ridx(N, IX, IY, IZn)] * TX * TY * DZ +
                   G[ridx(N, IX, IYn, IZ)] * TX * DY * TZ + G[ridx(N, IX, IYn, IZn)] * TX * DY * DZ +
                   G[ridx(N, IXn, IY, IZ)] * DX * TY * TZ + G[ridx(N, IXn, IY, IZn)] * DX * TY * DZ +
                   G[ridx(N, IXn, IYn, IZ)] * DX * DY * TZ + G[ridx(N, IXn, IYn, IZn)] * DX * DY * DZ;
        disp[3 * i + a] = v;
        sum[a] += v;
      }
    }
    for (int a = 0; a < 3; a++) part[3 * t + a] = sum[a];
  }
  double sum[3] = {0, 0, 0};
  for (int t = 0; t < nt; t++)
    for (int a = 0; a < 3; a++) sum[a] += part[3 * t + a];
  free(part);
  for (int a = 0; a < 3; a++) mean_out[a] = sum[a] / (double)np;
}

/* Kick, src/main.c:688-742 (non-SCALEDEPENDENT branch 721-733). */
void orc_kick(long np, double *vel, double *disp, const double *D1, const double *D2,
              const double sumD[3], double omega, double dda, double ddD, double ddD2,
              double A, int usecola, double sumv_out[3]) {
  const int nt = omp_get_max_threads();
  double *part = calloc(3 * (size_t)nt, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    double sumxyz[3] = {0, 0, 0};
    for (long n = np * t / nt; n < np * (t + 1) / nt; n++) {
      for (int ax = 0; ax < 3; ax++) {
        disp[3 * n + ax] -= sumD[ax];
        double force = -1.5 * omega * disp[3 * n + ax] - usecola * (D1[3 * n + ax] * ddD + D2[3 * n + ax] * ddD2) / A;
        vel[3 * n + ax] += force * dda;
        sumxyz[ax] += vel[3 * n + ax];
      }
    }
    for (int ax = 0; ax < 3; ax++) part[3 * t + ax] = sumxyz[ax];
  }
  double sumxyz[3] = {0, 0, 0};
  for (int t = 0; t < nt; t++)
    for (int ax = 0; ax < 3; ax++) sumxyz[ax] += part[3 * t + ax];
  free(part);
  for (int ax = 0; ax < 3; ax++) sumv_out[ax] = sumxyz[ax] / (double)np;
}

/* Drift, src/main.c:747-787 (non-SCALEDEPENDENT branch 772-783). */
void orc_drift(long np, double *pos, const double *vel, const double *D1, const double *D2,
               const double sumv[3], double dyyy, double dD, double dD2, int usecola, double box) {
#pragma omp parallel for schedule(static)
  for (long n = 0; n < np; n++) {
    for (int ax = 0; ax < 3; ax++) {
      pos[3 * n + ax] += (vel[3 * n + ax] - sumv[ax]) * dyyy;
      pos[3 * n + ax] = orc_periodic_wrap(pos[3 * n + ax] + usecola * (D1[3 * n + ax] * dD + D2[3 * n + ax] * dD2), box);
    }
  }
}

/* adjust_pofk_parameters, src/compute_pofk.c:758-805 (integer k units). */
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

/* pofk_bin_index, src/compute_pofk.c:30-46 */
static int pofk_bin_index(double kmag, double kmin, double kmax, int nbins, int bintype) {
  if (bintype == 0) return (int)((kmag - kmin) / (kmax - kmin) * nbins + 0.5);
  if (bintype == 1) {
    if (kmag <= 0.0) return -1;
    return (int)(log(kmag / kmin) / log(kmax / kmin) * nbins + 0.5);
  }
  return 0;
}

/* k_from_index, src/compute_pofk.c:51-64 */
static double k_from_index(int index, double kmin, double kmax, int nbins, int bintype, double box) {
  if (bintype == 0) return (kmin + (kmax - kmin) / (double)nbins * index) * 2.0 * M_PI / box;
  if (bintype == 1) return exp(log(kmin) + log(kmax / kmin) / (double)nbins * index) * 2.0 * M_PI / box;
  return 0.0;
}

/* Shared mode loop of compute_power_spectrum / bin_up_RSD_power_spectrum
 * (compute_pofk.c:123-223 and 575-690). */
static void bin_modes_rows(const double *dk, int N, int i0, int i1, double kmin, double kmax, int nbins,
                           int bintype, double *p0, double *p2, double *p4, double *kb, double *nb) {
  const int NH = N / 2 + 1;
  const double norm = 1.0 / pow((double)N, 6);
  for (int i = i0; i < i1; i++) {
    int d0 = i > N / 2 ? N - i : i;
    double gx = d0 == 0 ? 1.0 : sin((PI * d0) / (double)N) / ((PI * d0) / (double)N);
    for (int j = 0; j < NH; j++) {
      int d1 = j;
      double gy = d1 == 0 ? 1.0 : sin((PI * d1) / (double)N) / ((PI * d1) / (double)N);
      for (int pass = 0; pass < 3; pass++) {
        int kz_lo, kz_hi;
        double w;
        if (pass == 0) { kz_lo = 0; kz_hi = 1; w = 1.0; }
        else if (pass == 1) { kz_lo = N / 2; kz_hi = N / 2 + 1; w = 1.0; }
        else { kz_lo = 1; kz_hi = N / 2; w = 2.0; }
        for (int k = kz_lo; k < kz_hi; k++) {
          int d2 = k;
          double gz;
          if (pass == 0) gz = 1.0;
          else if (pass == 1) gz = 2.0 / PI;
          else gz = sin((PI * d2) / (double)N) / ((PI * d2) / (double)N);
          double kmag = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
          double mu2;
          if (pass == 0) { mu2 = d2 * d2 / (kmag * kmag); if (i == 0 && j == 0) mu2 = 0.0; }
          else mu2 = (d2 * d2 / kmag / kmag);
          int nk = pofk_bin_index(kmag, kmin, kmax, nbins, bintype);
          if (nk >= 0 && nk < nbins) {
            double gc = 1.0 / pow(gx * gy * gz, 4.0) * norm;
            for (int mir = 0; mir < 2; mir++) {
              int jj = j;
              if (mir == 1) {
                if (!(j != N / 2 && j != 0)) break;
                jj = N - j;
              }
              size_t c = ((size_t)i * N + jj) * NH + d2;
              double pk = (dk[2 * c] * dk[2 * c] + dk[2 * c + 1] * dk[2 * c + 1]) * gc;
              p0[nk] += w * pk;
              if (p2) p2[nk] += w * pk * mu2;
              if (p4) p4[nk] += w * pk * mu2 * mu2;
              kb[nk] += w * kmag;
              nb[nk] += w;
            }
          }
        }
      }
    }
  }
}

/* The mode loop over contiguous x ranges, one per thread; the per-range bin
 * sums are added in range order, so the result does not depend on
 * scheduling. */
static void bin_modes(const double *dk, int N, double kmin, double kmax, int nbins, int bintype,
                      double *p0, double *p2, double *p4, double *kb, double *nb) {
  int nt = omp_get_max_threads();
  if (nt > N) nt = N;
  const size_t nb5 = 5 * (size_t)nbins;
  double *part = calloc(nb5 * nt, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    double *q = part + nb5 * t;
    bin_modes_rows(dk, N, (int)((long)N * t / nt), (int)((long)N * (t + 1) / nt), kmin, kmax, nbins, bintype, q,
                   p2 ? q + nbins : NULL, p4 ? q + 2 * (size_t)nbins : NULL, q + 3 * (size_t)nbins,
                   q + 4 * (size_t)nbins);
  }
  for (int t = 0; t < nt; t++) {
    const double *q = part + nb5 * t;
    for (int b = 0; b < nbins; b++) {
      p0[b] += q[b];
      if (p2) p2[b] += q[nbins + b];
      if (p4) p4[b] += q[2 * (size_t)nbins + b];
      kb[b] += q[3 * (size_t)nbins + b];
      nb[b] += q[4 * (size_t)nbins + b];
    }
  }
  free(part);
}

int orc_pofk(const double *deltak, int N, int Ns, double box, int *nbins_io, int bintype,
             int sub, double kmin_hmpc, double kmax_hmpc, double *kbin, double *pk,
             double *kmean, double *nmodes) {
  int nbins = *nbins_io;
  double kmin = kmin_hmpc * box / (2.0 * M_PI), kmax = kmax_hmpc * box / (2.0 * M_PI);
  int cap = nbins > 0 ? nbins : N;
  adjust_pofk(N, &nbins, &bintype, &sub, &kmin, &kmax);
  if (nbins > cap && *nbins_io > 0) return -1;
  double *p = calloc(nbins, sizeof(double)), *kb = calloc(nbins, sizeof(double)), *nb = calloc(nbins, sizeof(double));
  bin_modes(deltak, N, kmin, kmax, nbins, bintype, p, NULL, NULL, kb, nb);
  for (int i = 0; i < nbins; i++) {
    double P = 0, K = 0;
    if (nb[i] > 0) {
      P = (p[i] / nb[i]) * pow(box, 3);
      if (sub) P -= pow(box / (double)Ns, 3);
      K = (kb[i] / nb[i]) * 2.0 * M_PI / box;
    }
    kbin[i] = k_from_index(i, kmin, kmax, nbins, bintype, box);
    pk[i] = P;
    kmean[i] = K;
    nmodes[i] = nb[i];
  }
  free(p); free(kb); free(nb);
  *nbins_io = nbins;
  return nbins;
}

/* PtoMesh_RSD (compute_pofk.c:280-393) + bin_up_RSD_power_spectrum
 * (compute_pofk.c:518-753) for one LOS axis; vnorm is the factor
 * (Hubble/A)/(100 A H(A)) * N/Box of compute_pofk.c:290-291. */
int orc_pofk_rsd_axis(const double *pos, const double *vel, const double *vel_extra, long np,
                      int axis, int N, int Ns, double box, double vnorm,
                      int *nbins_io, int bintype, int sub, double kmin_hmpc, double kmax_hmpc,
                      double *kout, double *P0, double *P2, double *P4, double *nout) {
  const size_t P = 2 * (size_t)(N / 2 + 1);
  const size_t slice = (size_t)N * P;
  double *d = malloc(sizeof(double) * (size_t)(N + 1) * slice);
  const double scaleBox = (double)N / box;
  const double WPAR = pow((double)N / (double)Ns, 3);
  for (size_t i = 0; i < (size_t)(N + 1) * slice; i++) d[i] = -1.0;
  for (long i = 0; i < np; i++) {
    double X, Y, Z, V;
    if (axis == 1) { X = pos[3 * i] * scaleBox; Y = pos[3 * i + 2] * scaleBox; Z = pos[3 * i + 1] * scaleBox; }
    else { X = pos[3 * i] * scaleBox; Y = pos[3 * i + 1] * scaleBox; Z = pos[3 * i + 2] * scaleBox; }
    V = vel[3 * i + axis] + (vel_extra ? vel_extra[3 * i + axis] : 0.0);
    V *= vnorm;
    Z += V;
    if (Z >= (double)N) Z -= (double)N;
    if (Z < 0) Z += (double)N;
    unsigned IX = (unsigned)X, IY = (unsigned)Y, IZ = (unsigned)Z;
    double DX = X - (double)IX, DY = Y - (double)IY, DZ = Z - (double)IZ;
    double TX = 1.0 - DX, TY = 1.0 - DY, TZ = 1.0 - DZ;
    DY *= WPAR;
    TY *= WPAR;
    if (IY >= (unsigned)N) IY = 0;
    if (IZ >= (unsigned)N) IZ = 0;
    unsigned IXn = IX + 1, IYn = IY + 1, IZn = IZ + 1;
    if (IYn >= (unsigned)N) IYn = 0;
    if (IZn >= (unsigned)N) IZn = 0;
    d[ridx(N, IX, IY, IZ)] += TX * TY * TZ;
    d[ridx(N, IX, IY, IZn)] += TX * TY * DZ;
    d[ridx(N, IX, IYn, IZ)] += TX * DY * TZ;
    d[ridx(N, IX, IYn, IZn)] += TX * DY * DZ;
    d[ridx(N, IXn, IY, IZ)] += DX * TY * TZ;
    d[ridx(N, IXn, IY, IZn)] += DX * TY * DZ;
    d[ridx(N, IXn, IYn, IZ)] += DX * DY * TZ;
    d[ridx(N, IXn, IYn, IZn)] += DX * DY * DZ;
  }
  if (np != 0)
    for (size_t i = 0; i < slice; i++) d[i] += d[(size_t)N * slice + i] + 1.0;
  orc_fft_r2c(N, d);
  int nbins = *nbins_io;
  double kmin = kmin_hmpc * box / (2.0 * M_PI), kmax = kmax_hmpc * box / (2.0 * M_PI);
  adjust_pofk(N, &nbins, &bintype, &sub, &kmin, &kmax);
  if (*nbins_io > 0 && nbins > *nbins_io) { free(d); return -1; }
  double *p0 = calloc(nbins, 8), *p2 = calloc(nbins, 8), *p4 = calloc(nbins, 8), *kb = calloc(nbins, 8), *nb = calloc(nbins, 8);
  bin_modes(d, N, kmin, kmax, nbins, bintype, p0, p2, p4, kb, nb);
  for (int i = 0; i < nbins; i++) {
    double a0 = 0, a2 = 0, a4 = 0, kk = 0;
    if (nb[i] > 0) {
      a0 = (p0[i] / nb[i]) * pow(box, 3);
      a2 = (p2[i] / nb[i]) * pow(box, 3);
      a4 = (p4[i] / nb[i]) * pow(box, 3);
      a4 = 9.0 * (35.0 * a4 - 30.0 * a2 + 3.0 * a0) / 8.0;
      a2 = 5.0 * (3.0 * a2 - 1.0 * a0) / 2.0;
      if (sub) {
        a0 -= pow(box / (double)Ns, 3);
        a2 -= pow(box / (double)Ns, 3);
        a4 -= pow(box / (double)Ns, 3);
      }
      kk = k_from_index(i, kmin, kmax, nbins, bintype, box);
    }
    kout[i] = kk; P0[i] = a0; P2[i] = a2; P4[i] = a4; nout[i] = nb[i];
  }
  free(p0); free(p2); free(p4); free(kb); free(nb); free(d);
  *nbins_io = nbins;
  return nbins;
}
