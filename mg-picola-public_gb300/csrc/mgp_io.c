/*
 * Output writers in the reference's formats (see mgp_io.h).
 */
#include "mgp_io.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int mgp_set_error(int code, const char *fmt, ...);

#define GRAVITY 6.672e-8   /* src/vars.h:60 */
#define HUBBLE 3.2407789e-18 /* src/vars.h:62 */

void mgp_units_init(const mgp_params *p, mgp_units *u) {
  u->UnitTime_in_s = p->UnitLength_in_cm / p->UnitVelocity_in_cm_per_s;
  u->G = GRAVITY / pow(p->UnitLength_in_cm, 3) * p->UnitMass_in_g * pow(u->UnitTime_in_s, 2);
  u->Hubble = HUBBLE * u->UnitTime_in_s;
  u->lengthfac = p->UnitLength_in_cm / 3.085678e24;
  u->velfac = p->UnitVelocity_in_cm_per_s / 1.0e5;
}

void mgp_snapshot_name(const mgp_params *p, double Z, char *buf, size_t len) {
  int zi, zf;
  if (Z < 0.0) {
    zi = zf = 0;
  } else {
    zi = (int)floor(Z);
    zf = (int)((Z - zi) * 1000);
  }
  snprintf(buf, len, "%s/%s_z%dp%03d.%d", p->OutputDir, p->FileBase, zi, zf, 0);
}

static int wr(const void *ptr, size_t sz, size_t n, FILE *fp) {
  return fwrite(ptr, sz, n, fp) == n ? 0 : -1;
}

/* write_gadget_header (src/main.c:1106-1149) + the position and velocity
 * blocks of Output (src/main.c:913-977). */
int mgp_write_gadget(const char *path, const mgp_params *p, double A, const float *pos, const float *vel, size_t np) {
  FILE *fp = fopen(path, "w");
  if (!fp) return mgp_set_error(MGP_EIO, "Can't write in file '%s'", path);
  mgp_units u;
  mgp_units_init(p, &u);
  mgp_gadget_header h;
  memset(&h, 0, sizeof(h));
  unsigned long long tot = (unsigned long long)p->Nsample * p->Nsample * p->Nsample;
  h.npart[1] = (unsigned int)np;
  h.npartTotal[1] = (unsigned int)tot;
  h.npartTotalHighWord[1] = (unsigned int)(tot >> 32);
  h.mass[1] = (3.0 * p->Omega * u.Hubble * u.Hubble * p->Box * p->Box * p->Box) / (8.0 * 3.14159265358979323846 * u.G * tot);
  h.time = A;
  h.redshift = 1.0 / A - 1.0;
  h.num_files = 1;
  h.BoxSize = p->Box * u.lengthfac;
  h.Omega0 = p->Omega;
  h.OmegaLambda = 1.0 - p->Omega;
  h.HubbleParam = p->HubbleParam;
  int dummy = (int)sizeof(h), rc = 0;
  rc |= wr(&dummy, sizeof(int), 1, fp);
  rc |= wr(&h, sizeof(h), 1, fp);
  rc |= wr(&dummy, sizeof(int), 1, fp);
  dummy = (int)(sizeof(float) * 3 * np);
  rc |= wr(&dummy, sizeof(int), 1, fp);
  rc |= wr(pos, sizeof(float), 3 * np, fp);
  rc |= wr(&dummy, sizeof(int), 1, fp);
  rc |= wr(&dummy, sizeof(int), 1, fp);
  rc |= wr(vel, sizeof(float), 3 * np, fp);
  rc |= wr(&dummy, sizeof(int), 1, fp);
  if (fclose(fp) != 0) rc = -1;
  if (rc) return mgp_set_error(MGP_EIO, "I/O error (fwrite) writing '%s'", path);
  return MGP_OK;
}

/* ASCII branch of Output (src/main.c:1000-1027). */
int mgp_write_ascii(const char *path, const float *pos, const float *vel, size_t np) {
  FILE *fp = fopen(path, "w");
  if (!fp) return mgp_set_error(MGP_EIO, "Can't write in file '%s'", path);
  int rc = fprintf(fp, "%u\n", (unsigned int)np) < 0;
  for (size_t n = 0; n < np && !rc; n++)
    rc = fprintf(fp, "%12.6f %12.6f %12.6f %12.6f %12.6f %12.6f\n", pos[3 * n], pos[3 * n + 1], pos[3 * n + 2],
                 vel[3 * n], vel[3 * n + 1], vel[3 * n + 2]) < 0;
  if (fclose(fp) != 0) rc = 1;
  if (rc) return mgp_set_error(MGP_EIO, "I/O error writing '%s'", path);
  return MGP_OK;
}

/* Output_Info (src/main.c:1067-1099), one task. */
int mgp_write_info(const mgp_params *p, double A, size_t np) {
  char buf[1100];
  double Z = (1.0 / A) - 1.0;
  snprintf(buf, sizeof(buf), "%s/info_%s_z%dp%03d.txt", p->OutputDir, p->FileBase, (int)Z, (int)rint((Z - (int)Z) * 1000));
  FILE *fp = fopen(buf, "w");
  if (!fp) return mgp_set_error(MGP_EIO, "Can't write in file '%s'", buf);
  fprintf(fp, "#    FILENUM      XMIN         YMIN        ZMIN         XMAX         YMAX         ZMAX         NPART    \n");
  fprintf(fp, "%12d %12.6lf %12.6lf %12.6lf %12.6lf %12.6lf %12.6lf %12u\n", 0, 0.0, 0.0, 0.0, p->Box, p->Box, p->Box,
          (unsigned int)np);
  fclose(fp);
  return MGP_OK;
}

static void zlabel(double a, int *zint, int *zfrac) {
  double znow = 1.0 / a - 1.0;
  *zint = (int)znow;
  *zfrac = (int)((znow - *zint) * 1000);
}

/* compute_power_spectrum file output (src/compute_pofk.c:238-260). */
int mgp_write_pofk(const mgp_params *p, double a, const char *label, int nbins, const double *kbin, const double *pk,
                   const double *kmean, const double *n) {
  int zi, zf;
  zlabel(a, &zi, &zf);
  char fn[1200];
  snprintf(fn, sizeof(fn), "%s/pofk_%s_z%d.%03d_%s.txt", p->OutputDir, p->FileBase, zi, zf, label);
  FILE *fp = fopen(fn, "w");
  if (!fp) return mgp_set_error(MGP_EIO, "Can't write in file '%s'", fn);
  fprintf(fp, "#  k_bin (h/Mpc)        P(k) (Mpc/h)^3     k_mean_bin (h/Mpc)     Delta = k^3P(k)/2pi^2\n");
  for (int i = 1; i < nbins; i++) {
    if (n[i] > 0) {
      double Delta = pk[i] * kbin[i] * kbin[i] * kbin[i] / 2.0 / M_PI / M_PI;
      fprintf(fp, "%10.5f   %10.5f   %10.5f   %10.5f\n", kbin[i], pk[i], kmean[i], Delta);
    }
  }
  fclose(fp);
  return MGP_OK;
}

/* compute_RSD_powerspectrum file output (src/compute_pofk.c:455-478). */
int mgp_write_pofk_rsd(const mgp_params *p, double a, int nbins, const double *k, const double *P0, const double *P2,
                       const double *P4, const double *s0, const double *s2, const double *s4, const double *ny) {
  int zi, zf;
  zlabel(a, &zi, &zf);
  char fn[1200];
  snprintf(fn, sizeof(fn), "%s/pofk_RSD_%s_z%d.%03d.txt", p->OutputDir, p->FileBase, zi, zf);
  FILE *fp = fopen(fn, "w");
  if (!fp) return mgp_set_error(MGP_EIO, "Can't write in file '%s'", fn);
  fprintf(fp, "#  k (h/Mpc)      P0 (Mpc/h)^3      P2 (Mpc/h)^3      P4 (Mpc/h)^3     sigma0     sigma2     sigma4\n");
  for (int i = 0; i < nbins; i++)
    if (ny[i] > 0 && k[i] > 0.0)
      fprintf(fp, "%10.5f   %10.5f   %10.5f   %10.5f   %10.5f   %10.5f   %10.5f\n", k[i], P0[i], P2[i], P4[i], s0[i], s2[i], s4[i]);
  fclose(fp);
  return MGP_OK;
}

/* ------------------------------------------------ IC particle files
 * The readers of src/readICfromfile.c:221-531.  Fortran-style records
 * (int byte count, payload, int byte count); the counts are checked. */
static int rec_read(FILE *fp, void *buf, size_t bytes, const char *path) {
  int m0 = 0, m1 = 0;
  if (fread(&m0, sizeof(int), 1, fp) != 1 || fread(buf, 1, bytes, fp) != bytes || fread(&m1, sizeof(int), 1, fp) != 1)
    return mgp_set_error(MGP_EIO, "short read in '%s'", path);
  if ((size_t)m0 != bytes || m1 != m0)
    return mgp_set_error(MGP_EIO, "record of %d bytes where %zu expected in '%s'", m0, bytes, path);
  return MGP_OK;
}

static int grow(double **pos, size_t *cap, size_t need) {
  if (need <= *cap) return MGP_OK;
  size_t c = *cap ? *cap : 1024;
  while (c < need) c *= 2;
  double *q = (double *)realloc(*pos, sizeof(double) * 3 * c);
  if (!q) return mgp_set_error(MGP_ENOMEM, "particle buffer of %zu particles", c);
  *pos = q;
  *cap = c;
  return MGP_OK;
}

int mgp_read_particle_files(const mgp_params *p, double **pos_out, size_t *n_out) {
  *pos_out = NULL;
  *n_out = 0;
  const int type = p->TypeInputParticleFiles, nf = p->NumInputParticleFiles;
  if (type < 1 || type > 3) return mgp_set_error(MGP_EPARAM, "Error: unknown file-format [%d]", type);
  if (nf < 1) return mgp_set_error(MGP_EPARAM, "NumInputParticleFiles = %d", nf);
  double *pos = NULL;
  size_t n = 0, cap = 0;
  int rc = MGP_OK;
  for (int f = 0; f < nf && rc == MGP_OK; f++) {
    char path[1100];
    if (type == 1)
      snprintf(path, sizeof(path), "%s/part_%05d.out%05d", p->InputParticleFileDir, p->RamsesOutputNumber, f + 1);
    else
      snprintf(path, sizeof(path), "%s/%s.%d", p->InputParticleFileDir, p->InputParticleFilePrefix,
               type == 3 ? f : f + 1);
    FILE *fp = fopen(path, type == 2 ? "r" : "rb");
    if (!fp) {
      rc = mgp_set_error(MGP_EIO, "Error: cannot open file [%s]", path);
      break;
    }
    if (type == 3) {
      /* GADGET-1: header, then the type-1 positions in Box units (float) */
      mgp_gadget_header h;
      rc = rec_read(fp, &h, sizeof(h), path);
      const size_t np = rc == MGP_OK ? h.npart[1] : 0;
      float *buf = np ? (float *)malloc(sizeof(float) * 3 * np) : NULL;
      if (rc == MGP_OK && np && !buf) rc = mgp_set_error(MGP_ENOMEM, "GADGET read buffer");
      if (rc == MGP_OK && np) rc = rec_read(fp, buf, sizeof(float) * 3 * np, path);
      if (rc == MGP_OK) rc = grow(&pos, &cap, n + np);
      if (rc == MGP_OK) {
        const double normfac = 1.0 / h.BoxSize;
        for (size_t q = 0; q < 3 * np; q++) {
          float x = (float)(buf[q] * normfac); /* the reference keeps the float buffer */
          if (x >= 1.0f) x = (float)(x - 1.0);
          pos[3 * n + q] = x;
        }
        n += np;
      }
      free(buf);
    } else if (type == 2) {
      /* ASCII: npart, then "x y z mass" per line, x in [0,1) */
      int np = 0;
      if (fscanf(fp, "%d", &np) != 1 || np < 0) rc = mgp_set_error(MGP_EIO, "bad particle count in '%s'", path);
      if (rc == MGP_OK) rc = grow(&pos, &cap, n + (size_t)np);
      for (int q = 0; q < np && rc == MGP_OK; q++) {
        double x, y, z, m;
        if (fscanf(fp, "%lf %lf %lf %lf", &x, &y, &z, &m) != 4) {
          rc = mgp_set_error(MGP_EIO, "short particle list in '%s'", path);
          break;
        }
        double v[3] = {x, y, z};
        for (int a = 0; a < 3; a++) pos[3 * (n + q) + a] = v[a] >= 1.0 ? v[a] - 1.0 : v[a];
      }
      if (rc == MGP_OK) n += (size_t)np;
    } else {
      /* RAMSES part file: ncpu, ndim, npart, localseed[4], nstar_tot,
       * mstar_tot[2], mstar_lost[2], nsink, then x, y, z (double, in [0,1)) */
      int hdr[3], seed4[4], nstar, m2[2], l2[2], nsink;
      rc = rec_read(fp, &hdr[0], sizeof(int), path);
      if (rc == MGP_OK) rc = rec_read(fp, &hdr[1], sizeof(int), path);
      if (rc == MGP_OK) rc = rec_read(fp, &hdr[2], sizeof(int), path);
      if (rc == MGP_OK) rc = rec_read(fp, seed4, sizeof(seed4), path);
      if (rc == MGP_OK) rc = rec_read(fp, &nstar, sizeof(int), path);
      if (rc == MGP_OK) rc = rec_read(fp, m2, sizeof(m2), path);
      if (rc == MGP_OK) rc = rec_read(fp, l2, sizeof(l2), path);
      if (rc == MGP_OK) rc = rec_read(fp, &nsink, sizeof(int), path);
      const size_t np = rc == MGP_OK && hdr[2] > 0 ? (size_t)hdr[2] : 0;
      double *buf = np ? (double *)malloc(sizeof(double) * np) : NULL;
      if (rc == MGP_OK && np && !buf) rc = mgp_set_error(MGP_ENOMEM, "RAMSES read buffer");
      if (rc == MGP_OK) rc = grow(&pos, &cap, n + np);
      for (int a = 0; a < 3 && rc == MGP_OK && np; a++) {
        rc = rec_read(fp, buf, sizeof(double) * np, path);
        for (size_t q = 0; q < np && rc == MGP_OK; q++) pos[3 * (n + q) + a] = buf[q] >= 1.0 ? buf[q] - 1.0 : buf[q];
      }
      free(buf);
      if (rc == MGP_OK) n += np;
    }
    fclose(fp);
  }
  if (rc != MGP_OK) {
    free(pos);
    return rc;
  }
  *pos_out = pos;
  *n_out = n;
  return MGP_OK;
}

void mgp_free_particles(double *pos) { free(pos); }
