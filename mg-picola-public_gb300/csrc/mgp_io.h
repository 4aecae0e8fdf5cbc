/*
 * Output writers with the reference's file formats: GADGET-1 snapshots and
 * ASCII particle files (src/main.c:792-1061, 1106-1149), the info file
 * (src/main.c:1067-1099) and P(k) tables (src/compute_pofk.c:240-260,
 * 455-478).
 */
#ifndef MGP_IO_H
#define MGP_IO_H
#include <stddef.h>

#include "mgpicola.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Unit conversions of set_units (src/2LPT.c:35-42). */
typedef struct {
  double UnitTime_in_s, G, Hubble;
  double lengthfac, velfac;
} mgp_units;
void mgp_units_init(const mgp_params *p, mgp_units *u);

/* GADGET-1 header (src/vars.h:204-224), 256 bytes. */
typedef struct {
  unsigned int npart[6];
  double mass[6];
  double time;
  double redshift;
  int flag_sfr;
  int flag_feedback;
  unsigned int npartTotal[6];
  int flag_cooling;
  int num_files;
  double BoxSize;
  double Omega0;
  double OmegaLambda;
  double HubbleParam;
  int flag_stellarage;
  int flag_metals;
  unsigned int npartTotalHighWord[6];
  int flag_entropy_instead_u;
  char fill[60];
} mgp_gadget_header;

/* Snapshot file name "<OutputDir>/<FileBase>_z%dp%03d.0" for redshift z. */
void mgp_snapshot_name(const mgp_params *p, double z, char *buf, size_t len);
/* pos/vel already in output units (Mpc/h, km/s), AoS float [np][3]. */
int mgp_write_gadget(const char *path, const mgp_params *p, double A, const float *pos, const float *vel, size_t np);
/* Positions of the IC particle files of p (TypeInputParticleFiles,
 * NumInputParticleFiles, InputParticleFileDir/Prefix, RamsesOutputNumber),
 * in [0,1) of the box, [n][3]; *pos is malloc'ed (free it). */
int mgp_read_particle_files(const mgp_params *p, double **pos, size_t *n);
int mgp_write_ascii(const char *path, const float *pos, const float *vel, size_t np);
int mgp_write_info(const mgp_params *p, double A, size_t np);
/* P(k) file "pofk_<FileBase>_z%d.%03d_<label>.txt" (bins from 1, n > 0). */
int mgp_write_pofk(const mgp_params *p, double a, const char *label, int nbins, const double *kbin, const double *pk,
                   const double *kmean, const double *n);
int mgp_write_pofk_rsd(const mgp_params *p, double a, int nbins, const double *k, const double *P0, const double *P2,
                       const double *P4, const double *s0, const double *s2, const double *s4, const double *ny);

#ifdef __cplusplus
}
#endif
#endif
