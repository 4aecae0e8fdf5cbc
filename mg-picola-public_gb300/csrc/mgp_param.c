/*
 * Parameter-file reader compatible with MG-PICOLA's read_parameterfile
 * (src/read_param.c:107-445) and read_mg_parameters
 * (src/user_defined_functions.h:227-406): flat "key value" lines, '%' starts
 * a comment line, every key registered for the chosen model is mandatory,
 * unknown or repeated keys are errors.  The set of keys depends on the model
 * (the reference's compile-time MODEL) and on the COMPUTE_POFK and
 * EQUATIONOFSTATE_PARAMETRIZATION options.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mgpicola.h"

enum { T_FLOAT = 1, T_STRING = 2, T_INT = 3 };

typedef struct {
  char tag[50];
  void *addr;
  int type;
  int seen;
} key_t_;

static char g_perr[1024];
int mgp_set_error(int code, const char *fmt, ...);

int mgp_params_default(mgp_params *p) {
  if (!p) return MGP_EINVAL;
  memset(p, 0, sizeof(*p));
  p->model = MGP_MODEL_LCDM;
  p->smoothing_filter = MGP_FILTER_NONE;
  p->include_screening = 1;
  p->input_pofk_is_for_lcdm = 1;
  p->input_sigma8_is_for_lcdm = 1;
  p->fofr0 = 1e-5;
  p->nfofr = 1.0;
  p->Rsmooth = 1.0;
  p->rcH0_DGP = 1.0;
  p->w_0 = -1.0;
  p->pofk_compute_every_step = 1;
  p->pofk_nbins = 0;
  p->pofk_subtract_shotnoise = 1;
  strcpy(p->OutputDir, "output");
  strcpy(p->FileBase, "mgpicola");
  p->NumFilesWrittenInParallel = 1;
  p->UseCOLA = 1;
  p->Buffer = 1.5;
  p->Nmesh = 64;
  p->Nsample = 32;
  p->Box = 256.0;
  p->Init_Redshift = 19.0;
  p->Seed = 5001;
  p->WhichSpectrum = 2;
  p->Omega = 0.267;
  p->OmegaBaryon = 0.049;
  p->HubbleParam = 0.71;
  p->Sigma8 = 0.8;
  p->PrimordialIndex = 0.96;
  p->UnitLength_in_cm = 3.085678e24;
  p->UnitMass_in_g = 1.989e43;
  p->UnitVelocity_in_cm_per_s = 1e5;
  p->InputSpectrum_UnitLength_in_cm = 3.085678e24;
  p->Noutputs = 1;
  p->output_redshift[0] = 0.0;
  p->output_nsteps[0] = 10;
  return MGP_OK;
}

#define ADD(name, field, ktype)                   \
  do {                                            \
    strcpy(keys[nt].tag, name);                   \
    keys[nt].addr = (void *)&(p->field);          \
    keys[nt].type = ktype;                        \
    keys[nt].seen = 0;                            \
    nt++;                                         \
  } while (0)

/* read_outputs, src/read_param.c:32-89 */
static int read_outputs(mgp_params *p) {
  FILE *fd = fopen(p->OutputRedshiftFile, "r");
  if (!fd) {
    snprintf(g_perr, sizeof(g_perr), "Output Redshift File '%s' not found", p->OutputRedshiftFile);
    return mgp_set_error(MGP_EIO, "%s", g_perr);
  }
  char buf[500];
  int n = 0;
  while (fgets(buf, sizeof(buf), fd)) {
    double red;
    int nsteps;
    if (buf[0] == '%') continue;
    int got = sscanf(buf, "%lf, %d", &red, &nsteps);
    if (got > 0) {
      if (got != 2) {
        fclose(fd);
        snprintf(g_perr, sizeof(g_perr), "Line in Output Redshift File '%s' is in incorrect format", buf);
        return mgp_set_error(MGP_EPARAM, "%s", g_perr);
      }
      if (nsteps <= 0 && (p->Init_Redshift - red) / p->Init_Redshift > 1.0E-6) {
        fclose(fd);
        snprintf(g_perr, sizeof(g_perr), "nsteps <= 0 up to redshift %lf", red);
        return mgp_set_error(MGP_EPARAM, "%s", g_perr);
      }
      if (n == 64) {
        fclose(fd);
        snprintf(g_perr, sizeof(g_perr), "more than 64 output redshifts");
        return mgp_set_error(MGP_EPARAM, "%s", g_perr);
      }
      p->output_redshift[n] = red;
      p->output_nsteps[n] = nsteps;
      n++;
    }
  }
  fclose(fd);
  if (n == 0) {
    snprintf(g_perr, sizeof(g_perr), "Found no output redshifts in file '%s'", p->OutputRedshiftFile);
    return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  }
  /* descending order, duplicates are fatal (sort_redshift) */
  for (int i = 1; i < n; i++) {
    double z = p->output_redshift[i];
    int s = p->output_nsteps[i], j = i - 1;
    while (j >= 0 && p->output_redshift[j] < z) {
      p->output_redshift[j + 1] = p->output_redshift[j];
      p->output_nsteps[j + 1] = p->output_nsteps[j];
      j--;
    }
    p->output_redshift[j + 1] = z;
    p->output_nsteps[j + 1] = s;
  }
  for (int i = 1; i < n; i++)
    if (p->output_redshift[i] == p->output_redshift[i - 1]) {
      snprintf(g_perr, sizeof(g_perr), "Duplicate output redshift (%lf) in Output Redshift File", p->output_redshift[i]);
      return mgp_set_error(MGP_EPARAM, "%s", g_perr);
    }
  if (p->output_redshift[0] > p->Init_Redshift) {
    snprintf(g_perr, sizeof(g_perr), "The highest output redshift (%lf) is greater than the initial redshift (%lf)",
             p->output_redshift[0], p->Init_Redshift);
    return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  }
  p->Noutputs = n;
  return MGP_OK;
}


int mgp_read_parameterfile(const char *fname, int model, int pofk_keys, int read_outputs_flag, mgp_params *p) {
  key_t_ keys[128];
  int nt = 0;
  g_perr[0] = 0;
  if (!fname || !p) return MGP_EINVAL;
  int use_w0wa = p->use_w0wa, readic = p->ReadParticlesFromFile, mnu = p->massive_neutrinos;
  int sdep = p->scaledependent;
  mgp_params_default(p);
  p->model = model;
  p->use_w0wa = use_w0wa;
  p->massive_neutrinos = mnu;
  p->scaledependent = sdep;
  if (readic) {
    /* src/read_param.c:129-151 (READICFROMFILE) */
    ADD("ReadParticlesFromFile", ReadParticlesFromFile, T_INT);
    ADD("InputParticleFileDir", InputParticleFileDir, T_STRING);
    ADD("InputParticleFilePrefix", InputParticleFilePrefix, T_STRING);
    ADD("TypeInputParticleFiles", TypeInputParticleFiles, T_INT);
    ADD("NumInputParticleFiles", NumInputParticleFiles, T_INT);
    ADD("RamsesOutputNumber", RamsesOutputNumber, T_INT);
  }
  if (model == MGP_MODEL_DGP) p->smoothing_filter = MGP_FILTER_GAUSSIAN;
  /* read_mg_parameters, user_defined_functions.h:233-405 */
  ADD("modified_gravity_active", modified_gravity_active, T_INT);
  ADD("use_lcdm_growth_factors", use_lcdm_growth_factors, T_INT);
  ADD("input_pofk_is_for_lcdm", input_pofk_is_for_lcdm, T_INT);
  ADD("input_sigma8_is_for_lcdm", input_sigma8_is_for_lcdm, T_INT);
  ADD("inverted_initial_condition", inverted_initial_condition, T_INT);
  ADD("amplitude_fixed_initial_condition", amplitude_fixed_initial_condition, T_INT);
  ADD("include_screening", include_screening, T_INT);
  if (mnu) {
    /* read_mg_parameters, user_defined_functions.h:261-273 (MASSIVE_NEUTRINOS) */
    ADD("nu_include_massive_neutrinos", nu_include_massive_neutrinos, T_INT);
    ADD("nu_SumMassNuEV", nu_SumMassNuEV, T_FLOAT);
    ADD("nu_FilenameTransferInfofile", nu_FilenameTransferInfofile, T_STRING);
  }
  if (pofk_keys) {
    ADD("pofk_compute_every_step", pofk_compute_every_step, T_INT);
    ADD("pofk_compute_rsd_pofk", pofk_compute_rsd_pofk, T_INT);
    ADD("pofk_nbins", pofk_nbins, T_INT);
    ADD("pofk_bintype", pofk_bintype, T_INT);
    ADD("pofk_subtract_shotnoise", pofk_subtract_shotnoise, T_INT);
    ADD("pofk_kmin", pofk_kmin, T_FLOAT);
    ADD("pofk_kmax", pofk_kmax, T_FLOAT);
  } else {
    /* fiducial P(k) settings without COMPUTE_POFK (compute_pofk.c:96-105) */
    p->pofk_compute_every_step = 0;
    p->pofk_nbins = p->Nmesh / 2;
  }
  if (use_w0wa) {
    ADD("w_0", w_0, T_FLOAT);
    ADD("w_a", w_a, T_FLOAT);
  }
  switch (model) {
    case MGP_MODEL_FOFR:
      ADD("fofr0", fofr0, T_FLOAT);
      ADD("nfofr", nfofr, T_FLOAT);
      break;
    case MGP_MODEL_MBETA:
      ADD("range_symm", range_symm, T_FLOAT);
      ADD("assb_symm", assb_symm, T_FLOAT);
      ADD("beta_symm", beta_symm, T_FLOAT);
      break;
    case MGP_MODEL_DGP:
      ADD("Rsmooth", Rsmooth, T_FLOAT);
      ADD("rcH0_DGP", rcH0_DGP, T_FLOAT);
      break;
    case MGP_MODEL_BRANSDICKE:
      /* the reference registers Omegar2/Omegav2 (user_defined_functions.h:393-399) */
      ADD("wBD", wBD, T_FLOAT);
      ADD("Omegah2", Omegah2, T_FLOAT);
      ADD("Omegar2", Omegarh2, T_FLOAT);
      ADD("Omegav2", Omegavh2, T_FLOAT);
      break;
    default:
      break;
  }
  /* standard keys, src/read_param.c:167-265 */
  ADD("OutputDir", OutputDir, T_STRING);
  ADD("FileBase", FileBase, T_STRING);
  ADD("OutputRedshiftFile", OutputRedshiftFile, T_STRING);
  ADD("NumFilesWrittenInParallel", NumFilesWrittenInParallel, T_INT);
  ADD("UseCOLA", UseCOLA, T_INT);
  ADD("Buffer", Buffer, T_FLOAT);
  ADD("Nmesh", Nmesh, T_INT);
  ADD("Nsample", Nsample, T_INT);
  ADD("Box", Box, T_FLOAT);
  ADD("Init_Redshift", Init_Redshift, T_FLOAT);
  ADD("Seed", Seed, T_INT);
  ADD("SphereMode", SphereMode, T_INT);
  ADD("WhichSpectrum", WhichSpectrum, T_INT);
  ADD("WhichTransfer", WhichTransfer, T_INT);
  ADD("FileWithInputSpectrum", FileWithInputSpectrum, T_STRING);
  ADD("FileWithInputTransfer", FileWithInputTransfer, T_STRING);
  ADD("Omega", Omega, T_FLOAT);
  ADD("OmegaBaryon", OmegaBaryon, T_FLOAT);
  ADD("HubbleParam", HubbleParam, T_FLOAT);
  ADD("Sigma8", Sigma8, T_FLOAT);
  ADD("PrimordialIndex", PrimordialIndex, T_FLOAT);
  ADD("UnitVelocity_in_cm_per_s", UnitVelocity_in_cm_per_s, T_FLOAT);
  ADD("UnitLength_in_cm", UnitLength_in_cm, T_FLOAT);
  ADD("UnitMass_in_g", UnitMass_in_g, T_FLOAT);
  ADD("InputSpectrum_UnitLength_in_cm", InputSpectrum_UnitLength_in_cm, T_FLOAT);

  FILE *fd = fopen(fname, "r");
  if (!fd) {
    snprintf(g_perr, sizeof(g_perr), "Parameter file '%s' not found", fname);
    return mgp_set_error(MGP_EIO, "%s", g_perr);
  }
  int err = 0;
  char buf[500], b1[500], b2[500], b3[500];
  while (fgets(buf, sizeof(buf), fd)) {
    if (sscanf(buf, "%499s%499s%499s", b1, b2, b3) < 2) continue;
    if (b1[0] == '%') continue;
    int j = -1;
    for (int i = 0; i < nt; i++)
      if (!keys[i].seen && strcmp(b1, keys[i].tag) == 0) { j = i; break; }
    if (j < 0) {
      if (!err) snprintf(g_perr, sizeof(g_perr), "In file %s: Tag '%s' not allowed or multiple defined", fname, b1);
      err = 1;
      continue;
    }
    keys[j].seen = 1;
    switch (keys[j].type) {
      case T_FLOAT: *(double *)keys[j].addr = atof(b2); break;
      case T_STRING: strcpy((char *)keys[j].addr, b2); break;
      case T_INT: *(int *)keys[j].addr = atoi(b2); break;
    }
  }
  fclose(fd);
  for (int i = 0; i < nt; i++)
    if (!keys[i].seen) {
      if (!err) snprintf(g_perr, sizeof(g_perr), "I miss a value for tag '%s' in parameter file '%s'", keys[i].tag, fname);
      err = 1;
    }
  if (err) return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  if (p->NumFilesWrittenInParallel < 1) {
    snprintf(g_perr, sizeof(g_perr), "NumFilesWrittenInParallel is less than 1");
    return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  }
  if (p->WhichSpectrum != 0 && p->WhichTransfer != 0) {
    snprintf(g_perr, sizeof(g_perr), "You are running with both power spectrum and transfer function");
    return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  }
  if (p->WhichSpectrum == 0 && p->WhichTransfer == 0) {
    snprintf(g_perr, sizeof(g_perr), "You are running with neither power spectrum nor transfer function");
    return mgp_set_error(MGP_EPARAM, "%s", g_perr);
  }
  if (!pofk_keys) p->pofk_nbins = p->Nmesh / 2, p->pofk_kmax = 2.0 * 3.14159265358979323846 / p->Box * (p->Nmesh / 2.0);
  if (read_outputs_flag) return read_outputs(p);
  return MGP_OK;
}
