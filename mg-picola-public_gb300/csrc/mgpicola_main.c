/*
 * mgpicola_run: the command-line driver, the drop-in for the reference's
 * executable MG_PICOLA_<MODEL> <ParameterFile> (src/main.c:33-57).
 *
 * The reference fixes the model and its options when it is compiled
 * (Makefile MODEL = DGP, FOFR, FOFR_LCDM, MBETA, BRANSDICKE, FOFRNU and the
 * COMPUTE_POFK, EQUATIONOFSTATE_PARAMETRIZATION, READICFROMFILE and
 * GADGET_STYLE switches); here they are run-time options:
 *
 *   mgpicola_run [-model NAME] [-pofk] [-w0wa] [-readic] [-ascii]
 *                [-filter gaussian|tophat|sharpk] [-device N] <ParameterFile>
 *
 * NAME is one of the reference's MODEL values plus MBETA_LCDM (the m(a),
 * beta(a) model with scale-independent growth); the default is the
 * Makefile's DGP.  Invoked through a link named MG_PICOLA_<MODEL>, the
 * program takes the model from its own name, so the link is a drop-in for
 * the reference's executable.  It reads the parameter file with the
 * reference's keys (read_param.c:107-445), runs the initial conditions and
 * the time loop (main.c:231-611) on one GPU, and writes the same snapshot,
 * P(k) and info files.  Errors print the library's message and exit with
 * status 1, where the reference calls FatalError/MPI_Abort.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mgpicola.h"

typedef struct {
  const char *name;
  int model, scaledependent, neutrinos;
} model_def;

/* Makefile:61-106 */
static const model_def MODELS[] = {
    {"DGP", MGP_MODEL_DGP, 0, 0},         {"FOFR", MGP_MODEL_FOFR, 1, 0},   {"FOFR_LCDM", MGP_MODEL_FOFR, 0, 0},
    {"MBETA", MGP_MODEL_MBETA, 1, 0},     {"MBETA_LCDM", MGP_MODEL_MBETA, 0, 0},
    {"BRANSDICKE", MGP_MODEL_BRANSDICKE, 0, 0}, {"FOFRNU", MGP_MODEL_FOFR, 1, 1},
};

static const model_def *find_model(const char *name) {
  for (size_t i = 0; i < sizeof(MODELS) / sizeof(MODELS[0]); i++)
    if (strcmp(MODELS[i].name, name) == 0) return &MODELS[i];
  return NULL;
}

static int usage(void) {
  fprintf(stdout, "Input parameters not found\n");
  fprintf(stdout, "Call with <ParameterFile>\n");
  fprintf(stdout, "  options: -model DGP|FOFR|FOFR_LCDM|MBETA|MBETA_LCDM|BRANSDICKE|FOFRNU  -pofk  -w0wa  -readic\n"
                  "           -ascii  -filter gaussian|tophat|sharpk  -device N\n");
  return 1;
}

int main(int argc, char **argv) {
  const model_def *md = find_model("DGP");
  /* a link named MG_PICOLA_<MODEL> selects the model */
  const char *base = strrchr(argv[0], '/');
  base = base ? base + 1 : argv[0];
  if (strncmp(base, "MG_PICOLA_", 10) == 0) {
    const model_def *m = find_model(base + 10);
    if (!m) {
      fprintf(stderr, "ERROR: MODEL %s is not recognized\n", base + 10);
      return 1;
    }
    md = m;
  }
  int pofk = 0, w0wa = 0, readic = 0, ascii = 0, device = 0, filter = -1;
  const char *paramfile = NULL;
  for (int i = 1; i < argc; i++) {
    const char *a = argv[i];
    if (strcmp(a, "-model") == 0 && i + 1 < argc) {
      md = find_model(argv[++i]);
      if (!md) {
        fprintf(stderr, "ERROR: MODEL %s is not recognized\n", argv[i]);
        return 1;
      }
    } else if (strcmp(a, "-pofk") == 0) {
      pofk = 1;
    } else if (strcmp(a, "-w0wa") == 0) {
      w0wa = 1;
    } else if (strcmp(a, "-readic") == 0) {
      readic = 1;
    } else if (strcmp(a, "-ascii") == 0) {
      ascii = 1;
    } else if (strcmp(a, "-device") == 0 && i + 1 < argc) {
      device = atoi(argv[++i]);
    } else if (strcmp(a, "-filter") == 0 && i + 1 < argc) {
      const char *f = argv[++i];
      filter = strcmp(f, "gaussian") == 0 ? MGP_FILTER_GAUSSIAN
               : strcmp(f, "tophat") == 0 ? MGP_FILTER_TOPHAT
               : strcmp(f, "sharpk") == 0 ? MGP_FILTER_SHARPK
                                           : -2;
      if (filter == -2) {
        fprintf(stderr, "ERROR: smoothing filter %s is not recognized\n", f);
        return 1;
      }
    } else if (a[0] == '-' && a[1]) {
      fprintf(stderr, "ERROR: unknown option %s\n", a);
      return usage();
    } else {
      paramfile = a;
    }
  }
  if (!paramfile) return usage();

  mgp_params p;
  memset(&p, 0, sizeof(p));
  p.use_w0wa = w0wa;
  p.ReadParticlesFromFile = readic;
  p.scaledependent = md->scaledependent;
  p.massive_neutrinos = md->neutrinos;
  if (mgp_read_parameterfile(paramfile, md->model, pofk, 1, &p) != MGP_OK) {
    fprintf(stderr, "%s\n", mgp_last_error());
    return 1;
  }
  if (filter >= 0) p.smoothing_filter = filter;
  fprintf(stdout, "MG-PICOLA GB300: model %s, Nsample %d, Nmesh %d, Box %g, %d output(s), device %d\n", md->name,
          p.Nsample, p.Nmesh, p.Box, p.Noutputs, device);
  fflush(stdout);
  mgp_ctx *ctx = NULL;
  if (mgp_create(&p, device, &ctx) != MGP_OK) {
    fprintf(stderr, "%s\n", mgp_last_error());
    return 1;
  }
  int rc = mgp_run(ctx, !ascii);
  if (rc != MGP_OK) fprintf(stderr, "%s\n", mgp_last_error());
  mgp_destroy(ctx);
  if (rc == MGP_OK) fprintf(stdout, "Run complete: outputs in %s\n", p.OutputDir);
  return rc == MGP_OK ? 0 : 1;
}
