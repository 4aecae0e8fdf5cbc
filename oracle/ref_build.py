"""Recipe: compile MG-PICOLA's own C sources, unmodified, into single-rank
reference binaries (test infrastructure only).

The reference needs FFTW3-MPI, GSL and MPI, which this image does not have;
the sources are compiled against the project-written shims in
oracle/ref_shim (single-rank MPI, the oracle's FFTW-convention FFTs, GSL
calls restated from their documentation).  Sources are read in place from
the reference tree; outputs go to oracle/_ref/ only.  Built in double
precision (MEMORY_MODE and SINGLE_PRECISION off) with GAUSSIAN, COMPUTE_POFK
and GADGET_STYLE, one binary per model as the reference Makefile does.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's src/ directory; the reference binaries are built only when it is given
REF_SRC = os.environ.get("MGP_REFERENCE_SRC", "")
OUT = os.path.join(HERE, "_ref")
SOURCES = ["main.c", "auxPM.c", "2LPT.c", "cosmo.c", "power.c", "compute_pofk.c", "read_param.c", "vars.c",
           "wrappers.c", "timer.c", "msg.c", "jbd.c"]
SHIM = [os.path.join(HERE, "ref_shim", "ref_shim.c"), os.path.join(HERE, "orc_fft.c"), os.path.join(HERE, "orc_rng.c"),
        os.path.join(HERE, "orc_interp2d.c")]
COMMON = ["-DGAUSSIAN", "-DCOMPUTE_POFK", "-DGADGET_STYLE"]
# model -> preprocessor flags (Makefile:61-106)
MODELS = {
    "FOFR_LCDM": ["-DFOFRGRAVITY"],
    "DGP": ["-DDGPGRAVITY", "-DGAUSSIANFILTER"],
    "BRANSDICKE": ["-DBRANSDICKE"],
    "MBETA_LCDM": ["-DMBETAMODEL"],
    "FOFR": ["-DFOFRGRAVITY", "-DSCALEDEPENDENT"],
    "MBETA": ["-DMBETAMODEL", "-DSCALEDEPENDENT"],
    "FOFRNU": ["-DFOFRGRAVITY", "-DMASSIVE_NEUTRINOS", "-DSCALEDEPENDENT"],
    # initial conditions read from particle files (src/readICfromfile.c)
    "FOFR_LCDM_IC": ["-DFOFRGRAVITY", "-DREADICFROMFILE"],
    # ASCII snapshots instead of GADGET-1 (GADGET_STYLE off)
    "FOFR_LCDM_ASCII": ["-DFOFRGRAVITY"],
    # w(a) = w0 + wa (1 - a) background
    "FOFR_LCDM_W0WA": ["-DFOFRGRAVITY", "-DEQUATIONOFSTATE_PARAMETRIZATION"],
    # nDGP with the top-hat / sharp-k smoothing filter (src/mg.h:318-338)
    "DGP_TOPHAT": ["-DDGPGRAVITY", "-DTOPHATFILTER"],
    "DGP_SHARPK": ["-DDGPGRAVITY", "-DSHARPKFILTER"],
}
NO_GADGET_STYLE = {"FOFR_LCDM_ASCII"}
# sources a build adds to SOURCES
EXTRA_SOURCES = {"FOFR_LCDM_IC": ["readICfromfile.c"]}


def available():
    return bool(REF_SRC) and os.path.isdir(REF_SRC) and all(os.path.exists(os.path.join(REF_SRC, s)) for s in SOURCES)


def binary(model):
    return os.path.join(OUT, "MG_PICOLA_" + model)


def build(models=None, verbose=False):
    if not available():
        raise RuntimeError("reference sources not found (set MGP_REFERENCE_SRC to the reference's src/ directory)")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "ref_shim", "include"), "-I" + REF_SRC]
    srcs = [os.path.join(REF_SRC, s) for s in SOURCES] + SHIM
    headers = [os.path.join(HERE, "orc.h")] + [os.path.join(d, f) for d, _, fs in os.walk(os.path.join(HERE, "ref_shim"))
                                              for f in fs if f.endswith(".h")]
    newest = max(os.path.getmtime(s) for s in srcs + headers)
    for model in models or MODELS:
        out = binary(model)
        if os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        extra = [os.path.join(REF_SRC, f) for f in EXTRA_SOURCES.get(model, [])]
        common = [f for f in COMMON if not (model in NO_GADGET_STYLE and f == "-DGADGET_STYLE")]
        cmd = (["gcc", "-O2", "-std=gnu99", "-fopenmp", "-w", "-o", out] + common + MODELS[model] + inc + srcs +
               extra + ["-lm"])
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
