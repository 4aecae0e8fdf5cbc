"""Build recipe for the FP64 oracle (test infrastructure only).

Compiles oracle/*.c into oracle/build/liboracle.so with gcc + OpenMP.  Plain
C99, no architecture-specific flags, so the same recipe works on x86_64 and
aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["orc_fft.c", "orc_pm.c", "orc_cosmo.c", "orc_rng.c", "orc_mg.c", "orc_ic.c", "orc_run.c", "orc_interp2d.c",
           "orc_sd.c", "orc_nu.c"]
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "orc.h")])
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-fopenmp", "-Wall", "-Wno-unused-function",
           "-o", LIB] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
