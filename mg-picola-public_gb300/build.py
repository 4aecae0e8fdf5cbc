"""Build recipe for libmgpicola.so (sm_103a CUDA + host C, cuFFT).

Compiles the CUDA translation units with nvcc for sm_103a only and the host C
sources with gcc, in parallel, and links an in-tree shared library
(mg-picola-public_gb300/lib/libmgpicola.so).  No architecture-specific host
flags, so the same recipe builds on x86_64 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmgpicola.so")
# the command-line driver (MG_PICOLA_<MODEL> <ParameterFile>), linked to the library
EXE = os.path.join(LIBDIR, "mgpicola_run")
EXE_SOURCE = "mgpicola_main.c"

CU_SOURCES = ["mgp_kernels.cu", "mgp_api.cu", "mgp_run.cu", "mgp_noalloc.cu", "mgp_sd.cu", "mgp_nn.cu", "mgp_tiles.cu", "mgp_fft.cu"]
C_SOURCES = ["mgp_cosmo.c", "mgp_param.c", "mgp_io.c"]
HEADERS = ["mgp_internal.h", "mgp_device.cuh", "mgp_cosmo.h", "mgp_rng.h", "mgp_io.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False):
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mgpicola.h")]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-I" + INCLUDE, "-I" + CSRC] + ARCH)
    for s in C_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append(["gcc", "-c", src, "-o", obj, "-O2", "-std=gnu99", "-fPIC", "-Wall",
                         "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include")])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
        for j, f in zip(jobs, futs):
            r = f.result()
            if verbose or r.returncode:
                print(" ".join(j))
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("compile failed: " + j[2])
    if _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-lcufft", "-lm", "-L" + os.path.join(cuda, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            print(" ".join(cmd))
            sys.stdout.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("link failed")
    src = os.path.join(CSRC, EXE_SOURCE)
    if _stale(EXE, [src, LIB, os.path.join(INCLUDE, "mgpicola.h")]):
        cmd = ["gcc", "-O2", "-std=gnu99", "-Wall", "-o", EXE, src, "-I" + INCLUDE, "-L" + LIBDIR, "-lmgpicola",
               "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            print(" ".join(cmd))
            sys.stdout.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("driver link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
