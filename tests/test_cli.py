"""The command-line driver mgpicola_run, the drop-in for the reference's
MG_PICOLA_<MODEL> <ParameterFile> (src/main.c:33-57).

CPU: the usage message and exit status without a parameter file, unknown
models and options, and parser errors, all before any GPU work.
GPU: a golden case (the reference's DGP build with COMPUTE_POFK, run here
from its own sources) through a parameter file and the executable, invoked
by a link named MG_PICOLA_DGP; its P(k) file and GADGET snapshot match the
reference's within the bars of tests/test_gpu_golden.py.
"""
import os
import subprocess

import numpy as np
import pytest

import mgpicola as M

EXE = os.path.join(os.path.dirname(M.LIB_PATH), "mgpicola_run")


def run(args, **kw):
    return subprocess.run([EXE] + args, capture_output=True, text=True, timeout=300, **kw)


def test_usage_without_parameter_file():
    r = run([])
    assert r.returncode == 1
    assert r.stdout.startswith("Input parameters not found\nCall with <ParameterFile>\n")


def test_unknown_model_and_option(tmp_path):
    assert "MODEL NOPE is not recognized" in run(["-model", "NOPE", "x.txt"]).stderr
    assert "unknown option -bogus" in run(["-bogus", "x.txt"]).stderr
    link = tmp_path / "MG_PICOLA_NOPE"
    os.symlink(EXE, link)
    r = subprocess.run([str(link), "x.txt"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "MODEL NOPE is not recognized" in r.stderr


def test_parser_errors_exit_1(tmp_path):
    r = run([str(tmp_path / "missing.txt")])
    assert r.returncode == 1 and "Parameter file" in r.stderr and "not found" in r.stderr
    pf = tmp_path / "p.txt"
    pf.write_text("Nmesh 32\n")
    r = run(["-model", "FOFR_LCDM", str(pf)])
    assert r.returncode == 1 and "I miss a value for tag" in r.stderr


# parameter-file keys per model (read_param.c:167-265, user_defined_functions.h:233-405)
STD_KEYS = ["OutputDir", "FileBase", "OutputRedshiftFile", "NumFilesWrittenInParallel", "UseCOLA", "Buffer", "Nmesh",
            "Nsample", "Box", "Init_Redshift", "Seed", "SphereMode", "WhichSpectrum", "WhichTransfer",
            "FileWithInputSpectrum", "FileWithInputTransfer", "Omega", "OmegaBaryon", "HubbleParam", "Sigma8",
            "PrimordialIndex", "UnitVelocity_in_cm_per_s", "UnitLength_in_cm", "UnitMass_in_g",
            "InputSpectrum_UnitLength_in_cm"]
MG_KEYS = ["modified_gravity_active", "use_lcdm_growth_factors", "input_pofk_is_for_lcdm", "input_sigma8_is_for_lcdm",
           "inverted_initial_condition", "amplitude_fixed_initial_condition", "include_screening"]
POFK_KEYS = ["pofk_compute_every_step", "pofk_compute_rsd_pofk", "pofk_nbins", "pofk_bintype",
             "pofk_subtract_shotnoise", "pofk_kmin", "pofk_kmax"]


def write_paramfile(p, path, model_keys):
    zfile = str(path) + ".z"
    with open(zfile, "w") as f:
        for i in range(p.Noutputs):
            f.write("%.6f, %d\n" % (p.output_redshift[i], p.output_nsteps[i]))
    p.OutputRedshiftFile = zfile.encode()
    with open(path, "w") as f:
        for k in MG_KEYS + model_keys + POFK_KEYS + STD_KEYS:
            v = getattr(p, k)
            if isinstance(v, bytes):
                v = v.decode() or "none"
            elif isinstance(v, float):
                v = repr(v)
            f.write("%s %s\n" % (k, v))
    return str(path)


@pytest.mark.gpu
def test_golden_dgp_case_through_the_executable(tmp_path):
    from test_gpu_golden import params_for, rel_rms, max_rel

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_dgp.npz"))
    out = str(tmp_path / "out")
    p = params_for(g, out, str(tmp_path))
    pf = write_paramfile(p, tmp_path / "dgp.txt", ["Rsmooth", "rcH0_DGP"])
    link = tmp_path / "MG_PICOLA_DGP"
    os.symlink(EXE, link)
    r = subprocess.run([str(link), "-pofk", pf], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    pk = np.loadtxt(os.path.join(out, "pofk_run_z0.000_CDM.txt"))
    assert pk.shape == g["pk"].shape
    np.testing.assert_allclose(pk[:, 0], g["pk"][:, 0], atol=6e-6)
    assert max_rel(pk[:, 1], g["pk"][:, 1]) < 1e-3
    n = p.Nsample ** 3
    raw = open(os.path.join(out, "run_z0p000.0"), "rb").read()
    if "gadget_header" in g.files:
        np.testing.assert_array_equal(np.frombuffer(raw[:264], dtype=np.uint8), g["gadget_header"])
    pos = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3)
    vel = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3)
    idx = g["idx"]
    dx = np.abs(pos[idx] - g["pos"])
    dx = np.minimum(dx, p.Box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * p.Box / p.Nsample
    assert rel_rms(vel[idx], g["vel"]) < 1e-3
