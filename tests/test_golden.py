"""The FP64 oracle against golden fixtures produced by MG-PICOLA's own code.

tests/golden/ref_*.npz were written by tests/golden/make_golden.py, which
compiles the reference's unmodified sources against single-rank shims and
runs them.  Tolerances reflect the reference's output formats: P(k) is
written with %10.5f (absolute 5e-6) and snapshots in float32.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from golden import camb_tables, particle_files, spectrum_table

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_*.npz")))


def oracle_run(g, tmpdir=None):
    model = str(g["model"])
    nu = None
    if model == "FOFRNU":
        # the synthetic CAMB tables the fixture was made with
        info = camb_tables.write_tables(os.path.join(str(tmpdir), "camb"))
        nu = O.Neutrinos(info, 0.267, 0.049, 0.71, 0.96, float(g["nu_SumMassNuEV"]),
                         int(g["nu_include_massive_neutrinos"]))
    active = int(g["modified_gravity_active"])
    scr = int(g["include_screening"])
    if model.startswith("DGP"):
        # GAUSSIANFILTER (the DGP build), TOPHATFILTER or SHARPKFILTER
        filt = {"DGP": 1, "DGP_TOPHAT": 2, "DGP_SHARPK": 3}[model]
        mg = O.make_mg(O.DGP, 0.267, mg_active=active, include_screening=scr, rcH0=float(g["rcH0_DGP"]),
                       rsmooth=float(g["Rsmooth"]), smoothing_filter=filt)
    elif model == "BRANSDICKE":
        mg = O.make_mg(O.JBD_GEFF, 0.267, mg_active=active, wBD=float(g["wBD"]), Omegah2=float(g["Omegah2"]),
                       Omegarh2=float(g["Omegar2"]), Omegavh2=float(g["Omegav2"]))
    elif model.startswith("MBETA"):
        mg = O.make_mg(O.MBETA, 0.267, mg_active=active, include_screening=scr, assb_symm=float(g["assb_symm"]),
                       beta_symm=float(g["beta_symm"]), range_symm=float(g["range_symm"]),
                       scaledependent=int(model == "MBETA"))
    else:
        w0wa = dict(use_w0wa=1, w0=float(g["w_0"]), wa=float(g["w_a"])) if model == "FOFR_LCDM_W0WA" else {}
        mg = O.make_mg(O.FOFR, 0.267, mg_active=active, include_screening=scr, fofr0=float(g["fofr0"]),
                       nfofr=float(g["nfofr"]), scaledependent=int(model in ("FOFR", "FOFRNU")), nu=nu,
                       use_lcdm_growth=int(g["lcdm_growth"]) if "lcdm_growth" in g.files else 0, **w0wa)
    N, Ns, box = int(g["Nmesh"]), int(g["Nsample"]), float(g["Box"])
    rp = O.RunParams()
    rp.mg = mg
    table = None
    if "which_spectrum" in g.files and int(g["which_spectrum"]) == 1:
        # the tabulated spectrum the fixture was made with, as log10 pairs
        path = spectrum_table.write_pk_table(os.path.join(str(tmpdir), "pk_table.dat"))
        kp = np.loadtxt(path)
        table = (np.ascontiguousarray(np.log10(kp[:, 0])), np.ascontiguousarray(np.log10(kp[:, 1])))
        pw = O.Power()
        pw.which_spectrum, pw.omega, pw.omega_b, pw.h, pw.ns, pw.sigma8 = 1, 0.267, 0.049, 0.71, 0.96, 0.8
        pw.ntab = len(kp)
        pw.tab_logk = table[0].ctypes.data_as(C.POINTER(C.c_double))
        pw.tab_logP = table[1].ctypes.data_as(C.POINTER(C.c_double))
        O.lib().orc_power_init(C.byref(pw))
        rp.pw = pw
    else:
        rp.pw = O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8, nu=nu)
    if model == "BRANSDICKE":
        # normalised with the file's Omega/h, evaluated with the background's
        rp.pw.omega, rp.pw.h = mg.omega, float(np.sqrt(mg.Omegah2 / mg.omega))
    rescale = 1.0
    if "pofk_lcdm" in g.files and int(g["pofk_lcdm"]) and active:
        # 2LPT.c:392-407: P(k) x mg_pofk_ratio(k, 1) (k-independent without
        # scale-dependent growth), / (sigma8_MG / sigma8_LCDM)^2
        cos = O.Cosmo(mg, float(g["Init_Redshift"]))
        rescale = cos.mg_pofk_ratio(0.1, 1.0)
        if not int(g["s8_lcdm"]):
            rescale /= O.lib().orc_mg_sigma8_enh(cos.h, C.byref(rp.pw), 1.0) ** 2
    sphere = int(g["sphere"]) if "sphere" in g.files else 0
    rp.ic = O.ICParams(N, Ns, box, int(g["Seed"]), sphere, int(g["amplitude_fixed_initial_condition"]),
                       int(g["inverted_initial_condition"]), rescale)
    rp.init_redshift = float(g["Init_Redshift"])
    rp.nsteps = int(g["nsteps"])
    rp.final_redshift = 0.0
    def opt(k, default):
        return type(default)(g[k]) if k in g.files else default

    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = opt("nbins", 16), opt("bintype", 0), opt("shotnoise", 0)
    rp.pofk_kmin, rp.pofk_kmax = opt("kmin", 0.0), opt("kmax", 0.0)
    rp.usecola = opt("cola", 1)
    keep = []
    if "ReadParticlesFromFile" in g.files and int(g["ReadParticlesFromFile"]):
        # the particle files the fixture was made from, read as the reference
        # reads them (float positions / BoxSize, wrapped)
        pos = particle_files.displaced_lattice(20, box)
        u = (pos.astype(np.float64) * (1.0 / box)).astype(np.float32)
        u = np.where(u >= 1.0, (u - np.float32(1.0)).astype(np.float32), u).astype(np.float64)
        resc = np.ones(3 * (N // 2) ** 2 + 1)
        keep += [np.ascontiguousarray(u), resc]
        rp.ic_pos01, rp.ic_n, rp.ic_rescale_rk = keep[0].ctypes.data, len(u), resc.ctypes.data
    n = Ns ** 3
    pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
    kb, pk, km, nm = (np.zeros(N) for _ in range(4))
    nb = O.lib().orc_run(rp, pos, vel, kb, pk, km, nm)
    del nu, table  # the tables stay alive through rp.mg / rp.pw until here
    return (kb[:nb], pk[:nb], km[:nb], nm[:nb]), pos, vel, box


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[4:-4] for p in GOLDEN])
def test_oracle_matches_reference_run(path, tmp_path):
    g = np.load(path)
    if "z1steps" in g.files and int(g["z1steps"]):
        pytest.skip("two outputs: the oracle's loop has one; mgp_run is checked against this case directly")
    if ("which_transfer" in g.files and int(g["which_transfer"])) or (
            "unit_length" in g.files and float(g["unit_length"]) != 3.085678e24):
        pytest.skip("tabulated transfer function / kpc units: mgp_run is checked against this case directly")
    (kb, pk, km, nm), pos, vel, box = oracle_run(g, tmp_path)
    m = nm > 0
    m[0] = False  # the reference writes bins from 1 (compute_pofk.c:251)
    # with massive neutrinos the oracle's P(k) is the total matter one
    ref = g["pk_total"] if "pk_total" in g else g["pk"]
    assert ref.shape[0] == m.sum()
    np.testing.assert_allclose(kb[m], ref[:, 0], atol=6e-6)
    np.testing.assert_allclose(pk[m], ref[:, 1], rtol=1e-6, atol=6e-6)
    np.testing.assert_allclose(km[m], ref[:, 2], atol=6e-6)
    idx = g["idx"]
    dx = np.abs(pos[idx] - g["pos"])
    dx = np.minimum(dx, box - dx)
    assert dx.max() < 2e-5 * box
    # GADGET velocities: velfac * Hubble / a^1.5 * v, a = 1, Hubble = 100 (code units)
    v = 100.0 * vel[idx]
    assert np.abs(g["vel"] - v).max() < 1e-6 * np.abs(v).max() + 1e-5
