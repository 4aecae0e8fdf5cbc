"""The CUDA path's mgp_run against the reference's own runs.

tests/golden/ref_*.npz hold the output of MG-PICOLA's unmodified sources
compiled against single-rank shims and run here (tests/golden/make_golden.py):
the final CDM P(k) file (and the total one of the neutrino build; the
READICFROMFILE build starts from two GADGET-1 particle files), the
redshift-space multipole files (compute_RSD_powerspectrum,
src/compute_pofk.c:403-512) where the case asked for them, and a subsample of
the final GADGET snapshot.  Every case is rerun here through mgp_run with the
same parameters and white-noise stream (COLA or standard PM, linear or
logarithmic bins, one or two outputs, cube or sphere mode cut, P(k) and
sigma8 quoted for LCDM or for the model, LCDM growth factors, Eisenstein-Hu
or tabulated spectrum or transfer function, Mpc/h or kpc/h units).  FP32 path vs FP64 reference over 5-7
steps: P(k) within 1e-3 relative; multipoles within 1e-3 of max |P0| (P2 and
P4 cross zero); positions rms < 1e-3 of the particle spacing; velocities 1e-3
relative rms.
"""
import glob
import os

import numpy as np
import pytest

import mgpicola as M
from golden import camb_tables, particle_files, spectrum_table

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_*.npz")))


def _f(g, k, default=0.0):
    return float(g[k]) if k in g.files else default


def params_for(g, out, tmp):
    model = str(g["model"])
    d = dict(Nmesh=int(g["Nmesh"]), Nsample=int(g["Nsample"]), Box=float(g["Box"]), Seed=int(g["Seed"]),
             Init_Redshift=float(g["Init_Redshift"]), pofk_nbins=int(_f(g, "nbins", 16)),
             pofk_bintype=int(_f(g, "bintype")), pofk_kmin=_f(g, "kmin"), pofk_kmax=_f(g, "kmax"),
             pofk_compute_every_step=1, pofk_subtract_shotnoise=int(_f(g, "shotnoise")),
             pofk_compute_rsd_pofk=int(_f(g, "rsd")),
             input_pofk_is_for_lcdm=int(_f(g, "pofk_lcdm")), input_sigma8_is_for_lcdm=int(_f(g, "s8_lcdm", 1)),
             use_lcdm_growth_factors=int(_f(g, "lcdm_growth")), SphereMode=int(_f(g, "sphere")),
             amplitude_fixed_initial_condition=int(_f(g, "amplitude_fixed_initial_condition")),
             inverted_initial_condition=int(_f(g, "inverted_initial_condition")),
             Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8, PrimordialIndex=0.96,
             WhichSpectrum=int(_f(g, "which_spectrum", 2)), WhichTransfer=int(_f(g, "which_transfer")),
             UnitLength_in_cm=_f(g, "unit_length", 3.085678e24),
             InputSpectrum_UnitLength_in_cm=_f(g, "input_unit_length", 3.085678e24),
             UseCOLA=int(_f(g, "cola", 1)), OutputDir=out, FileBase="run",
             modified_gravity_active=int(_f(g, "modified_gravity_active")),
             include_screening=int(_f(g, "include_screening", 1)))
    if d["WhichSpectrum"] == 1:
        d["FileWithInputSpectrum"] = spectrum_table.write_pk_table(os.path.join(tmp, "pk_table.dat"))
    if d["WhichTransfer"] == 1:
        d["FileWithInputTransfer"] = spectrum_table.write_transfer_table(os.path.join(tmp, "t_table.dat"))
    if model == "FOFR_LCDM_IC":
        # two GADGET-1 files of the displaced lattice the fixture was made from
        d.update(ReadParticlesFromFile=1, TypeInputParticleFiles=3, NumInputParticleFiles=2, RamsesOutputNumber=0,
                 InputParticleFileDir=particle_files.write_ic_files(os.path.join(tmp, "ic"), d["Box"]),
                 InputParticleFilePrefix="ics")
    if model.startswith("FOFR"):  # FOFR, FOFR_LCDM, FOFRNU, FOFR_LCDM_IC, FOFR_LCDM_ASCII, FOFR_LCDM_W0WA
        d.update(model=M.MODEL_FOFR, fofr0=_f(g, "fofr0"), nfofr=_f(g, "nfofr"))
        if model == "FOFR_LCDM_W0WA":
            d.update(use_w0wa=1, w_0=_f(g, "w_0"), w_a=_f(g, "w_a"))
    elif model.startswith("DGP"):
        filt = {"DGP": M.FILTER_GAUSSIAN, "DGP_TOPHAT": M.FILTER_TOPHAT, "DGP_SHARPK": M.FILTER_SHARPK}[model]
        d.update(model=M.MODEL_DGP, rcH0_DGP=_f(g, "rcH0_DGP"), Rsmooth=_f(g, "Rsmooth"), smoothing_filter=filt)
    elif model == "BRANSDICKE":
        d.update(model=M.MODEL_BRANSDICKE, wBD=_f(g, "wBD"), Omegah2=_f(g, "Omegah2"), Omegarh2=_f(g, "Omegar2"),
                 Omegavh2=_f(g, "Omegav2"))
    elif model.startswith("MBETA"):
        d.update(model=M.MODEL_MBETA, range_symm=_f(g, "range_symm"), assb_symm=_f(g, "assb_symm"),
                 beta_symm=_f(g, "beta_symm"))
    if model in ("FOFR", "MBETA", "FOFRNU"):
        d.update(scaledependent=1)
    if model == "FOFRNU":
        d.update(massive_neutrinos=1, nu_include_massive_neutrinos=int(_f(g, "nu_include_massive_neutrinos")),
                 nu_SumMassNuEV=_f(g, "nu_SumMassNuEV"),
                 nu_FilenameTransferInfofile=camb_tables.write_tables(os.path.join(tmp, "camb")))
    p = M.default_params(**d)
    if int(_f(g, "z1steps")):
        # two outputs: z = 1, then z = 0
        p.Noutputs = 2
        p.output_redshift[0], p.output_nsteps[0] = 1.0, int(g["z1steps"])
        p.output_redshift[1], p.output_nsteps[1] = 0.0, int(g["nsteps"])
    else:
        p.Noutputs = 1
        p.output_redshift[0], p.output_nsteps[0] = 0.0, int(g["nsteps"])
    return p


def rel_rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2) / np.mean(np.asarray(b, np.float64) ** 2)))


def max_rel(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[4:-4] for p in GOLDEN])
def test_run_matches_reference_run(path, tmp_path):
    g = np.load(path)
    out = str(tmp_path / "out")
    os.makedirs(out)
    p = params_for(g, out, str(tmp_path))
    ascii_out = str(g["model"]).endswith("_ASCII")
    with M.Context(p) as ctx:
        ctx.run(gadget=not ascii_out)
    # the info file (Output_Info, src/main.c:1067-1099) as text
    if "info_txt" in g.files:
        assert open(os.path.join(out, "info_run_z0p000.txt")).read() == str(g["info_txt"])
    pk = np.loadtxt(os.path.join(out, "pofk_run_z0.000_CDM.txt"))
    assert pk.shape == g["pk"].shape
    np.testing.assert_allclose(pk[:, 0], g["pk"][:, 0], atol=6e-6)
    assert max_rel(pk[:, 1], g["pk"][:, 1]) < 1e-3
    if "pk_total" in g.files:
        tot = np.loadtxt(os.path.join(out, "pofk_run_z0.000_total.txt"))
        assert max_rel(tot[:, 1], g["pk_total"][:, 1]) < 1e-3
    rsd = [k for k in g.files if k.startswith("rsd_")]
    for key in rsd:
        ref = g[key]
        got = np.loadtxt(os.path.join(out, "pofk_RSD_run_z%s.txt" % key[4:]))
        assert got.shape == ref.shape, key
        np.testing.assert_allclose(got[:, 0], ref[:, 0], atol=6e-6)
        scale = np.abs(ref[:, 1]).max()
        # P0, P2, P4 and the y/z-LOS differences (sigma columns)
        assert np.abs(got[:, 1:] - ref[:, 1:]).max() < 1e-3 * scale, key
    snaps = [("z0p000", "pos", "vel")]
    if "pk_z1" in g.files:
        pk1 = np.loadtxt(os.path.join(out, "pofk_run_z1.000_CDM.txt"))
        assert max_rel(pk1[:, 1], g["pk_z1"][:, 1]) < 1e-3
        snaps.append(("z1p000", "pos_z1", "vel_z1"))
    n = p.Nsample ** 3
    idx = g["idx"]
    # snapshots are written in Mpc/h (lengthfac, src/main.c:913-977)
    box_out = p.Box * p.UnitLength_in_cm / 3.085678e24
    for tag, kp, kv in snaps:
        if ascii_out:
            # ASCII snapshot (src/main.c:1000-1025): the count, then %12.6f columns
            lines = open(os.path.join(out, "run_%s.0" % tag)).read().splitlines()
            assert lines[0] == str(g["ascii_first_line"])
            rows = np.array([[float(v) for v in l.split()] for l in lines[1:]])
            pos, vel = rows[:, :3], rows[:, 3:]
        else:
            raw = open(os.path.join(out, "run_%s.0" % tag), "rb").read()
            if tag == "z0p000" and "gadget_header" in g.files:
                # the GADGET-1 header block byte for byte (src/main.c:1106-1149)
                np.testing.assert_array_equal(np.frombuffer(raw[:264], dtype=np.uint8), g["gadget_header"])
            pos = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3)
            vel = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3)
        dx = np.abs(pos[idx] - g[kp])
        dx = np.minimum(dx, box_out - dx)
        assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box_out / p.Nsample, tag
        assert rel_rms(vel[idx], g[kv]) < 1e-3, tag


def test_golden_rsd_cases_present():
    names = [os.path.basename(p) for p in GOLDEN]
    assert "ref_lcdm_rsd.npz" in names and "ref_fofr_rsd.npz" in names
    g = np.load(os.path.join(os.path.dirname(GOLDEN[0]), "ref_fofr_rsd.npz"))
    assert len([k for k in g.files if k.startswith("rsd_")]) == 5  # four steps and the output
