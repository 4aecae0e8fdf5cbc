"""Massive neutrinos on the CUDA path (the reference's MASSIVE_NEUTRINOS
build, scale dependent) on synthetic CAMB tables (tests/golden/camb_tables.py):

  - the per-step k-space neutrino density (src/auxPM.c:383-421) against the
    FP64 oracle applied to the same CDM delta(k) and stored IC field;
  - the CDM and total matter P(k) (src/auxPM.c:369-372, 423-426);
  - mgp_run against the reference's own run of the same parameters
    (tests/golden/ref_{lcdm,fofr}_nu.npz, made by make_golden.py) and the
    oracle's KDK loop.

FP32 vs FP64 bars as the scale-dependent tests: fields 1e-5 relative rms,
P(k) 1e-3, positions 1e-3 of the particle spacing.
"""
import os

import numpy as np
import pytest

import mgpicola as M
from golden import camb_tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def info(tmp_path_factory):
    return camb_tables.write_tables(str(tmp_path_factory.mktemp("camb")))


def params(info, model, N=32, Ns=16, box=128.0, **kw):
    d = dict(Nmesh=N, Nsample=Ns, Box=box, Seed=4242, Init_Redshift=19.0, pofk_nbins=16, pofk_bintype=0,
             pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0,
             input_pofk_is_for_lcdm=0, input_sigma8_is_for_lcdm=1, scaledependent=1, massive_neutrinos=1,
             nu_include_massive_neutrinos=1, nu_SumMassNuEV=camb_tables.SUM_MNU_EV, nu_FilenameTransferInfofile=info)
    if model == "fofr":
        d.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    d.update(kw)
    return M.default_params(**d)


def oracle_nu(info, p):
    return O.Neutrinos(info, p.Omega, p.OmegaBaryon, p.HubbleParam, p.PrimordialIndex, p.nu_SumMassNuEV,
                       p.nu_include_massive_neutrinos)


def rel_rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2) / np.mean(np.asarray(b, np.float64) ** 2)))


@pytest.mark.parametrize("A", [0.05, 0.6])
def test_neutrino_density_matches_oracle(info, A):
    """After get_displacements delta(k) is the total matter field:
    cdmfac delta_cdm(k) + OmegaNu/Omega N^3 T_nu(k, a)/T_cb(k, 1) delta_IC(k).
    The particles sit at the IC (a = 0.05); at A = 0.6 the neutrino term is
    grown further than the CDM field, a parity case only."""
    p = params(info, "lcdm")
    N = p.Nmesh
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.get_displacements(A)
        rho = ctx.grid(0)[:, :, :N].astype(np.float64)
        total = ctx.grid(1).astype(np.float64)
        ic = ctx.grid(7).astype(np.float64)
        k, pk_cdm, _, n = ctx.pofk()
        _, pk_tot, _, _ = ctx.pofk(total=True)
    nu = oracle_nu(info, p)
    ref = O.fft_r2c(rho)  # the CDM delta(k) of the same density (LCDM: no fifth force rewrites it)
    nu.add_density(A, N, p.Box, ref, ic)
    assert rel_rms(total, ref) < 1e-5
    m = n > 0
    m[0] = False
    _, pko, _, _ = O.pofk(ref, N, p.Nsample, p.Box, p.pofk_nbins, 0, 0, 0.0, 0.0)
    assert np.max(np.abs(pk_tot[m] - pko[m]) / pko[m]) < 1e-3
    # on small scales the neutrinos have free-streamed: P_tot -> cdmfac^2 P_cdm
    cdmfac = (p.Omega - nu.omega_nu) / p.Omega
    assert pk_tot[m][-1] / pk_cdm[m][-1] == pytest.approx(cdmfac ** 2, rel=2e-3)
    if A == 0.05:
        assert np.all(pk_tot[m] / pk_cdm[m] < 1.0)


def test_without_include_flag_nothing_is_added(info):
    p = params(info, "lcdm", nu_include_massive_neutrinos=0)
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.get_displacements(0.3)
        rho = ctx.grid(0)[:, :, :p.Nmesh].astype(np.float64)
        dk = ctx.grid(1).astype(np.float64)
        _, a, _, _ = ctx.pofk()
        _, b, _, _ = ctx.pofk(total=True)
    assert rel_rms(dk, O.fft_r2c(rho)) < 1e-5
    np.testing.assert_array_equal(a, b)


def _oracle_run(info, p, model, nsteps):
    nu = oracle_nu(info, p)
    rp = O.RunParams()
    if model == "fofr":
        rp.mg = O.make_mg(O.FOFR, p.Omega, mg_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0, scaledependent=1,
                          nu=nu)
    else:
        rp.mg = O.make_mg(O.LCDM, p.Omega, scaledependent=1, nu=nu)
    rp.pw = O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex,
                         sigma8=p.Sigma8, nu=nu)
    rp.ic = O.ICParams(p.Nmesh, p.Nsample, p.Box, p.Seed, 0, 0, 0, 1.0)
    rp.init_redshift = p.Init_Redshift
    rp.nsteps = nsteps
    rp.final_redshift = 0.0
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = p.pofk_nbins, 0, 0
    rp.pofk_kmin, rp.pofk_kmax = 0.0, 0.0
    rp.usecola = 1
    n = p.Nsample ** 3
    pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
    kb, pk, km, nm = (np.zeros(max(p.pofk_nbins, p.Nmesh)) for _ in range(4))
    nb = O.lib().orc_run(rp, pos, vel, kb, pk, km, nm)
    return pos, vel, (kb[:nb], pk[:nb], km[:nb], nm[:nb])


@pytest.mark.parametrize("model", ["lcdm", "fofr"])
def test_run_matches_reference_and_oracle(info, model, tmp_path):
    """mgp_run: GADGET snapshot at z = 0 and the CDM and total P(k) files
    against the reference's run (golden) and the oracle's loop."""
    N, Ns, box, nsteps = 32, 16, 128.0, 5
    out = str(tmp_path)
    p = params(info, model, N, Ns, box, OutputDir=out, FileBase="run", Noutputs=1)
    p.output_redshift[0], p.output_nsteps[0] = 0.0, nsteps
    with M.Context(p) as ctx:
        ctx.run(gadget=True)
    raw = open(os.path.join(out, "run_z0p000.0"), "rb").read()
    n = Ns ** 3
    pos = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3)
    vel = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3)
    pk_cdm = np.loadtxt(os.path.join(out, "pofk_run_z0.000_CDM.txt"))
    pk_tot = np.loadtxt(os.path.join(out, "pofk_run_z0.000_total.txt"))
    # the reference's own run (P(k) written with %10.5f, snapshots in float)
    g = np.load(os.path.join(GOLDEN, "ref_%s_nu.npz" % model))
    assert pk_cdm.shape == g["pk"].shape and pk_tot.shape == g["pk_total"].shape
    assert np.max(np.abs(pk_cdm[:, 1] - g["pk"][:, 1]) / g["pk"][:, 1]) < 1e-3
    assert np.max(np.abs(pk_tot[:, 1] - g["pk_total"][:, 1]) / g["pk_total"][:, 1]) < 1e-3
    idx = g["idx"]
    dx = np.abs(pos[idx] - g["pos"])
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box / Ns
    assert rel_rms(vel[idx], g["vel"]) < 1e-3
    # the oracle's loop: every particle, and the total P(k)
    opos, ovel, (kb, pko, kmo, no) = _oracle_run(info, p, model, nsteps)
    dx = np.abs(pos - opos)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box / Ns
    assert rel_rms(vel, 100.0 * ovel) < 1e-3
    m = no > 0
    m[0] = False
    assert np.max(np.abs(pk_tot[:, 1] - pko[m]) / pko[m]) < 1e-3


def test_neutrinos_need_scale_dependent_build(info):
    with pytest.raises(M.MGPError, match="SCALEDEPENDENT"):
        M.Context(params(info, "lcdm", scaledependent=0))
