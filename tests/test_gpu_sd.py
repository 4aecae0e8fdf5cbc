"""Scale-dependent growth (the reference's SCALEDEPENDENT build) on the CUDA
path against the FP64 oracle.

The oracle builds each LPT field as the reference does (full-mesh C2R per
order, trilinear read-out, mean removal: from_cdisp_store_to_ZA,
src/2LPT.c:1539-1735); the CUDA path folds the spectrum onto the Nsample
grid when Nmesh is a multiple of Nsample and follows the full-mesh algorithm
with the trilinear read-out otherwise (Nmesh/Nsample = 1.5, 2.5 here).  FP32 vs FP64: fields within 1e-4 relative rms, runs within 1e-3 in
P(k) and 1e-3 of the particle spacing in positions.
"""
import os
import struct

import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODELS = {
    "fofr": (dict(model=M.MODEL_FOFR, fofr0=1e-5, nfofr=1.0), O.FOFR, dict(fofr0=1e-5, nfofr=1.0)),
    "mbeta": (dict(model=M.MODEL_MBETA, assb_symm=0.5, beta_symm=1.0, range_symm=1.0), O.MBETA,
              dict(assb_symm=0.5, beta_symm=1.0, range_symm=1.0)),
}


def params(model, N=32, Ns=16, box=128.0, **kw):
    mk = MODELS[model][0]
    d = dict(Nmesh=N, Nsample=Ns, Box=box, Seed=4242, Init_Redshift=19.0, pofk_nbins=16, pofk_bintype=0,
             pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0,
             modified_gravity_active=1, include_screening=1, input_pofk_is_for_lcdm=0, scaledependent=1)
    d.update(mk)
    d.update(kw)
    return M.default_params(**d)


def oracle_mg(model):
    _, om, okw = MODELS[model]
    return O.make_mg(om, 0.267, mg_active=1, include_screening=1, scaledependent=1, **okw)


def power():
    return O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8)


def rel_rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2) / np.mean(np.asarray(b) ** 2)))


def oracle_fields(model, N, Ns, box, A, AFF, ftype, seed=4242):
    _, _, dk, s2 = O.ic_2lpt(N, Ns, box, seed, power(), want_k=True)
    oc = O.Cosmo(oracle_mg(model), 19.0, box, N)
    return (O.sd_field(oc, dk, N, Ns, box, A, AFF, ftype, 1) + O.sd_field(oc, s2, N, Ns, box, A, AFF, ftype, 2))


@pytest.mark.parametrize("model,N,Ns", [("fofr", 32, 16), ("mbeta", 32, 16), ("fofr", 32, 32), ("fofr", 48, 16),
                                        ("fofr", 24, 16), ("mbeta", 40, 16)])
def test_sd_ic_positions_match_oracle(model, N, Ns):
    box = 128.0
    p = params(model, N, Ns, box)
    ai = 1.0 / 20.0
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        pos, vel, d1, d2 = ctx.get_particles()
    D = oracle_fields(model, N, Ns, box, ai, ai, O.FIELD_D)
    q = np.stack(np.meshgrid(*(np.arange(Ns),) * 3, indexing="ij"), -1).reshape(-1, 3) * (box / Ns)
    ref = np.mod(q + D, box)
    dx = np.abs(pos - ref)
    dx = np.minimum(dx, box - dx)
    # x = q + D + D2 at a_i (main.c:297-301); FP32 fields vs FP64: 1e-4 of the spacing
    assert dx.max() < 1e-4 * box / Ns
    assert np.all(vel == 0)
    # the kick slot holds the D field after the IC
    assert rel_rms(d1, D) < 1e-4


@pytest.mark.parametrize("model,N,Ns", [("fofr", 32, 16), ("mbeta", 32, 16), ("fofr", 24, 16)])
def test_sd_step_fields_match_oracle(model, N, Ns):
    box = 128.0
    A, AFF = 0.4, 0.45
    p = params(model, N, Ns, box)
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.assign_fields(A, AFF, M.FIELD_ddDddy, M.FIELD_deltaD)
        _, _, kick, drift = ctx.get_particles()
        ctx.assign_fields(A, AFF, M.FIELD_D)
        _, _, dfield, _ = ctx.get_particles()
        with pytest.raises(M.MGPError):
            ctx.assign_fields(A, AFF, M.FIELD_D, M.FIELD_ddDddy)  # one slot
    assert rel_rms(kick, oracle_fields(model, N, Ns, box, A, AFF, O.FIELD_ddDddy)) < 1e-4
    assert rel_rms(drift, oracle_fields(model, N, Ns, box, A, AFF, O.FIELD_deltaD)) < 1e-4
    assert rel_rms(dfield, oracle_fields(model, N, Ns, box, A, AFF, O.FIELD_D)) < 1e-4


def test_sd_kick_requires_fields():
    p = params("fofr")
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.get_displacements(0.05)
        with pytest.raises(M.MGPError):
            ctx.kick_drift(0.05, 0.06, 0.05, 0.07)


def test_sd_rejects_odd_lattice():
    with pytest.raises(M.MGPError, match="even Nsample"):
        M.Context(params("fofr", N=30, Ns=15))


def _oracle_run(model, p, nsteps):
    rp = O.RunParams()
    rp.mg = oracle_mg(model)
    rp.pw = power()
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


@pytest.mark.parametrize("model,N", [("fofr", 32), ("mbeta", 32), ("fofr", 24)])
def test_sd_run_matches_oracle(model, N, tmp_path):
    """mgp_run with scale-dependent growth: the GADGET snapshot at z = 0 and
    the P(k) file against the oracle's KDK loop."""
    Ns, box, nsteps = 16, 128.0, 5
    out = str(tmp_path)
    p = params(model, N, Ns, box, OutputDir=out, FileBase="sd", Noutputs=1)
    p.output_redshift[0], p.output_nsteps[0] = 0.0, nsteps
    with M.Context(p) as ctx:
        ctx.run(gadget=True)
    opos, ovel, (kb, pko, kmo, no) = _oracle_run(model, p, nsteps)
    raw = open(os.path.join(out, "sd_z0p000.0"), "rb").read()
    n = Ns ** 3
    assert struct.unpack("<i", raw[264:268])[0] == 12 * n
    pos = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3)
    vel = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3)
    dx = np.abs(pos - opos)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box / Ns
    # GADGET velocities at a = 1: velfac * Hubble * v = 100 v (code units)
    assert rel_rms(vel, 100.0 * ovel) < 1e-3
    pk = np.loadtxt(os.path.join(out, "pofk_sd_z0.000_CDM.txt"))
    m = no > 0
    m[0] = False  # files start at bin 1 (compute_pofk.c:251)
    assert pk.shape[0] == m.sum()
    assert np.max(np.abs(pk[:, 1] - pko[m]) / pko[m]) < 1e-3


def test_sd_step_host_matches_device_step():
    """The host-buffer step with scale-dependent growth (chunked position
    upload, velocities on the side stream, LPT fields assigned by the step)
    against mgp_step on device-resident particles.  The host path carries
    positions as absolute float32 coordinates in [0, Box) between steps, as
    the reference's P[].Pos (ULP ~ 7.6e-6 Mpc/h at Box 128), where the
    device path keeps float displacements from the lattice; with the f(R)
    screening that allows 2e-5 relative rms in the velocities."""
    p = params("fofr")
    A0 = 1.0 / 20.0
    da = (1.0 - A0) / 5
    with M.Context(p) as c1, M.Context(p) as c2:
        c1.displacement_fields()
        c2.displacement_fields()
        pos, vel, d1, d2 = c1.get_particles()
        A, AI = A0, A0
        for _ in range(3):
            c1.step_host(A, AI, A + 0.5 * da, A + da, pos, vel, d1, d2)
            c2.step(A, AI, A + 0.5 * da, A + da)
            A, AI = A + da, A + 0.5 * da
        pos2, vel2, _, _ = c2.get_particles()
    box, Ns = p.Box, p.Nsample
    dx = np.abs(pos - pos2)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-5 * box / Ns
    assert rel_rms(vel, vel2) < 2e-5
