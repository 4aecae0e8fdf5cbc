"""Parity at the benchmark workloads' own sizes, through the C ABI.

- LCDM 64^3 particles / 128^3 mesh (Box 256, 10 linear-in-a steps z = 19 -> 0,
  seed 5001, 64 linear bins over [2 pi/Box, k_Nyquist], shot noise
  subtracted) against the FP64 oracle run in the test.
- nDGP rcH0 = 1 with density screening at the 512^3/1024^3 workload's cell
  size (256^3 / 512^3, Box 512, its full 50-step schedule, seed 5003,
  amplitude-fixed ICs) against the stored FP64 oracle run
  (tests/golden/orc_ndgp_256_512_50.npz).
- The 512^3 / 1024^3 workload itself at the start of step 3 of its 50-step
  schedule against the stored FP64 oracle run
  (tests/golden/orc_ndgp_512_1024_3.npz).

Bars (FP32 path against FP64): P(k) within 1e-3 relative for every bin with
k <= 0.5 h/Mpc (the stated accuracy target), and the rms particle position
difference below the bound given at each assert, in units of the particle
spacing.  Mode counts and bin wave numbers are integer/exact work.
"""
import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O
from tests.golden import oracle_runs as R

pytestmark = pytest.mark.gpu


def test_lcdm_64_128_ten_steps_matches_oracle():
    N, Ns, box, nsteps, nbins, seed = 128, 64, 256.0, 10, 64, 5001
    kmin, kmax = 2 * np.pi / box, np.pi * N / box
    p = M.default_params(Nmesh=N, Nsample=Ns, Box=box, Seed=seed, Init_Redshift=19.0, pofk_compute_every_step=1,
                         pofk_nbins=nbins, pofk_bintype=0, pofk_kmin=kmin, pofk_kmax=kmax, pofk_subtract_shotnoise=1,
                         WhichSpectrum=2, UseCOLA=1, Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8,
                         PrimordialIndex=0.96)
    A0 = 1.0 / 20.0
    da = (1.0 - A0) / nsteps
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        A, AI = A0, A0
        for _ in range(nsteps):
            ctx.step(A, AI, A + 0.5 * da, A + da)
            A, AI = A + da, A + 0.5 * da
        ctx.get_displacements(A)
        k, pk, km, n = ctx.pofk()
        pos = ctx.get_particles()[0]
    rp = O.RunParams()
    rp.mg = O.make_mg(O.LCDM, 0.267)
    rp.pw = O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8)
    rp.ic = O.ICParams(N, Ns, box, seed, 0, 0, 0, 1.0)
    rp.init_redshift, rp.nsteps, rp.final_redshift = 19.0, nsteps, 0.0
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = nbins, 0, 1
    rp.pofk_kmin, rp.pofk_kmax, rp.usecola = kmin, kmax, 1
    opos, ovel = np.zeros((Ns ** 3, 3)), np.zeros((Ns ** 3, 3))
    kb, po, kmo, no = (np.zeros(max(nbins, N)) for _ in range(4))
    nb = O.lib().orc_run(rp, opos, ovel, kb, po, kmo, no)
    assert nb == nbins == len(pk)
    np.testing.assert_array_equal(n, no[:nb])
    np.testing.assert_allclose(k, kb[:nb], rtol=1e-14)
    m = (no[:nb] > 0) & (kb[:nb] > 0) & (kb[:nb] <= 0.5)
    assert m.sum() >= 15
    assert np.max(np.abs(pk[m] / po[:nb][m] - 1.0)) < 1e-3
    dx = np.abs(pos.astype(np.float64) - opos)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box / Ns


def _fixture_case(name):
    ref = R.load(name)
    if ref is None:
        pytest.skip("stored oracle run tests/golden/orc_%s.npz not present" % name)
    c = R.CASES[name]
    with M.Context(R.gpu_params(M, c)) as ctx:
        k, pk, pos = R.gpu_run(ctx, c)
    np.testing.assert_allclose(k, ref["k"], rtol=1e-14)
    return R.compare(ref, k, pk, pos)


def test_ndgp_workload_cell_size_full_schedule_matches_oracle():
    r = _fixture_case("ndgp_256_512_50")
    assert r["bins"] >= 35
    assert r["max_rel_err"] < 1e-3, r
    # 50 steps to z = 0 (measured 5.5e-6 of the spacing in lattice order)
    assert r["pos_rms_over_spacing"] < 1e-4, r


def test_ndgp_512_1024_workload_first_steps_match_oracle():
    r = _fixture_case("ndgp_512_1024_3")
    assert r["bins"] >= 75
    assert r["max_rel_err"] < 1e-3, r
    assert r["pos_rms_over_spacing"] < 1e-3, r
