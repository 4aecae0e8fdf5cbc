"""Batches of independent boxes (mgp_batch_*) against the FP64 oracle run of
each box on its own.

Every box of a batch has its own seed, IC flags and f(R) |fR0| (or nDGP
rcH0); the batch runs all of them in lock step in one captured CUDA graph.
Bar as the single-box runs: final P(k) within 1e-3 of the oracle, positions
rms < 1e-3 of the particle spacing, every recorded P(k) step reproduced on a
replay of the graph (to 1e-6 at the first step, 1e-4 later: float atomics
in the CIC deposit are not ordered).
"""
import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def params(**kw):
    d = dict(Nmesh=32, Nsample=16, Box=128.0, Seed=6001, Init_Redshift=19.0, pofk_nbins=16, pofk_bintype=0,
             pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0,
             input_pofk_is_for_lcdm=0)
    d.update(kw)
    return M.default_params(**d)


def oracle_run(p, mg, seed, inverted, fixed, nsteps):
    rp = O.RunParams()
    rp.mg = mg
    rp.pw = O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8)
    rp.ic = O.ICParams(p.Nmesh, p.Nsample, p.Box, seed, 0, fixed, inverted, 1.0)
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
    return pos, (kb[:nb], pk[:nb], km[:nb], nm[:nb])


def check_box(batch, b, p, mg, box, nsteps):
    pos, _ = batch.particles(b)
    k, pk, km, n = batch.pofk(b, nsteps)
    opos, (kb, pko, kmo, no) = oracle_run(p, mg, box["Seed"], box.get("inverted", 0), box.get("fixed", 0), nsteps)
    np.testing.assert_array_equal(n, no)
    m = no > 0
    m[0] = False
    assert np.max(np.abs(pk[m] - pko[m]) / pko[m]) < 1e-3
    dx = np.abs(pos - opos)
    dx = np.minimum(dx, p.Box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * p.Box / p.Nsample


def test_batch_fofr_sweep_matches_oracle():
    nsteps = 5
    p = params(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    boxes = [dict(Seed=6001, inverted=0, fofr0=1e-6), dict(Seed=6001, inverted=1, fofr0=1e-6),
             dict(Seed=6002, inverted=0, fofr0=1e-4), dict(Seed=6002, inverted=1, fofr0=1e-4, fixed=1)]
    with M.Batch(p, boxes) as batch:
        batch.run(nsteps)
        assert batch.graph_nodes() > 0
        first = [batch.pofk(b, s)[1].copy() for b in range(len(boxes)) for s in range(nsteps + 1)]
        for b, box in enumerate(boxes):
            mg = O.make_mg(O.FOFR, 0.267, fofr0=box["fofr0"], nfofr=1.0)
            check_box(batch, b, p, mg, box, nsteps)
        # the same graph replayed after fresh ICs gives the same numbers, up
        # to the order of the CIC's float atomics: 1e-6 at the first step,
        # grown by the nonlinear evolution to < 1e-4 after five steps
        batch.run(nsteps)
        again = [batch.pofk(b, s)[1] for b in range(len(boxes)) for s in range(nsteps + 1)]
    for i, (x, y) in enumerate(zip(first, again)):
        # bin 0 holds only the k = 0 mode (zero up to rounding)
        np.testing.assert_allclose(x[1:], y[1:], rtol=1e-6 if i % (nsteps + 1) == 0 else 1e-4, atol=0)


def test_batch_dgp_matches_oracle():
    nsteps = 4
    p = params(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1, rcH0_DGP=1.0, Rsmooth=1.0,
               smoothing_filter=M.FILTER_GAUSSIAN)
    boxes = [dict(Seed=7001, rcH0=0.5), dict(Seed=7002, rcH0=2.0), dict(Seed=7003, rcH0=1.0)]
    with M.Batch(p, boxes) as batch:
        batch.run(nsteps)
        for b, box in enumerate(boxes):
            mg = O.make_mg(O.DGP, 0.267, rcH0=box["rcH0"], rsmooth=1.0)
            check_box(batch, b, p, mg, box, nsteps)


def test_batch_lcdm_matches_single_box():
    nsteps = 3
    p = params()
    boxes = [dict(Seed=5001), dict(Seed=5002)]
    with M.Batch(p, boxes) as batch:
        batch.run(nsteps)
        for b, box in enumerate(boxes):
            check_box(batch, b, p, O.make_mg(O.LCDM, 0.267), box, nsteps)


def test_batch_rejects_single_box_calls():
    p = params()
    with M.Batch(p, [dict(Seed=1), dict(Seed=2)]) as batch:
        ctx = M.Context.__new__(M.Context)
        ctx.h = batch.h
        with pytest.raises(M.MGPError):
            ctx.get_displacements(0.1)
        ctx.h = None


def test_batch_autotune_keeps_parity():
    """The autotuner changes launch shapes only: after it picks the budgets
    (each a candidate of its set), every box still matches its oracle run, and
    a hand-set extreme budget (1 block per SM everywhere) too."""
    nsteps = 4
    p = params(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    boxes = [dict(Seed=6011, inverted=0, fofr0=1e-5), dict(Seed=6012, inverted=1, fofr0=3e-6)]
    with M.Batch(p, boxes) as batch:
        assert batch.tuning() == [8, 8, 8, 4] and batch.deposit_tiles() == 0
        ms = batch.autotune(nsteps)
        t = batch.tuning()
        assert ms > 0 and all(x in (1, 2, 4, 8, 16, 32) for x in t) and t[3] <= 16
        assert batch.deposit_tiles() in (0, 8, 16)
        batch.run(nsteps)
        for b, box in enumerate(boxes):
            check_box(batch, b, p, O.make_mg(O.FOFR, 0.267, fofr0=box["fofr0"], nfofr=1.0), box, nsteps)
        batch.set_tuning([1, 1, 1, 1])
        batch.run(nsteps)
        for b, box in enumerate(boxes):
            check_box(batch, b, p, O.make_mg(O.FOFR, 0.267, fofr0=box["fofr0"], nfofr=1.0), box, nsteps)
        with pytest.raises(M.MGPError):
            batch.set_tuning([0, 8, 8, 4])


@pytest.mark.parametrize("side", [8, 16])
def test_batch_tile_deposit_matches_oracle(side):
    """The tile deposit of a batch (all boxes' particles counted and bucketed
    by tile inside the graph, per-tile shared-memory sums) against each box's
    oracle run, and against the lattice-order deposit of the same batch: the
    P(k) of the first step agrees to float rounding (the two deposits sum in
    different orders)."""
    nsteps = 4
    p = params(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    boxes = [dict(Seed=6021, inverted=0, fofr0=1e-5), dict(Seed=6022, inverted=1, fofr0=1e-4),
             dict(Seed=6023, inverted=0, fofr0=1e-6)]
    with M.Batch(p, boxes) as batch:
        batch.run(nsteps)
        lat = [batch.pofk(b, 0)[1].copy() for b in range(len(boxes))]
        batch.set_deposit_tiles(side)
        assert batch.deposit_tiles() == side
        batch.run(nsteps)
        for b, box in enumerate(boxes):
            check_box(batch, b, p, O.make_mg(O.FOFR, 0.267, fofr0=box["fofr0"], nfofr=1.0), box, nsteps)
            np.testing.assert_allclose(batch.pofk(b, 0)[1][1:], lat[b][1:], rtol=1e-5, atol=0)
        batch.set_deposit_tiles(0)
        assert batch.deposit_tiles() == 0
        for bad in (4, 12, 24, -8):
            with pytest.raises(M.MGPError):
                batch.set_deposit_tiles(bad)


def test_batch_tile_deposit_rejects_meshes_it_does_not_divide():
    p = params(Nmesh=40, Nsample=20)
    with M.Batch(p, [dict(Seed=1), dict(Seed=2)]) as batch:
        batch.set_deposit_tiles(8)
        with pytest.raises(M.MGPError, match="divide"):
            batch.set_deposit_tiles(16)
