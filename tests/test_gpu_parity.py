"""Parity of the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances: the CUDA path computes in FP32 (grids, FFTs, particles) and the
oracle in FP64, so comparisons are relative rms / max errors with the bound
stated at each assert.  Bin indices, mode counts and lattice bookkeeping are
integer work and compared exactly.
"""
import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def params(N=32, Ns=16, box=128.0, **kw):
    d = dict(Nmesh=N, Nsample=Ns, Box=box, Seed=5001, Init_Redshift=19.0, pofk_nbins=16, pofk_bintype=0,
             pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0)
    d.update(kw)
    return M.default_params(**d)


def power_for(p):
    return O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex,
                        sigma8=p.Sigma8)


def rel_rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2) / np.mean(np.asarray(b) ** 2)))


def random_particles(Ns, box, seed=1, spread=0.3):
    """Lattice + random displacement (as COLA particles), plus D1/D2/vel."""
    rng = np.random.default_rng(seed)
    n = Ns ** 3
    q = np.stack(np.meshgrid(*(np.arange(Ns),) * 3, indexing="ij"), -1).reshape(-1, 3) * (box / Ns)
    disp = rng.normal(0, spread * box / Ns, (n, 3))
    pos = np.mod(q + disp, box).astype(np.float32)
    pos[pos >= box] = 0.0
    vel = rng.normal(0, 10.0, (n, 3)).astype(np.float32)
    d1 = rng.normal(0, 2.0, (n, 3)).astype(np.float32)
    d2 = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    return pos, vel, d1, d2


@pytest.mark.parametrize("N,Ns,fixed,inverted", [(32, 16, 0, 0), (32, 32, 1, 0), (32, 16, 0, 1), (24, 12, 0, 0)])
def test_ic_displacements_match_oracle(N, Ns, fixed, inverted):
    box = 100.0
    p = params(N, Ns, box, amplitude_fixed_initial_condition=fixed, inverted_initial_condition=inverted, Seed=777)
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        pos, vel, d1, d2 = ctx.get_particles()
        Di = ctx.growth(0, 1 / 20.0)
        Di2 = ctx.growth(3, 1 / 20.0)
    D1, D2 = O.ic_2lpt(N, Ns, box, 777, power_for(p), fixed=fixed, inverted=inverted)
    # FP32 FFTs of an FP64 field: relative rms bound 1e-5 (ZA) and 1e-4 (2LPT)
    assert rel_rms(d1, D1) < 1e-5
    assert rel_rms(d2, D2) < 1e-4
    assert np.all(vel == 0)
    q = np.stack(np.meshgrid(*(np.arange(Ns),) * 3, indexing="ij"), -1).reshape(-1, 3) * (box / Ns)
    ref = np.mod(q + D1 * Di + D2 * Di2, box)
    dx = np.abs(pos - ref)
    dx = np.minimum(dx, box - dx)
    assert dx.max() < 1e-4 * box / Ns


def test_cic_density_matches_oracle():
    N, Ns, box = 32, 16, 64.0
    p = params(N, Ns, box)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=3)
    # edge cases: particles on the box boundary, on cell corners and at 0
    pos[0] = [0.0, 0.0, 0.0]
    pos[1] = [np.nextafter(np.float32(box), np.float32(0))] * 3
    pos[2] = [2.0, 4.0, 6.0]  # exact grid points (cell = 2 Mpc/h)
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel, d1, d2)
        ctx.get_displacements(0.5)
        rho = ctx.grid(0)
    ref = O.cic(pos.astype(np.float64), N, Ns, box)
    # mass conservation of the deposit: mean of delta is zero
    assert abs(rho[:, :, :N].astype(np.float64).mean()) < 1e-6
    err = np.abs(rho[:, :, :N] - ref[:, :, :N]).max()
    assert err < 2e-5 * np.abs(ref[:, :, :N]).max()


@pytest.mark.parametrize("N,Ns,spread", [(32, 16, 0.3), (64, 32, 3.0), (128, 64, 8.0), (48, 32, 1.0)])
def test_tile_deposit_matches_lattice_order_deposit(N, Ns, spread):
    """The cell-tile deposit (particles bucketed by 8^3 or 16^3-cell tiles,
    shared-memory tiles added with float2 reductions) against the deposit in
    lattice order, and both against the oracle; large displacements put
    particles far from their lattice tile and on tile faces and box edges."""
    box = 2.0 * N
    p = params(N, Ns, box)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=11, spread=spread)
    pos[0] = [0.0, 0.0, 0.0]
    pos[1] = [np.nextafter(np.float32(box), np.float32(0))] * 3
    pos[2] = [32.0, 32.0, 32.0]  # a tile corner (cell 16)
    rho = []
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel, d1, d2)
        # tile deposit with the arrays in lattice order, and the deposit in
        # lattice order
        for tiles in (1, 0):
            ctx.set_particle_order(tiles)
            ctx.get_displacements(0.5)
            rho.append(ctx.grid(0)[:, :, :N].astype(np.float64))
        # the tile kick (here over a zero interval, without drift) rewrites
        # the arrays in the deposit's tile order; the deposit from those
        # arrays, and the particles handed back in lattice order
        ctx.set_particle_order(2)
        ctx.get_displacements(0.5)
        ctx.kick_drift(0.5, 0.5, 0.5, 0.5, drift=False)
        ctx.get_displacements(0.5)
        rho.append(ctx.grid(0)[:, :, :N].astype(np.float64))
        back = ctx.get_particles()
    ref = O.cic(pos.astype(np.float64), N, Ns, box)[:, :, :N]
    scale = np.abs(ref).max()
    for r in (rho[0], rho[2]):
        assert np.abs(r - rho[1]).max() < 2e-6 * scale
    assert np.abs(rho[0] - ref).max() < 2e-5 * scale
    assert abs(rho[0].mean()) < 1e-6
    dx = np.abs(back[0] - pos)
    assert np.minimum(dx, box - dx).max() < 1e-4 * box / Ns
    np.testing.assert_allclose(back[1], vel, rtol=1e-6, atol=1e-5)
    np.testing.assert_array_equal(back[2], d1)
    np.testing.assert_array_equal(back[3], d2)


# 16^3 tiles, power-of-two lattice; 8^3 tiles, general lattice; 8 x 8 x 64 tiles (meshes of 512 and more)
@pytest.mark.parametrize("N,Ns", [(64, 32), (48, 24), (512, 64)])
@pytest.mark.parametrize("tiles", [2, 1])  # tile deposit and kick (the default); tile deposit only
def test_tile_order_run_matches_lattice_order_run(tiles, N, Ns):
    """Five KDK steps with the cell-tile particle order (tile deposit; the
    kick per tile with the arrays rewritten in tile order every step, or the
    arrays kept in lattice order) against the lattice order: the same run up
    to float summation order."""
    box, nsteps = 2.0 * N, 5
    p = params(N, Ns, box)
    out = []
    for tiles in (tiles, 0):
        with M.Context(p) as ctx:
            ctx.set_particle_order(tiles)
            ctx.displacement_fields()
            A, AI = 0.05, 0.05
            da = (1.0 - A) / nsteps
            for _ in range(nsteps):
                ctx.step(A, AI, A + 0.5 * da, A + da)
                A, AI = A + da, A + 0.5 * da
            ctx.get_displacements(A)
            out.append((ctx.pofk(), ctx.get_particles()))
    (k0, pk0, _, n0), (pos0, vel0, _, _) = out[0]
    (k1, pk1, _, n1), (pos1, vel1, _, _) = out[1]
    np.testing.assert_array_equal(n0, n1)
    m = n0 > 0
    m[0] = False
    assert np.max(np.abs(pk0[m] / pk1[m] - 1)) < 1e-5
    dx = np.abs(pos0 - pos1)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-5 * box / Ns
    assert rel_rms(vel0, vel1) < 1e-5


@pytest.mark.parametrize("bintype,nbins,kmin,kmax", [(0, 16, 0.0, 0.0), (1, 12, 0.05, 1.5), (0, 40, 0.1, 0.9)])
def test_pofk_matches_oracle(bintype, nbins, kmin, kmax):
    N, Ns, box = 32, 16, 64.0
    p = params(N, Ns, box, pofk_bintype=bintype, pofk_nbins=nbins, pofk_kmin=kmin, pofk_kmax=kmax,
               pofk_subtract_shotnoise=1)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=4, spread=0.8)
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel, d1, d2)
        ctx.get_displacements(0.5)
        k, pk, km, n = ctx.pofk()
    g = O.cic(pos.astype(np.float64), N, Ns, box)
    O.lib().orc_fft_r2c(N, g)
    kb, pko, kmo, no = O.pofk(g, N, Ns, box, nbins, bintype, 1, kmin, kmax)
    assert len(k) == len(kb)
    np.testing.assert_array_equal(n, no)          # integer mode counts, exact
    np.testing.assert_allclose(k, kb, rtol=1e-14)  # bin k values
    np.testing.assert_allclose(km[n > 0], kmo[no > 0], rtol=1e-12)
    # P(k) includes shot-noise subtraction: compare the raw power; the bin that
    # holds only the k = 0 mode has (numerically) zero power and is skipped
    shot = (box / Ns) ** 3
    raw, rawo = pk + shot, pko + shot
    m = (no > 0) & (rawo > 1e-6 * rawo.max())
    assert np.max(np.abs(raw[m] - rawo[m]) / rawo[m]) < 2e-6


def test_forces_match_oracle():
    N, Ns, box = 32, 16, 64.0
    p = params(N, Ns, box)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=5, spread=0.6)
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel, d1, d2)
        ctx.get_displacements(0.5)
        f = [ctx.grid(w)[:, :, :N] for w in (2, 3, 4)]
    g = O.cic(pos.astype(np.float64), N, Ns, box)
    O.lib().orc_fft_r2c(N, g)
    fo = O.forces_kspace(g, N, box)
    for a in range(3):
        O.lib().orc_fft_c2r(N, fo[a])
        assert rel_rms(f[a], fo[a][:, :, :N]) < 1e-5


@pytest.mark.parametrize("N,Ns,tiles", [(32, 16, 2), (32, 16, 0), (64, 32, 2), (64, 32, 1), (48, 24, 2)])
def test_kick_drift_matches_oracle(N, Ns, tiles):
    """MtoParticles + Kick + Drift against the oracle: per cell tile with the
    forces staged in shared memory (order 2, the default; 8^3 and 16^3
    tiles), and in array order (orders 0 and 1)."""
    box = 2.0 * N
    p = params(N, Ns, box)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=6, spread=0.4)
    A, AI, AF, AFF = 0.30, 0.28, 0.32, 0.34
    with M.Context(p) as ctx:
        ctx.set_particle_order(tiles)
        ctx.set_particles(pos, vel, d1, d2)
        ctx.get_displacements(A)
        ctx.kick_drift(AI, AF, A, AFF, drift=True)
        pos2, vel2, _, _ = ctx.get_particles()
    mg = O.make_mg(O.LCDM, p.Omega)
    cos = O.Cosmo(mg, p.Init_Redshift)
    g = O.cic(pos.astype(np.float64), N, Ns, box)
    O.lib().orc_fft_r2c(N, g)
    fo = O.forces_kspace(g, N, box)
    for a in range(3):
        O.lib().orc_fft_c2r(N, fo[a])
    P = pos.astype(np.float64).copy()
    V = vel.astype(np.float64).copy()
    D1 = d1.astype(np.float64)
    D2 = d2.astype(np.float64)
    disp, sD = O.interp(fo, N, box, P)
    sumv = np.zeros(3)
    O.lib().orc_kick(P.shape[0], V, disp, D1, D2, sD, p.Omega, cos.Sphi(AI, AF, A), cos.growth_ddDddy(A),
                     cos.growth_ddD2ddy(A), A, 1, sumv)
    O.lib().orc_drift(P.shape[0], P, V, D1, D2, sumv, cos.Sq(A, AFF, AF), cos.growth_D(AFF) - cos.growth_D(A),
                      cos.growth_D2(AFF) - cos.growth_D2(A), 1, box)
    assert rel_rms(vel2, V) < 1e-5
    dx = np.abs(pos2 - P)
    dx = np.minimum(dx, box - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-5 * box / Ns


def _gpu_run(p, nsteps, zf=0.0):
    """The KDK loop of src/main.c:394-611 for one output, through the C ABI."""
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        A = 1.0 / (1.0 + p.Init_Redshift)
        AI = A
        ao = 1.0 / (1.0 + zf)
        da = (ao - A) / nsteps
        for ts in range(nsteps):
            AF, AFF = A + 0.5 * da, A + da
            ctx.get_displacements(A)
            ctx.kick_drift(AI, AF, A, AFF, drift=True)
            A, AI = AFF, AF
        ctx.get_displacements(A)
        pk = ctx.pofk()
        ctx.kick_drift(AI, A, A, A, drift=False)
        pos, vel, d1, d2 = ctx.get_particles()
        dDdy, dD2dy = ctx.growth(1, A), ctx.growth(4, A)
    return pos, vel, d1, d2, pk, dDdy, dD2dy


def _oracle_run(p, mg, nsteps, zf=0.0, pw_fix=None):
    rp = O.RunParams()
    rp.mg = mg
    rp.pw = power_for(p)
    if pw_fix is not None:
        # Brans-Dicke: the spectrum is normalised with the parameter file's
        # Omega/h before the background solve replaces them (main.c:186-196)
        import ctypes as C
        h = float(np.sqrt(mg.Omegah2 / mg.omega))
        rp.pw.omega, rp.pw.h = mg.omega, h
    rp.ic = O.ICParams(p.Nmesh, p.Nsample, p.Box, p.Seed, p.SphereMode, p.amplitude_fixed_initial_condition,
                       p.inverted_initial_condition, 1.0)
    rp.init_redshift = p.Init_Redshift
    rp.nsteps = nsteps
    rp.final_redshift = zf
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = p.pofk_nbins, p.pofk_bintype, 0
    rp.pofk_kmin, rp.pofk_kmax = p.pofk_kmin, p.pofk_kmax
    rp.usecola = 1
    n = p.Nsample ** 3
    pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
    cap = max(p.pofk_nbins, p.Nmesh)
    kb, pk, km, nm = (np.zeros(cap) for _ in range(4))
    nb = O.lib().orc_run(rp, pos, vel, kb, pk, km, nm)
    return pos, vel, (kb[:nb], pk[:nb], km[:nb], nm[:nb])


@pytest.mark.parametrize("model", ["lcdm", "fofr", "dgp", "jbd", "mbeta", "w0wa", "fofr_noscreen", "dgp_noscreen"])
def test_short_run_matches_oracle(model):
    N, Ns, box, nsteps = 32, 16, 128.0, 5
    kw = dict(Seed=4242)
    pw_fix = None
    if model == "fofr":
        kw.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0,
                  input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.FOFR, 0.267, fofr0=1e-5, nfofr=1.0)
    elif model == "dgp":
        kw.update(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1, rcH0_DGP=1.0, Rsmooth=1.0,
                  smoothing_filter=M.FILTER_GAUSSIAN, input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.DGP, 0.267, rcH0=1.0, rsmooth=1.0)
    elif model == "jbd":
        kw.update(model=M.MODEL_BRANSDICKE, modified_gravity_active=1, wBD=100.0, Omegah2=0.14, Omegarh2=4e-5,
                  Omegavh2=0.36, input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.JBD_GEFF, 0.267, wBD=100.0, Omegah2=0.14, Omegarh2=4e-5, Omegavh2=0.36)
        pw_fix = (mg.omega, None)
    elif model == "mbeta":
        kw.update(model=M.MODEL_MBETA, modified_gravity_active=1, include_screening=1, assb_symm=0.5,
                  beta_symm=1.0, range_symm=1.0, input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.MBETA, 0.267, assb_symm=0.5, beta_symm=1.0, range_symm=1.0)
    elif model == "w0wa":
        kw.update(use_w0wa=1, w_0=-0.9, w_a=0.2)
        mg = O.make_mg(O.LCDM, 0.267, use_w0wa=1, w0=-0.9, wa=0.2)
    elif model == "fofr_noscreen":
        kw.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=0, fofr0=1e-5, nfofr=1.0,
                  input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.FOFR, 0.267, fofr0=1e-5, nfofr=1.0, include_screening=0)
    elif model == "dgp_noscreen":
        kw.update(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=0, rcH0_DGP=1.0, Rsmooth=1.0,
                  smoothing_filter=M.FILTER_GAUSSIAN, input_pofk_is_for_lcdm=0)
        mg = O.make_mg(O.DGP, 0.267, rcH0=1.0, rsmooth=1.0, include_screening=0)
    else:
        mg = O.make_mg(O.LCDM, 0.267)
    p = params(N, Ns, box, **kw)
    pos, vel, d1, d2, (k, pk, km, n), dDdy, dD2dy = _gpu_run(p, nsteps)
    opos, ovel, (kb, pko, kmo, no) = _oracle_run(p, mg, nsteps, pw_fix=pw_fix)
    np.testing.assert_array_equal(n, no)
    m = no > 0
    m[0] = False  # bin 0 holds only the k = 0 mode
    # P(k) of the final density: FP32 path vs FP64 oracle within 1e-3
    assert np.max(np.abs(pk[m] - pko[m]) / pko[m]) < 1e-3
    dx = np.abs(pos - opos)
    dx = np.minimum(dx, box - dx)
    # particle positions: rms below 1e-3 of the particle spacing
    assert np.sqrt(np.mean(dx ** 2)) < 1e-3 * box / Ns
    v64 = vel.astype(np.float64)
    vout = v64 - v64.mean(0) + d1 * dDdy + d2 * dD2dy
    assert rel_rms(vout, ovel) < 1e-3


def test_rsd_multipoles_match_oracle():
    N, Ns, box = 32, 16, 64.0
    p = params(N, Ns, box, pofk_nbins=12, pofk_bintype=0, pofk_kmin=0.0, pofk_kmax=0.0, pofk_subtract_shotnoise=1)
    pos, vel, d1, d2 = random_particles(Ns, box, seed=8, spread=0.5)
    # realistic COLA velocities (redshift-space shifts of a few cells); the
    # reference wraps the shifted LOS coordinate only once (compute_pofk.c:331-332)
    vel *= 0.1
    A = 0.6
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel, d1, d2)
        k, P0, P2, P4, s0, s2, s4, n = ctx.pofk_rsd(A)
        dDdy, dD2dy = ctx.growth(1, A), ctx.growth(4, A)
        Hubble = 3.2407789e-18 * (3.085678e24 / 1e5)
        cos = O.Cosmo(O.make_mg(O.LCDM, p.Omega), p.Init_Redshift)
    import ctypes as C
    H = O.lib().orc_hubble(C.byref(O.make_mg(O.LCDM, p.Omega)), A)
    vnorm = (Hubble / A) / (100.0 * A * H) * N / box
    extra = (d1.astype(np.float64) * dDdy + d2.astype(np.float64) * dD2dy)
    res = []
    for axis in (1, 2):
        out = [np.zeros(N) for _ in range(5)]
        nb = C.c_int(12)
        O.lib().orc_pofk_rsd_axis(pos.astype(np.float64), vel.astype(np.float64), extra.ctypes.data, Ns ** 3, axis, N,
                                  Ns, box, vnorm, C.byref(nb), 0, 1, 0.0, 0.0, *out)
        res.append([o[:nb.value] for o in out])
    (ky, y0, y2, y4, ny), (kz, z0, z2, z4, nz) = res
    np.testing.assert_array_equal(n, ny)
    m = ny > 0
    np.testing.assert_allclose(k[m], ky[m], rtol=1e-14)
    shot = (box / Ns) ** 3
    for got, a, b in ((P0, y0, z0), (P2, y2, z2), (P4, y4, z4)):
        ref = 0.5 * (a + b)
        scale = np.abs(0.5 * (y0 + z0) + shot)
        assert np.max(np.abs(got[m] - ref[m]) / scale[m]) < 1e-5
    np.testing.assert_allclose(s0[m], np.abs(y0 - z0)[m] / np.sqrt(2), atol=1e-5 * np.abs(y0 + shot).max())


def test_set_one_of_positions_or_velocities_keeps_the_other():
    """After steps the positions and velocities carry global offsets; setting
    only velocities (positions) must not move the particles (change the
    velocities)."""
    p = params(32, 16, 128.0, Seed=4242)
    A0 = 1.0 / 20.0
    da = (1.0 - A0) / 5
    with M.Context(p) as c:
        c.displacement_fields()
        A, AI = A0, A0
        for _ in range(2):
            c.step(A, AI, A + 0.5 * da, A + da)
            A, AI = A + da, A + 0.5 * da
        pos, vel, _, _ = c.get_particles()
        c.set_particles(vel=vel * 0.5)
        pos2, vel2, _, _ = c.get_particles()
        assert np.abs(pos2 - pos).max() < 1e-6 * 128.0
        np.testing.assert_allclose(vel2, vel * 0.5, rtol=1e-5, atol=1e-5 * np.abs(vel).max())
        c.set_particles(pos=pos)
        pos3, vel3, _, _ = c.get_particles()
        np.testing.assert_allclose(vel3, vel2, rtol=1e-6, atol=1e-6 * np.abs(vel).max())
        dx = np.abs(pos3 - pos)
        assert np.minimum(dx, 128.0 - dx).max() < 1e-5 * 128.0


def test_run_writes_reference_formats(tmp_path):
    """mgp_run: GADGET-1 snapshot, info file and pofk files (src/main.c:792-1149,
    src/compute_pofk.c:238-478) with the reference's names and layouts."""
    N, Ns, box = 32, 16, 128.0
    out = str(tmp_path)
    p = params(N, Ns, box, pofk_compute_rsd_pofk=2, pofk_nbins=8, OutputDir=out, FileBase="snap", Noutputs=2)
    p.output_redshift[0], p.output_nsteps[0] = 1.0, 3
    p.output_redshift[1], p.output_nsteps[1] = 0.0, 3
    with M.Context(p) as ctx:
        ctx.run(gadget=True)
    import os
    import struct
    names = sorted(os.listdir(out))
    assert "snap_z1p000.0" in names and "snap_z0p000.0" in names
    assert "info_snap_z0p000.txt" in names and "pofk_RSD_snap_z0.000.txt" in names
    assert any(nm.startswith("pofk_snap_z0.000_CDM") for nm in names)
    raw = open(os.path.join(out, "snap_z0p000.0"), "rb").read()
    n = Ns ** 3
    assert len(raw) == 4 + 256 + 4 + 2 * (4 + 12 * n + 4)
    assert struct.unpack("<i", raw[:4])[0] == 256 and struct.unpack("<i", raw[260:264])[0] == 256
    npart = struct.unpack("<6I", raw[4:28])
    assert npart[1] == n
    mass = struct.unpack("<6d", raw[28:76])
    t, z = struct.unpack("<2d", raw[76:92])
    assert abs(t - 1.0) < 1e-12 and abs(z) < 1e-12 and mass[1] > 0
    boxsize = struct.unpack("<d", raw[4 + 128:4 + 136])[0]
    assert boxsize == box
    blk = struct.unpack("<i", raw[264:268])[0]
    assert blk == 12 * n
    posf = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3)
    assert posf.min() >= 0 and posf.max() < box
    lines = [l for l in open(os.path.join(out, "pofk_RSD_snap_z0.000.txt")) if not l.startswith("#")]
    assert len(lines) >= 4 and len(lines[0].split()) == 7


@pytest.mark.parametrize("lpt_once", [False, True])
@pytest.mark.parametrize("N,Ns", [(32, 16), (26, 13)])
def test_step_host_matches_device_step(N, Ns, lpt_once):
    """mgp_step_host (host buffers: the positions uploaded in chunks, each
    deposited on arrival; velocities and LPT displacements copied on a side
    stream that the kick waits for) against mgp_step on device-resident
    particles from the same state; the CIC's float atomics allow 1e-5 rms.
    13^3 particles do not split evenly into the upload chunks.  lpt_once:
    D1, D2 go with the first step only (NULL afterwards keeps the device
    copy), as a driver does with the fixed LPT displacements."""
    p = params(N, Ns, 128.0, Seed=4242)
    A0 = 1.0 / 20.0
    da = (1.0 - A0) / 5
    with M.Context(p) as c1, M.Context(p) as c2:
        c1.displacement_fields()
        c2.displacement_fields()
        pos, vel, d1, d2 = c1.get_particles()
        A, AI = A0, A0
        for i in range(3):
            keep = lpt_once and i > 0
            c1.step_host(A, AI, A + 0.5 * da, A + da, pos, vel, None if keep else d1, None if keep else d2)
            c2.step(A, AI, A + 0.5 * da, A + da)
            A, AI = A + da, A + 0.5 * da
        pos2, vel2, _, _ = c2.get_particles()
    dx = np.abs(pos - pos2)
    dx = np.minimum(dx, 128.0 - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-5 * 128.0 / Ns
    assert rel_rms(vel, vel2) < 1e-5
