"""Learned force closure: the CUDA forward and backward passes against the
FP64 numpy restatement of the network (oracle/orc_nn.py), the training
inputs and targets against numpy from the context's own grids, the
in-step application, and a small end-to-end training run that must reduce
the force error against a 3x finer mesh on a held-out seed.

Tolerances: the GPU keeps activations and gradients in BF16 between layers
(the oracle rounds at the same points), so outputs agree to 1e-2 and
gradients to 3e-2 relative rms; the loss to 1e-3.
"""
import numpy as np
import pytest

import mgpicola as M
from oracle import orc_nn as NN

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2) / max(np.mean(b ** 2), 1e-300)))


def rand_net(seed, sd=0.15):
    rng = np.random.default_rng(seed)
    w = rng.normal(0, sd, (4, 27, 16, 16)).astype(np.float32)
    b = rng.normal(0, 0.05, (4, 16)).astype(np.float32)
    w[3, :, 3:, :] = 0.0  # the last layer has three outputs
    b[3, 3:] = 0.0
    return w, b


def features(N, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (N, N, N, 3))
    return x.reshape(-1, 3).astype(np.float32)


def padded(x, N):
    X = np.zeros((N, N, N, 16))
    X[..., :3] = x.reshape(N, N, N, 3)
    return X


def test_closure_forward_matches_oracle():
    N = 16
    w, b = rand_net(1)
    x = features(N, 2)
    with M.Closure(N) as cl:
        cl.set_weights(w, b, 1.0)
        cl.set_sample(x, None)
        out = cl.forward()
    _, ref = NN.forward(padded(x, N), w.astype(np.float64), b.astype(np.float64))
    assert rel_rms(out, ref[..., :3].reshape(-1, 3)) < 1e-2


def test_closure_gradients_match_oracle():
    N = 16
    w, b = rand_net(3)
    x = features(N, 4)
    t = np.random.default_rng(5).normal(0, 1, (N ** 3, 3)).astype(np.float32)
    with M.Closure(N) as cl:
        cl.set_weights(w, b, 2.0)
        cl.set_sample(x, t)
        loss, gw, gb = cl.gradients()
    lr, _, gwr, gbr = NN.loss_and_grads(padded(x, N), w.astype(np.float64), b.astype(np.float64),
                                        t.reshape(N, N, N, 3).astype(np.float64), 2.0)
    assert abs(loss - lr) / lr < 1e-3
    for l in range(4):
        assert rel_rms(gw[l], gwr[l]) < 3e-2, l
        assert rel_rms(gb[l], gbr[l]) < 3e-2, l


def test_closure_training_reduces_loss():
    """A student net fitted to a teacher net's outputs on fixed inputs."""
    N = 16
    x = features(N, 6)
    wt, bt = rand_net(7)
    _, tgt = NN.forward(padded(x, N), wt.astype(np.float64), bt.astype(np.float64))
    with M.Closure(N, seed=11) as cl:
        cl.set_sample(x, tgt[..., :3].reshape(-1, 3).astype(np.float32))
        first = cl.train_step(2e-3)
        for _ in range(150):
            last = cl.train_step(2e-3)
    assert last < 0.5 * first


def _lcdm_ctx(N, Ns=16, box=128.0):
    p = M.default_params(Nmesh=N, Nsample=Ns, Box=box, Seed=4242, Init_Redshift=19.0, pofk_nbins=16,
                         pofk_compute_every_step=1, pofk_subtract_shotnoise=0)
    return M.Context(p)


def test_closure_features_and_target_match_numpy():
    Nc, r, A = 32, 3, 0.5
    with _lcdm_ctx(Nc) as c, _lcdm_ctx(Nc * r) as f, M.Closure(Nc) as cl:
        c.displacement_fields()
        pos, vel, _, _ = c.get_particles()
        f.set_particles(pos, vel)
        c.get_displacements(A)
        f.get_displacements(A)
        cl.features(c, A)
        rms = cl.target(f, c)
        x, t = cl.sample()
        dk = c.grid(1).view(np.complex64).reshape(Nc, Nc, Nc // 2 + 1).astype(np.complex128)
        fc = [c.grid(2 + a).reshape(Nc, Nc, -1)[:, :, :Nc] for a in range(3)]
        ff = [f.grid(2 + a).reshape(Nc * r, Nc * r, -1)[:, :, :Nc * r] for a in range(3)]
        om = c.params.Omega
    # delta(x) and Phi_N(x) exactly as the library's transforms define them
    delta = np.fft.irfftn(dk, s=(Nc,) * 3)
    d = np.fft.fftfreq(Nc, 1.0 / Nc)
    dz = np.arange(Nc // 2 + 1)
    rk = d[:, None, None] ** 2 + d[None, :, None] ** 2 + dz[None, None, :] ** 2
    norm = 1.0 / Nc ** 3 * 1.5 * om / A * (128.0 / 2997.92458 / (2 * np.pi)) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        phik = np.where(rk > 0, -norm * dk / rk, 0.0)
    phi = np.fft.irfftn(phik, s=(Nc,) * 3) * Nc ** 3
    ref = np.stack([np.arcsinh(delta), phi * 1e5, np.ones_like(delta)], -1).reshape(-1, 3)
    assert rel_rms(x, NN.to_bf16(ref)) < 1e-2
    # target: the fine force averaged over the 27 fine points around r i
    acc = [0.0, 0.0, 0.0]
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            for cc in (-1, 0, 1):
                for q in range(3):
                    acc[q] = acc[q] + np.roll(ff[q], (-a, -b, -cc), axis=(0, 1, 2))[::r, ::r, ::r]
    tref = np.stack([acc[q] / 27.0 - fc[q] for q in range(3)], -1).reshape(-1, 3)
    assert rel_rms(t, tref) < 1e-5
    assert abs(rms - np.sqrt(np.mean(tref ** 2))) < 1e-4 * rms


def test_closure_applied_in_step_adds_highpassed_forward_output():
    """The in-step closure force is out_scale times the high-passed network
    output, added through the force transforms (cutoff 12 cells here)."""
    N, A = 32, 0.5
    w, b = rand_net(13, sd=0.05)
    with _lcdm_ctx(N) as c, M.Closure(N) as cl:
        cl.set_weights(w, b, 0.3)
        cl.set_highpass(12.0)
        sigma = cl.highpass()
        c.displacement_fields()
        c.get_displacements(A)
        plain = [c.grid(2 + a).reshape(N, N, -1)[:, :, :N].copy() for a in range(3)]
        cl.features(c, A)
        out = cl.forward().reshape(N, N, N, 3)
        cl.attach(c)
        c.get_displacements(A)
        withc = [c.grid(2 + a).reshape(N, N, -1)[:, :, :N].copy() for a in range(3)]
        M.Closure.detach(c)
    # the second deposit differs from the first at the 1e-6 level (order of the
    # CIC's float atomics), which moves a few BF16 feature roundings by one ulp
    hp = NN.highpass(out.astype(np.float64), sigma)
    assert sigma == 12.0
    for a in range(3):
        assert rel_rms(withc[a] - plain[a], 0.3 * hp[..., a]) < 2e-3


def test_closure_particle_loss_gradients_match_oracle():
    N, n = 16, 5000
    w, b = rand_net(21)
    x = features(N, 22)
    rng = np.random.default_rng(23)
    cells = rng.uniform(0, N, (n, 3)).astype(np.float32)
    tp = rng.normal(0, 1, (n, 3)).astype(np.float32)
    with M.Closure(N) as cl:
        cl.set_weights(w, b, 1.5)
        cl.set_highpass(5.0)
        cl.set_sample(x, None)
        cl.set_particle_sample(cells, tp)
        c2, t2 = cl.particle_sample()
        loss, gw, gb = cl.gradients()
    assert np.array_equal(c2, cells) and np.array_equal(t2, tp)
    lr, _, gwr, gbr = NN.loss_and_grads_particles(padded(x, N), w.astype(np.float64), b.astype(np.float64),
                                                  cells.astype(np.float64), tp.astype(np.float64), 1.5,
                                                  hp=5.0)
    assert abs(loss - lr) / lr < 1e-3
    for l in range(4):
        assert rel_rms(gw[l], gwr[l]) < 3e-2, l
        assert rel_rms(gb[l], gbr[l]) < 3e-2, l


def _interp(F, cells):
    """CIC interpolation of a periodic [N][N][N] grid at cell coordinates."""
    return sum(w * F[idx] for idx, w in NN.cic_corners(cells.astype(np.float64), F.shape[0]))


def test_closure_particle_target_matches_numpy():
    Nc, r, A = 32, 3, 0.5
    with _lcdm_ctx(Nc) as c, _lcdm_ctx(Nc * r) as f, M.Closure(Nc) as cl:
        c.displacement_fields()
        for _ in range(2):  # move the particles off the lattice
            c.get_displacements(0.1)
            c.kick_drift(0.1, 0.3, 0.1, 0.3)
        pos, vel, _, _ = c.get_particles()
        f.set_particles(pos, vel)
        c.get_displacements(A)
        f.get_displacements(A)
        rms = cl.target_particles(f, c, band=False)
        cells, t = cl.particle_sample()
        rms_b = cl.target_particles(f, c, band=True)
        _, t_b = cl.particle_sample()
        fc = [c.grid(2 + a).reshape(Nc, Nc, -1)[:, :, :Nc].astype(np.float64) for a in range(3)]
        ff = [f.grid(2 + a).reshape(Nc * r, Nc * r, -1)[:, :, :Nc * r].astype(np.float64) for a in range(3)]
        pos_c = c.get_particles()[0].astype(np.float64)
    box = 128.0
    want = np.mod(pos_c * Nc / box, Nc)
    dc = np.abs(cells - want)
    assert np.max(np.minimum(dc, Nc - dc)) < 1e-3
    cf = np.mod(pos.astype(np.float64) * Nc * r / box, Nc * r)
    tref = np.stack([_interp(ff[a], cf) - _interp(fc[a], cells) for a in range(3)], -1)
    assert rel_rms(t, tref) < 1e-4
    assert abs(rms - np.sqrt(np.mean(tref ** 2))) < 1e-3 * rms
    # band-limited: the fine force keeps only |k_i| < Nc/2 (fine integer units)
    Nf = Nc * r
    d = np.abs(np.fft.fftfreq(Nf, 1.0 / Nf))
    keep = (d[:, None, None] < Nc // 2) & (d[None, :, None] < Nc // 2) & (np.arange(Nf // 2 + 1)[None, None, :] < Nc // 2)
    fb = [np.fft.irfftn(np.fft.rfftn(ff[a]) * keep, s=(Nf,) * 3) for a in range(3)]
    tref_b = np.stack([_interp(fb[a], cf) - _interp(fc[a], cells) for a in range(3)], -1)
    assert rel_rms(t_b, tref_b) < 1e-4
    assert abs(rms_b - np.sqrt(np.mean(tref_b ** 2))) < 1e-3 * rms_b
    assert rms_b < rms


def test_closure_particle_samples_store_load_and_train():
    """Particle samples kept on the device: a stored slot loads back as the
    working sample, and training on a teacher's interpolated output lowers
    the particle loss."""
    N, n = 16, 4096
    x = features(N, 31)
    wt, bt = rand_net(32)
    _, out_t = NN.forward(padded(x, N), wt.astype(np.float64), bt.astype(np.float64))
    out_t = out_t - out_t.mean(axis=(0, 1, 2))  # the closure output carries no mean
    rng = np.random.default_rng(33)
    cells = rng.uniform(0, N, (n, 3))
    tp = sum(w[:, None] * out_t[idx][:, :3] for idx, w in NN.cic_corners(cells, N)).astype(np.float32)
    with M.Closure(N, seed=34) as cl:
        cl.set_highpass(0.0)  # only the mean is removed
        cl.reserve(2, n)
        cl.set_sample(x, None)
        cl.set_particle_sample(cells.astype(np.float32), tp)
        cl.store(1)
        cl.set_particle_sample(cells.astype(np.float32), np.zeros_like(tp))
        cl.load(1)
        c2, t2 = cl.particle_sample()
        assert np.array_equal(t2, tp)
        first = cl.train_step(2e-3)
        for _ in range(150):
            cl.load(1)
            last = cl.train_step(2e-3)
    assert last < 0.5 * first


def test_trained_closure_reduces_held_out_force_error():
    """End to end at 128^3 particles, Box 128 Mpc/h (1 Mpc/h per coarse cell,
    the learned-closure workload's resolution): particle samples from the
    128^3 and 384^3 meshes of four seeds, GPU training, then the force error
    on a held-out seed.  The untrained closure outputs zero (the plain PM
    force), so its error relative to the target's mean square is 1; the
    trained one must explain at least 30% of the band-limited fine-minus-
    coarse force on the held-out seed (measured: about 70%)."""
    import closure_train as T

    Nc, box, r, nsteps = 128, 128.0, 3, 30
    snaps = set(range(0, nsteps, 3)) | {nsteps - 1}
    with M.Closure(Nc, seed=5) as cl:
        cl.reserve(5 * len(snaps), Nc ** 3)
        cl.set_scale_table([0.1, 1.0], [1.0, 10.0])
        assert abs(cl.scale_at(np.sqrt(0.1)) - np.sqrt(10.0)) < 1e-9  # log-log interpolation
        assert cl.scale_at(0.05) == 1.0 and cl.scale_at(2.0) == 10.0  # held at the ends
        slot = 0
        for sd in range(7001, 7005):
            slot, _, _ = T.collect(cl, sd, "lcdm", Nc, r, Nc, box, nsteps, snaps, slot)
        ntrain = slot
        slot, _, _ = T.collect(cl, 7017, "lcdm", Nc, r, Nc, box, nsteps, snaps, slot)

        def held_out():  # each sample's loss is relative to its own mean square target
            out = []
            for s in range(ntrain, slot):
                cl.load(s)
                out.append(cl.gradients()[0])
            return np.array(out)

        before = held_out()
        hist = T.train(cl, ntrain, 16, 2e-3)
        after = held_out()
    assert np.allclose(before, 1.0, atol=1e-3)
    assert hist[-1] < hist[0]
    assert np.mean(after) < 0.7, after
    assert np.all(after < 1.0), after
