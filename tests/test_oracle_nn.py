"""The numpy restatement of the closure network (oracle/orc_nn.py): its
backward pass against central finite differences in FP64 (no BF16
rounding), on a small periodic grid."""
import numpy as np

from oracle import orc_nn as NN


def test_closure_oracle_gradients_match_finite_differences():
    N = 4
    rng = np.random.default_rng(0)
    X = np.zeros((N, N, N, 16))
    X[..., :3] = rng.normal(0, 1, (N, N, N, 3))
    Ws = rng.normal(0, 0.2, (4, 27, 16, 16))
    Ws[3, :, 3:, :] = 0
    bs = rng.normal(0, 0.1, (4, 16))
    bs[3, 3:] = 0
    T = rng.normal(0, 1, (N, N, N, 3))
    loss, _, gw, gb = NN.loss_and_grads(X, Ws, bs, T, 1.5, bf16=False)
    eps = 1e-6
    for (l, t, o, c) in [(0, 4, 2, 1), (1, 13, 7, 5), (2, 26, 15, 0), (3, 0, 2, 9), (3, 20, 1, 3)]:
        Wp, Wm = Ws.copy(), Ws.copy()
        Wp[l, t, o, c] += eps
        Wm[l, t, o, c] -= eps
        fd = (NN.loss_and_grads(X, Wp, bs, T, 1.5, bf16=False)[0] -
              NN.loss_and_grads(X, Wm, bs, T, 1.5, bf16=False)[0]) / (2 * eps)
        assert abs(fd - gw[l][t, o, c]) < 1e-6 + 1e-4 * abs(fd), (l, t, o, c, fd, gw[l][t, o, c])
    for (l, o) in [(0, 3), (2, 11), (3, 1)]:
        bp, bm = bs.copy(), bs.copy()
        bp[l, o] += eps
        bm[l, o] -= eps
        fd = (NN.loss_and_grads(X, Ws, bp, T, 1.5, bf16=False)[0] -
              NN.loss_and_grads(X, Ws, bm, T, 1.5, bf16=False)[0]) / (2 * eps)
        assert abs(fd - gb[l][o]) < 1e-6 + 1e-4 * abs(fd)


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265], np.float64)
    r = NN.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12


def test_particle_loss_gradients_match_finite_differences():
    N, n = 4, 40
    rng = np.random.default_rng(2)
    X = np.zeros((N, N, N, 16))
    X[..., :3] = rng.normal(0, 1, (N, N, N, 3))
    Ws = rng.normal(0, 0.2, (4, 27, 16, 16))
    Ws[3, :, 3:, :] = 0
    bs = rng.normal(0, 0.1, (4, 16))
    bs[3, 3:] = 0
    cells = rng.uniform(0, N, (n, 3))
    Tp = rng.normal(0, 1, (n, 3))
    for hp in (None, 1.5):
        loss, _, gw, gb = NN.loss_and_grads_particles(X, Ws, bs, cells, Tp, 0.7, bf16=False, hp=hp)
        eps = 1e-6
        for (l, t, o, c) in [(0, 7, 1, 2), (1, 13, 4, 9), (3, 22, 0, 5), (3, 1, 2, 14)]:
            Wp, Wm = Ws.copy(), Ws.copy()
            Wp[l, t, o, c] += eps
            Wm[l, t, o, c] -= eps
            fd = (NN.loss_and_grads_particles(X, Wp, bs, cells, Tp, 0.7, bf16=False, hp=hp)[0] -
                  NN.loss_and_grads_particles(X, Wm, bs, cells, Tp, 0.7, bf16=False, hp=hp)[0]) / (2 * eps)
            assert abs(fd - gw[l][t, o, c]) < 1e-6 + 1e-4 * abs(fd), (hp, l, t, o, c, fd, gw[l][t, o, c])
        for (l, o) in [(1, 6), (3, 2)]:
            bp, bm = bs.copy(), bs.copy()
            bp[l, o] += eps
            bm[l, o] -= eps
            fd = (NN.loss_and_grads_particles(X, Ws, bp, cells, Tp, 0.7, bf16=False, hp=hp)[0] -
                  NN.loss_and_grads_particles(X, Ws, bm, cells, Tp, 0.7, bf16=False, hp=hp)[0]) / (2 * eps)
            assert abs(fd - gb[l][o]) < 1e-6 + 1e-4 * abs(fd)


def test_highpass_removes_long_waves_and_keeps_short_ones():
    N = 16
    x = np.arange(N)
    F = np.zeros((N, N, N, 3))
    F[..., 0] = 3.0  # the mean: removed
    F[..., 1] = np.cos(2 * np.pi * 2 * x / N)[:, None, None] * np.ones((N, N, N))  # wavelength 8 cells: removed
    F[..., 2] = np.cos(2 * np.pi * 3 * x / N)[None, :, None] * np.ones((N, N, N))  # 5.3 cells: kept
    out = NN.highpass(F, 8.0)
    assert np.max(np.abs(out[..., :2])) < 1e-12
    assert np.allclose(out[..., 2], F[..., 2])


def test_particle_interpolation_weights_are_a_partition_of_unity():
    rng = np.random.default_rng(3)
    cells = np.vstack([rng.uniform(0, 8, (100, 3)), [[7.999999, 0.0, 3.5]]])
    corners = NN.cic_corners(cells, 8)
    assert np.allclose(sum(w for _, w in corners), 1.0)
    for idx, w in corners:
        for a in idx:
            assert a.min() >= 0 and a.max() < 8
    # a linear field (away from the periodic seam) is reproduced exactly
    g = np.arange(8.0)[:, None, None] + 0 * np.zeros((8, 8, 8))
    inner = cells[:100][cells[:100, 0] < 7]
    u = sum(w * g[idx] for idx, w in NN.cic_corners(inner, 8))
    assert np.allclose(u, inner[:, 0])
