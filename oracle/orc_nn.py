"""FP64 numpy restatement of the learned force closure's network (test
infrastructure only): four periodic 3x3x3 convolutions, ReLU after the first
three, MSE loss on the 3 residual components (on the mesh, or at particles
through the CIC interpolation), and the exact backward pass.

The GPU kernels keep activations, weights and gradients in BF16 between
layers and accumulate in FP32; `bf16=True` rounds at the same points so that
the comparison isolates the accumulation order.
"""
import numpy as np

TAPS = [(di, dj, dk) for di in (-1, 0, 1) for dj in (-1, 0, 1) for dk in (-1, 0, 1)]


def to_bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u.astype(np.uint32)).view(np.float32).astype(np.float64)


def shift(X, d):
    """Xs[v] = X[v + d], periodic (X is [N, N, N, C])."""
    return np.roll(X, shift=(-d[0], -d[1], -d[2]), axis=(0, 1, 2))


def conv(X, W, b=None):
    """Y[v, o] = sum_t sum_c X[v + d_t, c] W[t, o, c] (+ b[o])."""
    Y = np.zeros(X.shape[:3] + (W.shape[1],))
    for t, d in enumerate(TAPS):
        Y += shift(X, d) @ W[t].T
    return Y if b is None else Y + b


def forward(X, Ws, bs, bf16=True):
    r = to_bf16 if bf16 else (lambda a: a)
    acts = [r(X)]
    for l in range(3):
        acts.append(r(np.maximum(conv(acts[-1], r(Ws[l]), bs[l]), 0.0)))
    out = conv(acts[-1], r(Ws[3]), bs[3])
    return acts, out


def backward(acts, g, Ws, bf16=True):
    """Gradients of all weights and biases from d loss / d out (g, [N,N,N,16])."""
    r = to_bf16 if bf16 else (lambda a: a)
    gw, gb = [None] * 4, [None] * 4
    for l in range(3, -1, -1):
        Xl = acts[l]
        gw[l] = np.stack([g.reshape(-1, g.shape[-1]).T @ shift(Xl, d).reshape(-1, Xl.shape[-1]) for d in TAPS])
        gb[l] = g.reshape(-1, g.shape[-1]).sum(0)
        if l == 0:
            break
        W = r(Ws[l])
        dx = np.zeros(Xl.shape)
        for t, d in enumerate(TAPS):
            dx += shift(g @ W[t], (-d[0], -d[1], -d[2]))
        dx = r(dx)
        g = dx * (Xl > 0)
    return gw, gb


def loss_and_grads(X, Ws, bs, T, scale, bf16=True):
    """Loss = sum over voxels and 3 components of (scale out - T)^2 / (3 V);
    gradients of all weights [4][27][16][16] and biases [4][16]."""
    r = to_bf16 if bf16 else (lambda a: a)
    acts, out = forward(X, Ws, bs, bf16)
    V = X.shape[0] * X.shape[1] * X.shape[2]
    e = scale * out[..., :3] - T
    loss = float(np.sum(e * e) / (3.0 * V))
    g = np.zeros(out.shape)
    g[..., :3] = 2.0 * e * scale / (3.0 * V)
    gw, gb = backward(acts, r(g), Ws, bf16)
    return loss, out, gw, gb


def cic_corners(cells, N):
    """The 8 (voxel index triple, weight) pairs of the trilinear interpolation
    at cell coordinates `cells` [np][3] (mesh units) on a periodic N^3 mesh,
    the weights of the PM gather (src/auxPM.c:560-644)."""
    fl = np.floor(cells)
    d = cells - fl
    i0 = fl.astype(np.int64) % N
    i1 = (i0 + 1) % N
    out = []
    for bx in (0, 1):
        for by in (0, 1):
            for bz in (0, 1):
                idx = tuple(np.where(b, i1[:, a], i0[:, a]) for a, b in enumerate((bx, by, bz)))
                w = np.ones(len(cells))
                for a, b in enumerate((bx, by, bz)):
                    w = w * (d[:, a] if b else 1.0 - d[:, a])
                out.append((idx, w))
    return out


def highpass(F, lam):
    """Sharp high-pass of periodic [N, N, N, C] fields: the modes of integer
    wave vector n with wavelength N / |n| >= lam cells, and the mean, are
    removed (lam <= 0: only the mean)."""
    N = F.shape[0]
    d = np.fft.fftfreq(N, 1.0 / N)
    dz = np.arange(N // 2 + 1)
    n2 = d[:, None, None] ** 2 + d[None, :, None] ** 2 + dz[None, None, :] ** 2
    kc2 = (N / lam) ** 2 if lam > 0 else 0.0
    H = ((n2 > 0) & (n2 > kc2)).astype(np.float64)
    out = np.empty_like(F)
    for c in range(F.shape[-1]):
        out[..., c] = np.fft.irfftn(np.fft.rfftn(F[..., c]) * H, s=(N,) * 3, axes=(0, 1, 2))
    return out


def loss_and_grads_particles(X, Ws, bs, cells, Tp, scale, bf16=True, hp=None):
    """Particle loss = sum over particles and components of
    (scale u_p - Tp)^2 / (3 np), u_p the trilinear interpolation at the
    particle of the network output high-passed with cutoff wavelength hp
    cells (None: no filter);
    d loss / d out is the high-passed CIC deposit of the residuals (the
    filter is its own adjoint)."""
    r = to_bf16 if bf16 else (lambda a: a)
    acts, out = forward(X, Ws, bs, bf16)
    N, n = X.shape[0], len(cells)
    corners = cic_corners(np.asarray(cells, np.float64), N)
    uo = out[..., :3] if hp is None else highpass(out[..., :3], hp)
    u = np.zeros((n, 3))
    for idx, w in corners:
        u += w[:, None] * uo[idx]
    e = scale * u - Tp
    loss = float(np.sum(e * e) / (3.0 * n))
    g3 = np.zeros(out.shape[:3] + (3,))
    for idx, w in corners:
        np.add.at(g3, idx, (2.0 * scale / (3.0 * n)) * w[:, None] * e)
    g = np.zeros(out.shape)
    g[..., :3] = g3 if hp is None else highpass(g3, hp)
    gw, gb = backward(acts, r(g), Ws, bf16)
    return loss, out, gw, gb
