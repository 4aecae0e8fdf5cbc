"""CPU checks of the FP64 oracle: published known-answer vectors, analytic
solutions and the reference's own closed-form checks."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O


def test_philox_known_answers():
    # Random123 philox4x32-10 known-answer vectors (Salmon et al. 2011)
    L = O.lib()
    out = np.zeros(4, np.uint32)
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in cases:
        L.orc_philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32), out)
        assert [int(x) for x in out] == want


@pytest.mark.parametrize("N", [8, 16, 12])
def test_fft_matches_numpy(N):
    rng = np.random.default_rng(N)
    x = rng.standard_normal((N, N, N))
    g = O.fft_r2c(x)
    np.testing.assert_allclose(O.to_complex(g, N), np.fft.rfftn(x), atol=1e-10 * N ** 3)
    y = O.fft_c2r(np.fft.rfftn(x))
    np.testing.assert_allclose(y[:, :, :N] / N ** 3, x, atol=1e-12)


def test_c2r_keeps_hermitian_part_of_edge_planes():
    # Non-Hermitian content on the kz = 0 plane: only its Hermitian part
    # reaches the real output (real-output inverse DFT semantics).
    N = 8
    rng = np.random.default_rng(2)
    ck = np.zeros((N, N, N // 2 + 1), complex)
    ck[1, 2, 0] = 1.0 + 2.0j           # no partner at (-1, -2, 0)
    out = O.fft_c2r(ck)[:, :, :N]
    full = np.zeros((N, N, N), complex)
    full[1, 2, 0] = 0.5 * (1 + 2j)
    full[-1, -2, 0] = np.conj(0.5 * (1 + 2j))
    ref = np.fft.ifftn(full).real * N ** 3
    np.testing.assert_allclose(out, ref, atol=1e-12)
    (void := rng)  # noqa: F841


def test_growth_matches_lcdm_closed_form():
    # The reference's own check (cosmo.c:549-577): for LCDM the ODE growth
    # factor equals the closed form growthD (cosmo.c:1291-1356) for a > 0.2.
    mg = O.make_mg(O.LCDM, 0.267)
    c = O.Cosmo(mg, 19.0)
    for a in [0.25, 0.4, 0.6, 0.8, 1.0, 1.3]:
        assert abs(c.growth_D(a) / O.lib().orc_growthD_fit(0.267, a) - 1) < 1e-8
    # EdS limit at early times: D2 -> -3/7 D^2 normalised, ddD = 1.5 Om a D
    a = 1.0
    assert abs(c.growth_ddDddy(a) - 1.5 * 0.267 * a * c.growth_D(a)) < 1e-10


def test_sigma8_normalisation():
    p = O.make_power()
    s2 = O.lib().orc_tophat_sigma2(C.byref(p), 8.0)
    assert abs(np.sqrt(s2) - 0.8) < 1e-10


def test_cic_mass_conservation_and_lattice():
    N, Ns, box = 16, 8, 32.0
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, box, (Ns ** 3, 3))
    g = O.cic(pos, N, Ns, box)
    # sum of (1 + delta) = Np * WPAR = N^3
    assert abs((g[:, :, :N] + 1).sum() - N ** 3) < 1e-8
    # particles exactly on the lattice at N/Ns = 2: every other cell gets WPAR
    q = np.stack(np.meshgrid(*(np.arange(Ns),) * 3, indexing="ij"), -1).reshape(-1, 3) * (box / Ns)
    g = O.cic(q, N, Ns, box)
    d = g[:, :, :N] + 1
    assert np.allclose(d[::2, ::2, ::2], 8.0) and abs(d.sum() - N ** 3) < 1e-9


def test_forces_of_a_plane_wave():
    # delta(x) = A cos(k x): grad grad^-2 delta = A sin(k x)/k (analytic);
    # the kick then applies -1.5 Omega times this (main.c:712)
    N, box = 16, 50.0
    x = np.arange(N) * box / N
    kf = 2 * np.pi / box * 3
    delta = np.zeros((N, N, N))
    delta[:, :, :] = 0.1 * np.cos(kf * x)[:, None, None]
    g = O.fft_r2c(delta)
    f = O.forces_kspace(g, N, box)
    for a in range(3):
        O.lib().orc_fft_c2r(N, f[a])
    ref = 0.1 * np.sin(kf * x) / kf
    np.testing.assert_allclose(f[0][:, 0, 0], ref, atol=1e-12)
    assert np.abs(f[1][:, :, :N]).max() < 1e-12 and np.abs(f[2][:, :, :N]).max() < 1e-12


def test_pofk_bins_cover_all_modes():
    N, Ns, box = 16, 8, 64.0
    rng = np.random.default_rng(1)
    g = O.fft_r2c(rng.standard_normal((N, N, N)))
    kb, pk, km, n = O.pofk(g, N, Ns, box, 0, 0, 0, 0.0, 0.0)
    # default binning [0, N] in N bins: all N^3 modes with |k| < N - 1/2 land
    # in a bin; weights count the full (not half) k space
    total = 0
    for i in range(N):
        for j in range(N):
            for k in range(N):
                d = [min(i, N - i), min(j, N - j), min(k, N - k)]
                if int(np.sqrt(sum(v * v for v in d)) / N * N + 0.5) < N:
                    total += 1
    assert n.sum() == total


def test_ic_power_matches_input_spectrum():
    # amplitude-fixed IC: |delta(k)|^2 = P(k) mode by mode (2LPT.c:350-354)
    N, Ns, box = 32, 16, 200.0
    pw = O.make_power()
    D1, D2, dk, s2 = O.ic_2lpt(N, Ns, box, 5, pw, fixed=1, want_k=True)
    ck = O.to_complex(dk, N)
    kmag = 2 * np.pi / box * np.sqrt(3.0)
    i, j, k = 1, 1, 1
    assert abs(abs(ck[i, j, k]) ** 2 * box ** 3 - O.lib().orc_power_spec(C.byref(pw), kmag)) < 1e-9 * abs(ck[i, j, k]) ** 2 * box ** 3
    # Hermitian fill of the kz = 0 plane (2LPT.c:429-490)
    assert np.allclose(ck[3, 5, 0], np.conj(ck[N - 3, N - 5, 0]))
    # displacements have zero mean after the correction of 2LPT.c:1493-1508
    assert np.abs(D1.mean(0)).max() < 1e-12 and np.abs(D2.mean(0)).max() < 1e-12
