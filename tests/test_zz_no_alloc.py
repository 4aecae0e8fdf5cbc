"""The allocation-free P(k) entry point (mgp_pofk_noalloc) against mgp_pofk
and the FP64 oracle.

Callers that cannot allocate device memory -- code running inside another
framework's memory pool, or that must not let cudaMalloc/cudaFree
synchronise the device -- pass their own delta(k) grid and get P(k) back
with all scratch held in the library's fixed-size device array.  Here the
caller-owned grid is a torch CUDA tensor.  Each case calls the entry point
twice in a row: the second call finds the first call's contents in the
shared array and must give the same results, bit for bit.
"""
import numpy as np
import pytest

import mgpicola as M

pytestmark = pytest.mark.gpu


def _noalloc_twice(d_dk, N, Ns, box, nbins, bintype, sub, kmin, kmax):
    first = M.pofk_noalloc(d_dk.data_ptr(), N, Ns, box, nbins, bintype, sub, kmin, kmax)
    second = M.pofk_noalloc(d_dk.data_ptr(), N, Ns, box, nbins, bintype, sub, kmin, kmax)
    for a, b in zip(first, second):
        np.testing.assert_array_equal(a, b)  # reproducible, whatever the array held before
    return first


# (Nmesh, bin type, kmin in units of 2 pi/Box, bins): linear and logarithmic
# bins; kmin = 0 with log bins takes the reference's adjustment kmin -> 1
@pytest.mark.parametrize("N,bintype,kmin_f,nbins", [(64, 0, 1.0, 40), (64, 1, 1.0, 24), (64, 1, 0.0, 24),
                                                    (256, 0, 1.0, 256), (256, 1, 0.5, 100)])
def test_pofk_noalloc_matches_pofk_twice(N, bintype, kmin_f, nbins):
    torch = pytest.importorskip("torch")
    Ns, box = N // 2, 200.0
    kmin, kmax = kmin_f * 2 * np.pi / box, np.pi * N / box
    p = M.default_params(Nmesh=N, Nsample=Ns, Box=box, Seed=91, pofk_nbins=nbins, pofk_bintype=bintype,
                         pofk_kmin=kmin, pofk_kmax=kmax, pofk_compute_every_step=1, pofk_subtract_shotnoise=1)
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.get_displacements(1.0 / 20.0)
        ref = ctx.pofk()
        dk_host = ctx.grid(1)
    d_dk = torch.from_numpy(np.ascontiguousarray(dk_host)).cuda()
    torch.cuda.synchronize()
    k, pk, km, n = _noalloc_twice(d_dk, N, Ns, box, nbins, bintype, 1, kmin, kmax)
    assert len(k) == len(ref[0])
    np.testing.assert_array_equal(n, ref[3])            # integer mode counts: exact
    np.testing.assert_allclose(k, ref[0], rtol=1e-14)
    np.testing.assert_allclose(km, ref[2], rtol=1e-12)
    m = ref[3] > 0
    np.testing.assert_allclose(pk[m], ref[1][m], rtol=1e-9, atol=1e-9 * np.abs(ref[1][m]).max())


@pytest.mark.parametrize("bintype", [0, 1])
def test_pofk_noalloc_at_its_limits_against_the_oracle(bintype):
    """The largest mesh (1024, whose |k|^2 tables end at the array's end) and
    the largest bin count (2048), on a random delta(k), against the FP64
    oracle's binning (compute_pofk.c:71-271)."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O

    N, Ns, box, nbins = 1024, 512, 1024.0, 2048
    kmin, kmax = 2 * np.pi / box, np.pi * N / box
    g = torch.Generator(device="cuda").manual_seed(7 + bintype)
    d_dk = torch.randn((N, N, N // 2 + 1, 2), device="cuda", dtype=torch.float32, generator=g)
    torch.cuda.synchronize()
    k, pk, km, n = _noalloc_twice(d_dk, N, Ns, box, nbins, bintype, 0, kmin, kmax)
    host = d_dk.cpu().numpy().astype(np.float64).reshape(N, N, 2 * (N // 2 + 1))
    del d_dk
    ko, pko, kmo, no = O.pofk(host, N, Ns, box, nbins, bintype, 0, kmin, kmax)
    assert len(k) == len(ko) == nbins
    np.testing.assert_array_equal(n, no)
    np.testing.assert_allclose(k, ko, rtol=1e-13)
    m = no > 0
    assert m.sum() > nbins // 4
    np.testing.assert_allclose(km[m], kmo[m], rtol=1e-12)
    np.testing.assert_allclose(pk[m], pko[m], rtol=1e-5, atol=1e-7 * np.abs(pko[m]).max())


def test_pofk_noalloc_rejects_sizes_beyond_the_array():
    with pytest.raises(M.MGPError, match="Nmesh"):
        M.pofk_noalloc(1, 2048, 64, 100.0, 16, 0, 1, 0.0, 0.0)
    with pytest.raises(M.MGPError, match="Nmesh"):
        M.pofk_noalloc(1, 1026, 64, 100.0, 16, 0, 1, 0.0, 0.0)
    with pytest.raises(M.MGPError, match="bins"):
        M.pofk_noalloc(1, 64, 32, 100.0, 4096, 0, 1, 0.0, 0.0)
    with pytest.raises(M.MGPError, match="bins"):
        M.pofk_noalloc(1, 64, 32, 100.0, 2049, 0, 1, 0.0, 0.0)
