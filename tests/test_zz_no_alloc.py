"""The allocation-free P(k) entry point (mgp_pofk_noalloc) against mgp_pofk.

Callers that cannot allocate device memory -- code running inside another
framework's memory pool, or that must not let cudaMalloc/cudaFree
synchronise the device -- pass their own delta(k) grid and get P(k) back
with all scratch held in the library's fixed-size device array.  Here the
caller-owned grid is a torch CUDA tensor holding the context's delta(k).
"""
import numpy as np
import pytest

import mgpicola as M

pytestmark = pytest.mark.gpu


def test_pofk_noalloc_matches_pofk_twice():
    torch = pytest.importorskip("torch")
    N, Ns, box, nbins = 64, 32, 200.0, 40
    p = M.default_params(Nmesh=N, Nsample=Ns, Box=box, Seed=91, pofk_nbins=nbins, pofk_bintype=0,
                         pofk_kmin=2 * np.pi / box, pofk_kmax=np.pi * N / box, pofk_compute_every_step=1,
                         pofk_subtract_shotnoise=1)
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        ctx.get_displacements(1.0 / 20.0)
        ref = ctx.pofk()
        dk_host = ctx.grid(1)
    d_dk = torch.from_numpy(np.ascontiguousarray(dk_host)).cuda()
    torch.cuda.synchronize()
    for _ in range(2):  # the second call reuses the array the first one left behind
        k, pk, km, n = M.pofk_noalloc(d_dk.data_ptr(), N, Ns, box, nbins, 0, 1, 2 * np.pi / box, np.pi * N / box)
        assert len(k) == len(ref[0])
        np.testing.assert_array_equal(n, ref[3])            # integer mode counts: exact
        np.testing.assert_allclose(k, ref[0], rtol=1e-14)
        np.testing.assert_allclose(km, ref[2], rtol=1e-12)
        m = ref[3] > 0
        np.testing.assert_allclose(pk[m], ref[1][m], rtol=1e-9, atol=1e-9 * np.abs(ref[1][m]).max())


def test_pofk_noalloc_rejects_sizes_beyond_the_array():
    with pytest.raises(M.MGPError, match="Nmesh"):
        M.pofk_noalloc(1, 2048, 64, 100.0, 16, 0, 1, 0.0, 0.0)
    with pytest.raises(M.MGPError, match="bins"):
        M.pofk_noalloc(1, 64, 32, 100.0, 4096, 0, 1, 0.0, 0.0)
