"""The y pass of 1024^3 transforms (mgp_fft.cu) against cuFFT's 3D plans.

A single box with Nmesh = 1024 transforms its y lines with this library's
kernel and its z rows and x lines with cuFFT's 1D plans, the force pass
fused into the inverse y pass (mgp_set_fft_mode 1, the default); mode 0 is
cuFFT's 3D plans with the separate force pass.  The same particles give the
density spectrum, P(k) and the three force grids both ways; FP32 transforms
of 1024 points agree to a few 1e-7 relative rms, so the bound is 1e-5 of
each grid's rms (P(k): 1e-5 relative per bin).  Three models cover the three
force paths: LCDM (delta(k) straight into the fused force pass), nDGP with
screening (the screened density-plus-source spectrum, two extra transforms)
and f(R) with screening (the separate force pass, then three inverse
transforms).  Real-space grids are compared over their first 48 x planes:
every Fourier mode reaches every plane.
"""
import numpy as np
import pytest

import mgpicola as M

pytestmark = pytest.mark.gpu

PLANES = 48


def _params(model):
    kw = dict(Nmesh=1024, Nsample=64, Box=1024.0, Seed=5003, Init_Redshift=19.0, pofk_nbins=128, pofk_bintype=0,
              pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0)
    if model == "dgp":
        kw.update(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1, rcH0_DGP=1.0, Rsmooth=1.0,
                  smoothing_filter=M.FILTER_GAUSSIAN, input_pofk_is_for_lcdm=0)
    elif model == "fofr":
        kw.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0,
                  input_pofk_is_for_lcdm=0)
    return M.default_params(**kw)


def _rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2) / np.mean(b ** 2)))


def _fields(ctx, A):
    ctx.get_displacements(A)
    k, pk, km, n = ctx.pofk()
    return {"pk": (pk, n), "dk": ctx.grid(1, PLANES), "fx": ctx.grid(2, PLANES), "fy": ctx.grid(3, PLANES),
            "fz": ctx.grid(4, PLANES)}


@pytest.mark.parametrize("model", ["lcdm", "dgp", "fofr"])
def test_strided_passes_match_cufft_3d(model):
    A = 0.5
    with M.Context(_params(model)) as ctx:
        ctx.displacement_fields()
        ctx.set_fft_mode(0)
        ref = _fields(ctx, A)
        ctx.set_fft_mode(1)
        own = _fields(ctx, A)
        again = _fields(ctx, A)
    (pk0, n0), (pk1, n1) = ref["pk"], own["pk"]
    np.testing.assert_array_equal(n0, n1)
    m = n0 > 0
    m[0] = False
    assert np.max(np.abs(pk1[m] / pk0[m] - 1.0)) < 1e-5
    # the forward transform, kx planes 0..47 of delta(k)
    assert _rel_rms(own["dk"], ref["dk"]) < 1e-5
    for f in ("fx", "fy", "fz"):
        assert np.sqrt(np.mean(ref[f].astype(np.float64) ** 2)) > 0
        assert _rel_rms(own[f], ref[f]) < 1e-5, f
        # deterministic: the transforms have no atomics
        np.testing.assert_array_equal(own[f], again[f])


def test_strided_passes_full_step_positions():
    """One KDK step of the nDGP workload's model at 1024^3 both ways: the
    particles agree to float rounding of the forces (rms 1e-4 of the kick's
    displacement change)."""
    p = _params("dgp")
    A, AI, AF, AFF = 0.5, 0.49, 0.51, 0.52
    out = {}
    for mode in (0, 1):
        with M.Context(p) as ctx:
            ctx.set_fft_mode(mode)
            ctx.displacement_fields()
            pos0, vel0, _, _ = ctx.get_particles()
            ctx.step(A, AI, AF, AFF)
            pos, vel, _, _ = ctx.get_particles()
            out[mode] = (pos0, vel0, pos, vel)
    dv = out[0][3] - out[0][1]
    assert np.sqrt(np.mean(dv.astype(np.float64) ** 2)) > 0
    assert _rel_rms(out[1][3] - out[1][1], dv) < 1e-4
    d = (out[1][2] - out[0][2] + 512.0) % 1024.0 - 512.0
    assert np.sqrt(np.mean(d.astype(np.float64) ** 2)) < 1e-4 * 1024.0 / 64
