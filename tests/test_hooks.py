"""User model hooks (mgp_model_hooks): the functions of the reference's
src/user_defined_functions.h (lines 413-904) supplied as host callbacks.

CPU: hooks that restate the built-in f(R), nDGP and m(a)/beta(a) models
give the built-in growth factors, scalars and spectra; a model the library
does not have (Einstein-de Sitter background, constant mu) gives the known
growth exponent.  GPU: runs with restated hooks, including the screening
functions applied through the per-step device table, match the built-in
runs.
"""
import math

import numpy as np
import pytest

import mgpicola as M

OM = 0.267


def lcdm_H(a):
    return math.sqrt(OM / a ** 3 + 1.0 - OM)


def lcdm_dH(a):
    return -3.0 * OM / a ** 4 / (2.0 * lcdm_H(a))


def fofr_hooks(fofr0=1e-5, n=1.0):
    """src/user_defined_functions.h:462-522, 587-660, 725-750 for
    Hu-Sawicki f(R), written out as a user would."""
    def beta(a):
        return 1.0 / math.sqrt(6.0)

    def mass2(a):
        fac, fac0 = OM / a ** 3 + 4.0 * (1.0 - OM), OM + 4.0 * (1.0 - OM)
        return fac0 * (fac / fac0) ** (n + 2.0) / ((1.0 + n) * fofr0)

    def geff(a, k):
        k2 = (k * 2997.92458) ** 2
        if k2 == 0:
            return 1.0
        return 1.0 + 2.0 * beta(a) ** 2 * k2 / (k2 + a * a * mass2(a))

    def screen(a, phi):
        if phi >= 0.0:
            return 1.0
        phicrit = 1.5 * fofr0 * ((OM + 4.0 * (1.0 - OM)) / (OM / a ** 3 + 4.0 * (1.0 - OM))) ** (n + 1.0)
        return min(1.0, abs(phicrit / phi))

    return dict(hubble=lcdm_H, dhubbleda=lcdm_dH, beta_of_a=beta, mass2_of_a=mass2,
                coupling_function=lambda a: 2.0 * beta(a) ** 2, GeffoverG=geff, screening_factor_potential=screen)


def dgp_hooks(rcH0=1.0):
    def beta_dgp(a):
        return 1.0 + 2.0 * rcH0 * (lcdm_H(a) + a * lcdm_dH(a) / 3.0)

    def screen(a, density):
        fac = 8.0 / 9.0 * OM * (rcH0 / beta_dgp(a)) ** 2 * (1.0 + density)
        if fac < 1e-5:
            return 1.0
        return 2.0 * (math.sqrt(1.0 + fac) - 1.0) / fac

    def f2lpt(a):
        b = beta_dgp(a)
        return 1.0 - (2.0 * rcH0 ** 2 * OM) / (9.0 * a ** 3 * b ** 3 * (1 + 1.0 / (3.0 * b)))

    return dict(hubble=lcdm_H, dhubbleda=lcdm_dH, coupling_function=lambda a: 1.0 / (3.0 * beta_dgp(a)),
                GeffoverG=lambda a, k: 1.0 + 1.0 / (3.0 * beta_dgp(a)), Factor_2LPT=f2lpt,
                screening_factor_density=screen)


def params(model, **kw):
    d = dict(Nmesh=32, Nsample=16, Box=128.0, Seed=4242, Init_Redshift=19.0, pofk_nbins=16, pofk_bintype=0,
             pofk_kmin=0.0, pofk_kmax=0.0, pofk_compute_every_step=1, pofk_subtract_shotnoise=0,
             input_pofk_is_for_lcdm=0, Omega=OM)
    if model == "fofr":
        d.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    elif model == "dgp":
        d.update(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1, rcH0_DGP=1.0, Rsmooth=1.0,
                 smoothing_filter=M.FILTER_GAUSSIAN)
    d.update(kw)
    return M.default_params(**d)


@pytest.mark.parametrize("model", ["fofr", "dgp"])
def test_restated_hooks_give_the_built_in_model(model):
    p = params(model)
    h = M.ModelHooks.from_functions(**(fofr_hooks() if model == "fofr" else dgp_hooks()))
    a = np.array([0.05, 0.1, 0.3, 0.6, 1.0])
    for which in list(range(7)) + [10, 11, 12, 13, 15]:
        np.testing.assert_allclose(M.cosmo_eval_hooks(p, h, which, a), M.cosmo_eval_hooks(p, None, which, a),
                                   rtol=1e-12, atol=1e-300, err_msg="which %d" % which)


def test_hook_replaces_only_its_function():
    """A user mass2_of_a alone changes the built-in f(R) GeffoverG through
    it, as GeffoverG calls mass2_of_a in the reference."""
    p = params("fofr")
    m2 = fofr_hooks()["mass2_of_a"]
    h = M.ModelHooks.from_functions(mass2_of_a=lambda a: 4.0 * m2(a))
    a = np.array([0.5])
    k2 = (0.1 * 2997.92458) ** 2
    np.testing.assert_allclose(M.cosmo_eval_hooks(p, h, 11, a), 1.0 + (1.0 / 3.0) * k2 / (k2 + 0.25 * 4.0 * m2(0.5)),
                               rtol=1e-13)
    assert M.cosmo_eval_hooks(p, h, 12, a)[0] == pytest.approx(1.0 / 3.0, rel=1e-14)  # coupling unchanged


def test_new_model_einstein_de_sitter_constant_mu():
    """A model the library does not have: Omega = 1 background and mu = 1.2
    everywhere.  Then D'' + D'/2 = 1.5 mu D in ln a, solved by a^p and a^q,
    p, q = (-1 +- sqrt(1 + 24 mu))/4; the reference's initial condition
    D = D' = 1 at z = 200 (src/cosmo.c:409-470) fixes their mix, and the
    result is normalised at a = 1."""
    mu = 1.2
    p = params("lcdm", Omega=1.0, modified_gravity_active=1)
    h = M.ModelHooks.from_functions(hubble=lambda a: a ** -1.5, dhubbleda=lambda a: -1.5 * a ** -2.5,
                                    GeffoverG=lambda a, k: mu)
    r = math.sqrt(1.0 + 24.0 * mu)
    pe, qe = (-1.0 + r) / 4.0, (-1.0 - r) / 4.0
    ai = 1.0 / 201.0
    c1, c2 = (1.0 - qe) / (pe - qe), (pe - 1.0) / (pe - qe)
    D = lambda a: c1 * (a / ai) ** pe + c2 * (a / ai) ** qe  # noqa: E731
    a = np.array([0.05, 0.2, 0.5, 1.0])
    np.testing.assert_allclose(M.cosmo_eval_hooks(p, h, 0, a), D(a) / D(1.0), rtol=1e-6)
    # without the hook the same parameters are plain EdS: D = a
    np.testing.assert_allclose(M.cosmo_eval_hooks(p, None, 0, a), a, rtol=2e-6)


def _run(p, hooks, nsteps=5):
    with M.Context(p, hooks=hooks) as ctx:
        ctx.displacement_fields()
        A = 1.0 / 20.0
        AI, da = A, (1.0 - A) / nsteps
        for _ in range(nsteps):
            ctx.step(A, AI, A + 0.5 * da, A + da)
            A, AI = A + da, A + 0.5 * da
        ctx.get_displacements(A)
        pk = ctx.pofk()
        pos = ctx.get_particles()[0]
    return pk, pos


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["fofr", "dgp"])
def test_run_with_restated_hooks_matches_built_in(model):
    """The whole run, with the screening factor applied through the device
    table of the user's function (linear interpolation over 16384 asinh
    points) instead of the built-in formula."""
    p = params(model)
    h = M.ModelHooks.from_functions(**(fofr_hooks() if model == "fofr" else dgp_hooks()))
    (k0, pk0, _, n0), pos0 = _run(p, None)
    (k1, pk1, _, n1), pos1 = _run(p, h)
    np.testing.assert_array_equal(n0, n1)
    m = n0 > 0
    m[0] = False
    assert np.max(np.abs(pk1[m] / pk0[m] - 1.0)) < 1e-4
    dx = np.abs(pos1 - pos0)
    dx = np.minimum(dx, 128.0 - dx)
    assert np.sqrt(np.mean(dx ** 2)) < 1e-4 * 128.0 / 16
