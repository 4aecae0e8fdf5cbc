"""Massive neutrinos (the reference's MASSIVE_NEUTRINOS build, always scale
dependent): the host side against the FP64 oracle on synthetic CAMB tables
(tests/golden/camb_tables.py).

  - transfer tables: the reader and 2D bicubic tables reproduce the file
    values at the nodes (src/read_CAMB_data.h:41-170, 238-278);
  - OmegaNu / OmegaCDM and the cut below 1e-6
    (src/user_defined_functions.h:50-75);
  - growth factors with the neutrino factors mu_nu (src/cosmo.c:206-266,
    798-981), both the 1D tables at k = 1e-3 and D(k, a);
  - the CDM+baryon P(k) with the normalisation taken before OmegaCDM is set
    (src/power.c:226-257, 376-380; src/main.c:153-162);
  - mg_pofk_ratio and the sigma8 enhancement against the LCDM D(k, a) of the
    neutrino build (src/cosmo.c:688-756);
  - the parameter keys of that build and the reader's errors.
"""
import ctypes as C
import os

import numpy as np
import pytest

import mgpicola as M
from golden import camb_tables
from oracle import oracle as O
from test_host import write_param


@pytest.fixture(scope="module")
def info(tmp_path_factory):
    return camb_tables.write_tables(str(tmp_path_factory.mktemp("camb")))


def nu_params(info, model="lcdm", **kw):
    d = dict(Nmesh=32, Nsample=16, Box=128.0, Init_Redshift=19.0, scaledependent=1, massive_neutrinos=1, sd_nk=200,
             nu_include_massive_neutrinos=1, nu_SumMassNuEV=camb_tables.SUM_MNU_EV,
             nu_FilenameTransferInfofile=info, input_pofk_is_for_lcdm=0, input_sigma8_is_for_lcdm=1)
    if model == "fofr":
        d.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0)
    d.update(kw)
    return M.default_params(**d)


def oracle_cosmo(info, p, model="lcdm"):
    nu = O.Neutrinos(info, p.Omega, p.OmegaBaryon, p.HubbleParam, p.PrimordialIndex, p.nu_SumMassNuEV,
                     p.nu_include_massive_neutrinos)
    if model == "fofr":
        mg = O.make_mg(O.FOFR, p.Omega, mg_active=1, include_screening=1, fofr0=p.fofr0, nfofr=p.nfofr,
                       scaledependent=1, nu=nu, sd_nk=p.sd_nk)
    else:
        mg = O.make_mg(O.LCDM, p.Omega, scaledependent=1, nu=nu, sd_nk=p.sd_nk)
    return nu, O.Cosmo(mg, p.Init_Redshift, p.Box, p.Nmesh)


def test_transfer_tables_reproduce_the_files(info):
    nu = O.Neutrinos(info)
    k = np.exp(np.linspace(np.log(1e-4), np.log(100.0), 150))
    for iz in (0, 3, 7, 10):
        z = camb_tables.REDSHIFTS[iz]
        cols = np.array([[float("%.8e" % v) for v in row] for row in camb_tables.transfer_columns(k, z)])
        for ik in (0, 17, 80, 149):
            kk = cols[ik, 0]
            for which, col in ((nu.TNU, 5), (nu.TCDM, 1), (nu.TB, 2), (nu.TTOT, 6)):
                got = nu.transfer(which, kk, 1.0 / (1.0 + z))
                assert got == pytest.approx(cols[ik, col], rel=1e-9)
    # outside the table the lookup clamps
    assert nu.transfer(nu.TCDM, 1e-6, 1.0) == pytest.approx(nu.transfer(nu.TCDM, 1e-4, 1.0), rel=1e-9)
    assert nu.transfer(nu.TCDM, 0.1, 1.0 / 1001.0) == pytest.approx(nu.transfer(nu.TCDM, 0.1, 1.0 / 301.0),
                                                                    rel=1e-12)


def test_neutrino_omegas_and_cut(info):
    nu = O.Neutrinos(info, 0.267, 0.049, 0.71, 0.96, 0.4, 1)
    assert nu.omega_nu == pytest.approx(0.4 / (93.14 * 0.71 ** 2), rel=1e-14)
    assert nu.omega_cdm == pytest.approx(0.267 - 0.049 - nu.omega_nu, rel=1e-14)
    assert nu.mu2() == pytest.approx((0.267 - nu.omega_nu) / 0.267, rel=1e-14)
    # large k: the neutrinos free-stream, mu_1 -> (Omega - OmegaNu) / Omega
    assert nu.mu1(1.0, 10.0) == pytest.approx(nu.mu2(), rel=1e-4)
    assert nu.mu1(1.0, 1e-4) > nu.mu1(1.0, 0.1) > nu.mu2()
    tiny = O.Neutrinos(info, 0.267, 0.049, 0.71, 0.96, 1e-8, 1)
    assert tiny.omega_nu == 0.0 and tiny.mu1(1.0, 0.1) == 1.0 and tiny.mu2() == 1.0


@pytest.mark.parametrize("model", ["lcdm", "fofr"])
def test_host_growth_with_neutrinos_matches_oracle(info, model):
    p = nu_params(info, model)
    _, cos = oracle_cosmo(info, p, model)
    a = np.array([0.05, 0.2, 0.5, 1.0])
    # 1D tables at k = 1e-3 with mu_nu in the ODEs (cosmo.c:459-520)
    names = ["growth_D", "growth_dDdy", "growth_ddDddy", "growth_D2", "growth_dD2dy", "growth_ddD2ddy",
             "growth_DLCDM"]
    for which, name in enumerate(names):
        np.testing.assert_allclose(M.cosmo_eval(p, which, a), [getattr(cos, name)(x) for x in a], rtol=2e-6,
                                   err_msg=name)
    # D(k, a) tables (cosmo.c:886-981), normalised at a = 1 per k
    ks = np.array([0.01, 0.05, 0.2, 1.0, 2.0])
    kk, aa = (g.ravel() for g in np.meshgrid(ks, np.array([0.05, 0.3, 0.7]), indexing="ij"))
    for which in range(6):
        got = M.growth_scaledependent(p, which, kk, aa)
        ref = np.array([cos.growth_sd(which, x, y) for x, y in zip(kk, aa)])
        np.testing.assert_allclose(got, ref, rtol=2e-5, err_msg="which %d" % which)
    if model == "lcdm":
        # the neutrinos slow the growth on small scales: normalised at a = 1,
        # D(a) / D(1) at early a is larger where the growth was suppressed
        d = M.growth_scaledependent(p, 0, np.array([0.01, 1.0]), np.array([0.05, 0.05]))
        assert d[1] > d[0]


def test_host_power_spectrum_is_cdm_baryon(info):
    p = nu_params(info)
    nu = O.Neutrinos(info, p.Omega, p.OmegaBaryon, p.HubbleParam, p.PrimordialIndex, p.nu_SumMassNuEV, 1)
    pw = O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex,
                      sigma8=p.Sigma8, nu=nu)
    k = np.array([1e-3, 0.01, 0.1, 0.5, 1.0, 5.0])
    ref = [O.lib().orc_power_spec(C.byref(pw), x) for x in k]
    np.testing.assert_allclose(M.cosmo_eval(p, 7, k), ref, rtol=1e-9)
    # the normalisation used the baryon transfer function (OmegaCDM still 0)
    assert pw.nu_ocdm == pytest.approx(nu.omega_cdm)
    pb = O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex,
                      sigma8=p.Sigma8, nu=nu)
    pb.nu_ocdm = 0.0
    assert O.lib().orc_tophat_sigma2(C.byref(pb), 8.0) == pytest.approx(p.Sigma8 ** 2, rel=1e-6)


def test_host_pofk_ratio_and_sigma8_with_neutrinos(info):
    """f(R) + neutrinos: both against the LCDM D(k, a) of the neutrino build."""
    p = nu_params(info, "fofr")
    nu, cos = oracle_cosmo(info, p, "fofr")
    k = np.array([0.01, 0.1, 0.5, 1.0])
    np.testing.assert_allclose(M.cosmo_eval(p, 8, k), [cos.mg_pofk_ratio(x, 1.0) for x in k], rtol=5e-5)
    pw = O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex,
                      sigma8=p.Sigma8, nu=nu)
    a = np.array([0.5, 1.0])
    np.testing.assert_allclose(M.cosmo_eval(p, 9, a), [O.lib().orc_mg_sigma8_enh(cos.h, C.byref(pw), x) for x in a],
                               rtol=2e-5)
    assert M.cosmo_eval(p, 8, np.array([1.0]))[0] > 1.0  # f(R) enhances small scales


def test_neutrino_parameter_keys(tmp_path, info):
    keys = "nu_include_massive_neutrinos 1\nnu_SumMassNuEV 0.2\nnu_FilenameTransferInfofile %s\n" % info
    p = M.read_parameterfile(write_param(tmp_path, M.MODEL_FOFR, extra=keys), M.MODEL_FOFR, massive_neutrinos=True)
    assert p.massive_neutrinos == 1 and p.scaledependent == 1
    assert p.nu_include_massive_neutrinos == 1 and p.nu_SumMassNuEV == 0.2
    assert p.nu_FilenameTransferInfofile == info.encode()
    with pytest.raises(M.MGPError, match="miss a value for tag 'nu_SumMassNuEV'"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_FOFR, extra=keys.replace("nu_SumMassNuEV 0.2\n", "")),
                             M.MODEL_FOFR, massive_neutrinos=True)
    with pytest.raises(M.MGPError, match="not allowed or multiple"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_FOFR, extra=keys), M.MODEL_FOFR)


def test_neutrino_reader_errors(tmp_path, info):
    with pytest.raises(M.MGPError, match="cannot read"):
        M.cosmo_eval(nu_params(str(tmp_path / "missing.txt")), 0, np.array([1.0]))
    with pytest.raises(M.MGPError, match="SCALEDEPENDENT"):
        M.cosmo_eval(nu_params(info, scaledependent=0), 0, np.array([1.0]))


# --------------------------------------------------------------------------
# The reference's own CAMB example tables (camb_data/example_data_nu0.4, the
# inputs of its f(R)+neutrino test runs) and its own neutrino build, where
# the reference tree is given (MGP_REFERENCE_SRC = its src/ directory).
REAL_COSMO = dict(Omega=0.3175, OmegaBaryon=0.049, HubbleParam=0.671, Sigma8=0.7656, PrimordialIndex=0.966)


@pytest.fixture(scope="module")
def real_info(tmp_path_factory):
    from oracle import ref_build
    if not ref_build.available():
        pytest.skip("reference tree not given (MGP_REFERENCE_SRC)")
    d = os.path.join(os.path.dirname(ref_build.REF_SRC), "camb_data", "example_data_nu0.4")
    if not os.path.isdir(d):
        pytest.skip("reference CAMB example data not present")
    lines = open(os.path.join(d, "picola_transfer_info_nu0.4.txt")).read().split("\n")
    # the info file names its author's directory: point it at this copy
    info = os.path.join(str(tmp_path_factory.mktemp("realcamb")), "info.txt")
    with open(info, "w") as f:
        f.write("%s %s\n" % (d, lines[0].split()[1]) + "\n".join(lines[1:]) + "\n")
    return info


@pytest.mark.parametrize("model", ["lcdm", "fofr"])
def test_host_cosmology_on_reference_camb_tables(real_info, model):
    p = nu_params(real_info, model, nu_SumMassNuEV=0.4, fofr0=1e-4, **REAL_COSMO)
    nu, cos = oracle_cosmo(real_info, p, model)
    assert nu.omega_nu == pytest.approx(0.4 / (93.14 * 0.671 ** 2), rel=1e-14)
    kk, aa = (g.ravel() for g in np.meshgrid(np.array([0.01, 0.1, 0.5, 2.0]), np.array([0.05, 0.5]), indexing="ij"))
    for which in (0, 2, 3):
        np.testing.assert_allclose(M.growth_scaledependent(p, which, kk, aa),
                                   [cos.growth_sd(which, x, y) for x, y in zip(kk, aa)], rtol=2e-5)
    pw = O.make_power(omega=p.Omega, omega_b=p.OmegaBaryon, h=p.HubbleParam, ns=p.PrimordialIndex, sigma8=p.Sigma8,
                      nu=nu)
    k = np.array([1e-3, 0.05, 0.3, 2.0])
    np.testing.assert_allclose(M.cosmo_eval(p, 7, k), [O.lib().orc_power_spec(C.byref(pw), x) for x in k], rtol=1e-9)


def test_oracle_matches_reference_run_on_its_camb_tables(real_info, tmp_path):
    """The reference's f(R)+neutrino build (f_R0 = 1e-4, 0.4 eV, its example
    cosmology) run here on its own CAMB tables, against the oracle's loop."""
    from oracle import ref_build
    from golden import make_golden
    ref_build.build(models=["FOFRNU"])
    mg = dict(modified_gravity_active=1, fofr0=1e-4, nfofr=1.0, include_screening=1, inverted_initial_condition=0,
              amplitude_fixed_initial_condition=0, nu_include_massive_neutrinos=1, nu_SumMassNuEV=0.4)
    base = dict(Box=256.0)
    r = make_golden.run_reference("FOFRNU", mg, base=base, cosmo=REAL_COSMO, nu_info=real_info)
    nu = O.Neutrinos(real_info, 0.3175, 0.049, 0.671, 0.966, 0.4, 1)
    rp = O.RunParams()
    rp.mg = O.make_mg(O.FOFR, 0.3175, mg_active=1, include_screening=1, fofr0=1e-4, nfofr=1.0, scaledependent=1,
                      nu=nu)
    rp.pw = O.make_power(omega=0.3175, omega_b=0.049, h=0.671, ns=0.966, sigma8=0.7656, nu=nu)
    b = dict(make_golden.BASE, **base)
    rp.ic = O.ICParams(b["Nmesh"], b["Nsample"], b["Box"], b["Seed"], 0, 0, 0, 1.0)
    rp.init_redshift, rp.nsteps, rp.final_redshift = b["Init_Redshift"], b["nsteps"], 0.0
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = 16, 0, 0
    rp.pofk_kmin, rp.pofk_kmax, rp.usecola = 0.0, 0.0, 1
    n = b["Nsample"] ** 3
    pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
    kb, pk, km, nm = (np.zeros(b["Nmesh"]) for _ in range(4))
    nb = O.lib().orc_run(rp, pos, vel, kb, pk, km, nm)
    m = nm[:nb] > 0
    m[0] = False
    ref = r["pk_total"]
    assert ref.shape[0] == m.sum()
    np.testing.assert_allclose(pk[:nb][m], ref[:, 1], rtol=1e-6, atol=6e-6)
    dx = np.abs(pos - r["pos"])
    dx = np.minimum(dx, b["Box"] - dx)
    assert dx.max() < 2e-5 * b["Box"]
    v = 100.0 * vel
    assert np.abs(r["vel"] - v).max() < 1e-6 * np.abs(v).max() + 1e-5
    # the neutrinos are visible: total below CDM on every bin
    assert np.all(r["pk_total"][:, 1] < r["pk"][:, 1])
