"""CPU tests of the host side of libmgpicola.so: exported ABI, the
parameter-file reader and the FP64 host cosmology (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "mgpicola.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(mgp_[A-Za-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    L = M.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(M.EXPORTS) <= set(syms)


def test_params_struct_layout_matches_c():
    # the ctypes mirror must have the C size: check by round-tripping defaults
    p = M.default_params()
    assert p.Nmesh == 64 and p.Omega == pytest.approx(0.267) and p.UnitLength_in_cm == pytest.approx(3.085678e24)
    assert p.Noutputs == 1 and p.output_nsteps[0] == 10


STD = """% comment line
OutputDir                   {out}
FileBase                    test
OutputRedshiftFile          {out}/output_redshifts.dat
NumFilesWrittenInParallel   1
UseCOLA          1
Buffer           1.5
Nmesh            64
Nsample          32
Box              200.0
Init_Redshift    19.0
Seed             5001
SphereMode       0
WhichSpectrum    2
WhichTransfer    0
FileWithInputSpectrum  none
FileWithInputTransfer  none
Omega            0.267
OmegaBaryon      0.049
HubbleParam      0.71
Sigma8           0.8
PrimordialIndex  0.966
UnitLength_in_cm                3.085678e24
UnitMass_in_g                   1.989e43
UnitVelocity_in_cm_per_s        1e5
InputSpectrum_UnitLength_in_cm  3.085678e24
modified_gravity_active  1
include_screening        1
use_lcdm_growth_factors  0
input_pofk_is_for_lcdm   1
input_sigma8_is_for_lcdm 1
inverted_initial_condition        0
amplitude_fixed_initial_condition 0
"""
POFK = """pofk_compute_every_step   1
pofk_compute_rsd_pofk     2
pofk_nbins                64
pofk_bintype              1
pofk_subtract_shotnoise   1
pofk_kmin                 0.03
pofk_kmax                 2.0
"""
MODEL_KEYS = {M.MODEL_FOFR: "fofr0 1e-5\nnfofr 1.0\n", M.MODEL_DGP: "Rsmooth 1.0\nrcH0_DGP 1.2\n",
              M.MODEL_LCDM: "", M.MODEL_BRANSDICKE: "wBD 100\nOmegah2 0.14\nOmegar2 4e-5\nOmegav2 0.36\n",
              M.MODEL_MBETA: "range_symm 1.0\nassb_symm 0.5\nbeta_symm 1.0\n"}


def write_param(tmp_path, model, extra="", drop=None, pofk=True):
    out = str(tmp_path)
    with open(os.path.join(out, "output_redshifts.dat"), "w") as f:
        f.write("% header\n1.0, 5\n0, 10\n")
    txt = STD.format(out=out) + (POFK if pofk else "") + MODEL_KEYS[model] + extra
    if drop:
        txt = "\n".join(l for l in txt.splitlines() if not l.startswith(drop))
    fn = os.path.join(out, "params.txt")
    with open(fn, "w") as f:
        f.write(txt)
    return fn


@pytest.mark.parametrize("model", [M.MODEL_LCDM, M.MODEL_FOFR, M.MODEL_DGP, M.MODEL_BRANSDICKE, M.MODEL_MBETA])
def test_parameter_file_all_models(tmp_path, model):
    p = M.read_parameterfile(write_param(tmp_path, model), model)
    assert p.Nmesh == 64 and p.Nsample == 32 and p.Box == 200.0 and p.Seed == 5001
    assert p.pofk_nbins == 64 and p.pofk_bintype == 1 and p.pofk_kmax == 2.0
    # outputs sorted by descending redshift (read_outputs)
    assert p.Noutputs == 2 and p.output_redshift[0] == 1.0 and p.output_nsteps[1] == 10
    if model == M.MODEL_DGP:
        assert p.rcH0_DGP == 1.2 and p.smoothing_filter == M.FILTER_GAUSSIAN
    if model == M.MODEL_BRANSDICKE:
        assert p.Omegarh2 == 4e-5 and p.Omegavh2 == 0.36


def test_parameter_file_errors(tmp_path):
    with pytest.raises(M.MGPError, match="miss a value for tag 'Seed'"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, drop="Seed"), M.MODEL_LCDM)
    with pytest.raises(M.MGPError, match="not allowed or multiple"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, extra="Bogus 1\n"), M.MODEL_LCDM)
    with pytest.raises(M.MGPError, match="not allowed or multiple"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, extra="Seed 7\n"), M.MODEL_LCDM)
    # an f(R) key is unknown to the DGP model
    with pytest.raises(M.MGPError, match="fofr0"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_DGP, extra="fofr0 1e-5\n"), M.MODEL_DGP)
    with pytest.raises(M.MGPError, match="not found"):
        M.read_parameterfile(str(tmp_path / "nope.txt"), M.MODEL_LCDM)
    # without COMPUTE_POFK keys the pofk_* keys are unknown
    with pytest.raises(M.MGPError):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM), M.MODEL_LCDM, pofk_keys=False)
    p = M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, pofk=False), M.MODEL_LCDM, pofk_keys=False)
    assert p.pofk_nbins == 32


def test_host_cosmology_matches_oracle():
    p = M.default_params(Init_Redshift=19.0)
    a = np.array([0.05, 0.1, 0.3, 0.5, 1.0])
    cos = O.Cosmo(O.make_mg(O.LCDM, p.Omega), 19.0)
    names = ["growth_D", "growth_dDdy", "growth_ddDddy", "growth_D2", "growth_dD2dy", "growth_ddD2ddy",
             "growth_DLCDM"]
    for which, name in enumerate(names):
        got = M.cosmo_eval(p, which, a)
        ref = np.array([getattr(cos, name)(x) for x in a])
        np.testing.assert_allclose(got, ref, rtol=1e-9)
    ai, af, ar = np.array([0.05, 0.3]), np.array([0.1, 0.35]), np.array([0.07, 0.32])
    np.testing.assert_allclose(M.cosmo_coeff(p, 0, ai, af, ar), [cos.Sq(*t) for t in zip(ai, af, ar)], rtol=1e-11)
    np.testing.assert_allclose(M.cosmo_coeff(p, 1, ai, af, ar), [cos.Sphi(*t) for t in zip(ai, af, ar)], rtol=1e-12)
    pw = O.make_power()
    k = np.array([1e-3, 0.01, 0.1, 1.0, 10.0])
    np.testing.assert_allclose(M.cosmo_eval(p, 7, k), [O.lib().orc_power_spec(C.byref(pw), x) for x in k],
                               rtol=1e-10)


def test_host_standard_pm_coefficients_match_oracle():
    """Quinn et al. kick/drift coefficients of the non-COLA run (UseCOLA 0:
    StdDA 2, steps in ln a; src/cosmo.c:1165-1200, main.c:75-81)."""
    p = M.default_params(Init_Redshift=19.0, UseCOLA=0)
    cos = O.Cosmo(O.make_mg(O.LCDM, p.Omega), 19.0)
    ai, af = np.array([0.05, 0.3, 0.7]), np.array([0.08, 0.35, 0.9])
    np.testing.assert_allclose(M.cosmo_coeff(p, 2, ai, af, af), [cos.SqStd(*t) for t in zip(ai, af)], rtol=1e-11)
    np.testing.assert_allclose(M.cosmo_coeff(p, 3, ai, af, af), [cos.SphiStd(*t) for t in zip(ai, af)], rtol=1e-11)
    with pytest.raises(M.MGPError):
        M.cosmo_coeff(p, 4, ai, af, af)


def test_host_cosmology_mg_models():
    for model, kw, omk in [(M.MODEL_FOFR, dict(fofr0=1e-5, nfofr=1.0), dict(model=O.FOFR)),
                           (M.MODEL_DGP, dict(rcH0_DGP=1.0), dict(model=O.DGP))]:
        p = M.default_params(model=model, modified_gravity_active=1, **kw)
        mg = O.make_mg(omk["model"], p.Omega, fofr0=p.fofr0, nfofr=p.nfofr, rcH0=p.rcH0_DGP)
        cos = O.Cosmo(mg, 19.0)
        a = np.array([0.1, 0.5, 1.0])
        np.testing.assert_allclose(M.cosmo_eval(p, 0, a), [cos.growth_D(x) for x in a], rtol=1e-9)
        np.testing.assert_allclose(M.cosmo_eval(p, 3, a), [cos.growth_D2(x) for x in a], rtol=1e-9)


def test_create_fails_loudly_without_device_or_bad_params():
    p = M.default_params(Nmesh=7)
    with pytest.raises(M.MGPError):
        M.Context(p)


def test_host_cosmology_jbd_and_mbeta_and_w0wa():
    # Brans-Dicke: background solved by shooting (src/jbd.c); Omega and h are
    # replaced by the solution (user_defined_functions.h:135-143)
    p = M.default_params(model=M.MODEL_BRANSDICKE, modified_gravity_active=1, wBD=100.0, Omegah2=0.14,
                         Omegarh2=4e-5, Omegavh2=0.36)
    mg = O.make_mg(O.JBD_GEFF, 0.267, wBD=100.0, Omegah2=0.14, Omegarh2=4e-5, Omegavh2=0.36)
    cos = O.Cosmo(mg, 19.0)
    a = np.array([0.05, 0.2, 0.6, 1.0])
    np.testing.assert_allclose(M.cosmo_eval(p, 0, a), [cos.growth_D(x) for x in a], rtol=1e-7)
    np.testing.assert_allclose(M.cosmo_eval(p, 3, a), [cos.growth_D2(x) for x in a], rtol=1e-7)
    # symmetron-type m(a), beta(a): growth only changes through Geff(k = 1e-3)
    p = M.default_params(model=M.MODEL_MBETA, modified_gravity_active=1, assb_symm=0.5, beta_symm=1.0,
                         range_symm=1.0)
    mg = O.make_mg(O.MBETA, 0.267, assb_symm=0.5, beta_symm=1.0, range_symm=1.0)
    cos = O.Cosmo(mg, 19.0)
    np.testing.assert_allclose(M.cosmo_eval(p, 0, a), [cos.growth_D(x) for x in a], rtol=1e-9)
    # w0/wa background
    p = M.default_params(use_w0wa=1, w_0=-0.9, w_a=0.2)
    mg = O.make_mg(O.LCDM, 0.267, use_w0wa=1, w0=-0.9, wa=0.2)
    cos = O.Cosmo(mg, 19.0)
    np.testing.assert_allclose(M.cosmo_eval(p, 0, a), [cos.growth_D(x) for x in a], rtol=1e-9)


# The reference's own example parameter files (paramfiles/example_*.txt and
# the additions_*.txt keys of its COMPUTE_POFK / READICFROMFILE / MatchMaker
# builds), as the (key, value) tokens its parser sees
# (tests/golden/make_paramfile_golden.py), each with the MODEL its build uses.
REF_PARAMFILES = {
    "example_dgp_noscreening.txt": M.MODEL_DGP, "example_dgp_withscreening.txt": M.MODEL_DGP,
    "example_lcdm_dgpversion.txt": M.MODEL_DGP, "example_fofr_noscreening.txt": M.MODEL_FOFR,
    "example_fofr_withscreening.txt": M.MODEL_FOFR, "example_fofr_withscreening_lcdmgrowthfac.txt": M.MODEL_FOFR,
    "example_lcdm_fofrversion.txt": M.MODEL_FOFR, "example_mbeta.txt": M.MODEL_MBETA,
}


def _ref_tokens():
    import json
    return json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_paramfiles.json")))


def _write_tokens(path, pairs):
    with open(path, "w") as f:
        f.write("% written from the reference's example file\n")
        for k, v in pairs:
            f.write("%s %s\n" % (k, v))
    return str(path)


def _check_values(p, pairs):
    import ctypes as C
    for k, v in pairs:
        got = getattr(p, k)
        if isinstance(got, bytes):
            assert got.decode() == v, k
        elif isinstance(got, int):
            assert got == int(C.c_int(int(v)).value), k
        else:
            assert got == float(v), k


@pytest.mark.parametrize("name", sorted(REF_PARAMFILES))
@pytest.mark.parametrize("pofk", [False, True])
def test_reference_example_paramfiles_parse(tmp_path, name, pofk):
    """Every example file of the reference parses with its build's model,
    with and without the COMPUTE_POFK keys, to the values it states."""
    tok = _ref_tokens()
    pairs = tok[name] + (tok["additions_compute_pofk.txt"] if pofk else [])
    p = M.read_parameterfile(_write_tokens(tmp_path / name, pairs), REF_PARAMFILES[name], pofk_keys=pofk,
                             read_outputs=False)
    _check_values(p, pairs)
    if not pofk:
        assert p.pofk_compute_every_step == 0 and p.pofk_nbins == p.Nmesh // 2


def test_reference_readic_additions_parse(tmp_path):
    tok = _ref_tokens()
    pairs = tok["example_fofr_withscreening.txt"] + tok["additions_readicfromfile.txt"]
    p = M.read_parameterfile(_write_tokens(tmp_path / "ic.txt", pairs), M.MODEL_FOFR, pofk_keys=False,
                             read_outputs=False, read_ic_from_file=True)
    _check_values(p, pairs)
    # without the READICFROMFILE build the six keys are not allowed
    with pytest.raises(M.MGPError, match="ReadParticlesFromFile"):
        M.read_parameterfile(_write_tokens(tmp_path / "ic2.txt", pairs), M.MODEL_FOFR, pofk_keys=False,
                             read_outputs=False)


def test_reference_halofinder_keys_are_not_accepted(tmp_path):
    """The MatchMaker halo finder is not part of this library: its keys are
    unknown tags, as in a reference build without MATCHMAKER_HALOFINDER."""
    tok = _ref_tokens()
    pairs = tok["example_dgp_withscreening.txt"] + tok["additions_halofinder.txt"]
    with pytest.raises(M.MGPError, match="Tag '%s' not allowed" % tok["additions_halofinder.txt"][0][0]):
        M.read_parameterfile(_write_tokens(tmp_path / "hf.txt", pairs), M.MODEL_DGP, pofk_keys=False,
                             read_outputs=False)


def test_reference_bransdicke_example_keeps_the_key_mismatch(tmp_path):
    """Kept quirk: the reference's parser registers the Brans-Dicke keys
    Omegar2 and Omegav2 (src/user_defined_functions.h:389-399) while its
    example file names them Omegarh2 and Omegavh2 and gives no values, so
    its own BRANSDICKE build rejects that file.  The same file is rejected
    here with the reference's message; with the registered names and values
    it parses."""
    tok = _ref_tokens()
    pairs = tok["example_bransdicke.txt"]
    with pytest.raises(M.MGPError, match="Tag 'Omegarh2' not allowed"):
        M.read_parameterfile(_write_tokens(tmp_path / "bd.txt", pairs), M.MODEL_BRANSDICKE, pofk_keys=False,
                             read_outputs=False)
    fixed = [{"Omegarh2": ["Omegar2", "4e-5"], "Omegavh2": ["Omegav2", "0.36"], "wBD": ["wBD", "100"],
              "Omegah2": ["Omegah2", "0.14"]}.get(k, [k, v]) for k, v in pairs]
    p = M.read_parameterfile(_write_tokens(tmp_path / "bd2.txt", fixed), M.MODEL_BRANSDICKE, pofk_keys=False,
                             read_outputs=False)
    assert (p.wBD, p.Omegah2, p.Omegarh2, p.Omegavh2) == (100.0, 0.14, 4e-5, 0.36)
