"""2LPT initial conditions from particles (ReadParticlesFromFile,
src/readICfromfile.c:133-777) against the FP64 oracle on the same positions:
the particles of a Gaussian IC are deposited, their density taken as the
LCDM linear field at Init_Redshift, deconvolved, rescaled and turned into
ZA and 2LPT displacements.  Bar as the Gaussian IC: ZA rms relative error
< 1e-4, 2LPT < 1e-3 (the GPU deposits in float)."""
import ctypes as C
import os

import numpy as np
import pytest

import mgpicola as M
from oracle import oracle as O
from test_icfile import gadget_file

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, float) - b) ** 2) / np.mean(np.asarray(b, float) ** 2)))


def make(N, Ns, box, model, **kw):
    d = dict(Nmesh=N, Nsample=Ns, Box=box, Seed=4242, Init_Redshift=19.0, pofk_compute_every_step=0)
    mg = O.make_mg(O.LCDM, 0.267)
    if model == "fofr":
        d.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0,
                 input_pofk_is_for_lcdm=1)
        mg = O.make_mg(O.FOFR, 0.267, fofr0=1e-5, nfofr=1.0)
    d.update(kw)
    return M.default_params(**d), mg


def oracle_ic(p, mg, pos01):
    N, Ns, box = p.Nmesh, p.Nsample, p.Box
    cosmo = O.Cosmo(mg, p.Init_Redshift)
    ai = 1.0 / (1.0 + p.Init_Redshift)
    normfac = 1.0 / N ** 3 / cosmo.growth_DLCDM(ai)
    rk = np.arange(3 * (N // 2) ** 2 + 1)
    ks = 2 * np.pi / box * np.sqrt(rk)
    resc = np.array([1.0] + [np.sqrt(cosmo.mg_pofk_ratio(k, 1.0)) for k in ks[1:]])
    if not p.input_sigma8_is_for_lcdm:
        pw = O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8)
        resc /= O.lib().orc_mg_sigma8_enh(cosmo.h, C.byref(pw), 1.0)
    return O.ic_2lpt_from_particles(N, Ns, box, pos01, normfac, resc)


def gaussian_particles(p):
    with M.Context(p) as c:
        c.displacement_fields()
        return c.get_particles()[0].astype(np.float64)


def test_ic_from_positions_matches_oracle():
    p, mg = make(32, 16, 128.0, "lcdm")
    pos = gaussian_particles(p)
    with M.Context(p) as c:
        c.displacement_fields_from_positions(pos)
        x, v, d1, d2 = c.get_particles()
    u = pos / p.Box
    u -= np.floor(u)
    D1, D2 = oracle_ic(p, mg, u)
    assert rel_rms(d1, D1) < 1e-4
    assert rel_rms(d2, D2) < 1e-3
    assert np.abs(d1).max() > 0.1 * p.Box / p.Nsample  # a non-trivial field


def test_ic_from_gadget_files_matches_oracle(tmp_path):
    """f(R) with the MG P(k) rescaling and a sigma8 quoted for f(R), Nmesh =
    Nsample (the Nyquist planes of the field zeroed), two GADGET-1 files."""
    p, mg = make(16, 16, 64.0, "fofr", input_sigma8_is_for_lcdm=0)
    pos = gaussian_particles(p)
    half = len(pos) // 2
    gadget_file(os.path.join(tmp_path, "ics.0"), pos[:half], p.Box)
    gadget_file(os.path.join(tmp_path, "ics.1"), pos[half:], p.Box)
    p.ReadParticlesFromFile, p.TypeInputParticleFiles, p.NumInputParticleFiles = 1, 3, 2
    p.InputParticleFileDir, p.InputParticleFilePrefix = str(tmp_path).encode(), b"ics"
    u = M.read_particle_files(p)
    with M.Context(p) as c:
        c.displacement_fields()
        x, v, d1, d2 = c.get_particles()
    D1, D2 = oracle_ic(p, mg, u)
    assert rel_rms(d1, D1) < 1e-4
    assert rel_rms(d2, D2) < 1e-3


def test_ic_from_positions_recovers_a_gaussian_field():
    """The density of ZA-displaced particles at high redshift is the linear
    field: the IC rebuilt from them reproduces the original ZA displacements
    on large scales (k well below the particle Nyquist frequency)."""
    p, _ = make(64, 32, 256.0, "lcdm", Init_Redshift=49.0)
    with M.Context(p) as c:
        c.displacement_fields()
        pos, _, d1_ref, _ = c.get_particles()
    with M.Context(p) as c:
        c.displacement_fields_from_positions(pos.astype(np.float64))
        _, _, d1, _ = c.get_particles()
    # low-pass both displacement fields on the particle lattice and compare
    Ns = p.Nsample
    f = [np.fft.rfftn(a.reshape(Ns, Ns, Ns, 3)[..., q]) for a in (d1, d1_ref) for q in range(3)]
    kk = np.sqrt(np.fft.fftfreq(Ns, 1 / Ns)[:, None, None] ** 2 + np.fft.fftfreq(Ns, 1 / Ns)[None, :, None] ** 2 +
                 np.arange(Ns // 2 + 1)[None, None, :] ** 2)
    m = (kk > 0) & (kk < Ns / 8)
    num = sum(np.sum(np.abs(f[q][m] - f[q + 3][m]) ** 2) for q in range(3))
    den = sum(np.sum(np.abs(f[q + 3][m]) ** 2) for q in range(3))
    assert np.sqrt(num / den) < 0.05
