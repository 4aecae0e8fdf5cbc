"""ctypes binding of the FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module; the shipped library never does.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build  # noqa: F401  (package-relative when imported as oracle.oracle)

_lib = None

dptr = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
u32ptr = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")

LCDM, FOFR, DGP, JBD_GEFF, MBETA = 0, 1, 2, 3, 4


class MG(C.Structure):
    _fields_ = [("model", C.c_int), ("mg_active", C.c_int), ("include_screening", C.c_int),
                ("use_lcdm_growth", C.c_int), ("omega", C.c_double), ("fofr0", C.c_double),
                ("nfofr", C.c_double), ("rcH0", C.c_double), ("rsmooth", C.c_double),
                ("geff_const", C.c_double), ("w0", C.c_double), ("wa", C.c_double), ("use_w0wa", C.c_int),
                ("beta_symm", C.c_double), ("assb_symm", C.c_double), ("range_symm", C.c_double),
                ("smoothing_filter", C.c_int), ("wBD", C.c_double), ("Omegah2", C.c_double),
                ("Omegarh2", C.c_double), ("Omegavh2", C.c_double), ("scaledependent", C.c_int),
                ("sd_nk", C.c_int), ("sd_kmin", C.c_double), ("sd_kmax", C.c_double), ("nu", C.c_void_p)]


class Power(C.Structure):
    _fields_ = [("which_spectrum", C.c_int), ("omega", C.c_double), ("omega_b", C.c_double),
                ("h", C.c_double), ("ns", C.c_double), ("sigma8", C.c_double), ("ntab", C.c_int),
                ("tab_logk", C.POINTER(C.c_double)), ("tab_logP", C.POINTER(C.c_double)),
                ("norm", C.c_double), ("nu", C.c_void_p), ("nu_ocdm", C.c_double)]


class ICParams(C.Structure):
    _fields_ = [("N", C.c_int), ("Ns", C.c_int), ("box", C.c_double), ("seed", C.c_uint32),
                ("sphere_mode", C.c_int), ("fixed_amplitude", C.c_int), ("inverted", C.c_int),
                ("pofk_rescale", C.c_double)]


class RunParams(C.Structure):
    _fields_ = [("mg", MG), ("pw", Power), ("ic", ICParams), ("init_redshift", C.c_double),
                ("nsteps", C.c_int), ("final_redshift", C.c_double), ("pofk_nbins", C.c_int),
                ("pofk_bintype", C.c_int), ("pofk_subtract_shotnoise", C.c_int), ("pofk_kmin", C.c_double),
                ("pofk_kmax", C.c_double), ("usecola", C.c_int), ("ic_pos01", C.c_void_p), ("ic_n", C.c_long),
                ("ic_rescale_rk", C.c_void_p), ("stop_step", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_philox4x32_10.argtypes = [u32ptr, u32ptr, u32ptr]
        L.orc_stream_uniform.argtypes = [C.c_uint32, C.c_uint64]
        L.orc_stream_uniform.restype = C.c_double
        L.orc_fft_r2c.argtypes = [C.c_int, dptr]
        L.orc_fft_c2r.argtypes = [C.c_int, dptr]
        L.orc_fft1d.argtypes = [C.c_int, dptr, C.c_int]
        L.orc_cic.argtypes = [dptr, C.c_long, C.c_int, C.c_int, C.c_double, dptr]
        L.orc_lattice_positions.argtypes = [dptr, C.c_int, C.c_double, dptr]
        L.orc_forces_kspace.argtypes = [dptr, C.c_void_p, C.c_int, C.c_double, dptr, dptr, dptr]
        L.orc_interp.argtypes = [dptr, dptr, dptr, C.c_int, C.c_double, dptr, C.c_long, dptr, dptr]
        L.orc_kick.argtypes = [C.c_long, dptr, dptr, dptr, dptr, dptr, C.c_double, C.c_double, C.c_double,
                               C.c_double, C.c_double, C.c_int, dptr]
        L.orc_drift.argtypes = [C.c_long, dptr, dptr, dptr, dptr, dptr, C.c_double, C.c_double, C.c_double,
                                C.c_int, C.c_double]
        L.orc_periodic_wrap.argtypes = [C.c_double, C.c_double]
        L.orc_periodic_wrap.restype = C.c_double
        L.orc_pofk.argtypes = [dptr, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int), C.c_int, C.c_int,
                               C.c_double, C.c_double, dptr, dptr, dptr, dptr]
        L.orc_pofk.restype = C.c_int
        L.orc_pofk_rsd_axis.argtypes = [dptr, dptr, C.c_void_p, C.c_long, C.c_int, C.c_int, C.c_int, C.c_double,
                                        C.c_double, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_double, C.c_double,
                                        dptr, dptr, dptr, dptr, dptr]
        L.orc_pofk_rsd_axis.restype = C.c_int
        L.orc_fifth_force.argtypes = [C.POINTER(MG), C.c_double, C.c_int, C.c_double, dptr, dptr, dptr]
        for name in ["orc_hubble", "orc_dhubbleda", "orc_beta_dgp", "orc_beta_of_a", "orc_mass2_of_a",
                     "orc_coupling", "orc_factor_2lpt"]:
            f = getattr(L, name)
            f.argtypes = [C.POINTER(MG), C.c_double]
            f.restype = C.c_double
        L.orc_geff.argtypes = [C.POINTER(MG), C.c_double, C.c_double]
        L.orc_geff.restype = C.c_double
        L.orc_screen_potential.argtypes = [C.POINTER(MG), C.c_double, C.c_double]
        L.orc_screen_potential.restype = C.c_double
        L.orc_screen_density.argtypes = [C.POINTER(MG), C.c_double, C.c_double]
        L.orc_screen_density.restype = C.c_double
        L.orc_cosmo_create.argtypes = [C.POINTER(MG), C.c_double]
        L.orc_cosmo_create.restype = C.c_void_p
        L.orc_cosmo_create_sd.argtypes = [C.POINTER(MG), C.c_double, C.c_double, C.c_int]
        L.orc_cosmo_create_sd.restype = C.c_void_p
        L.orc_growth_sd.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.orc_growth_sd.restype = C.c_double
        L.orc_mg_pofk_ratio.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_mg_pofk_ratio.restype = C.c_double
        L.orc_mg_sigma8_enh.argtypes = [C.c_void_p, C.POINTER(Power), C.c_double]
        L.orc_mg_sigma8_enh.restype = C.c_double
        L.orc_dmass2_of_ada.argtypes = [C.POINTER(MG), C.c_double]
        L.orc_dmass2_of_ada.restype = C.c_double
        L.orc_second_order_kernel.argtypes = [C.POINTER(MG), C.c_double, C.c_double, C.c_double, C.c_double,
                                              C.c_double]
        L.orc_second_order_kernel.restype = C.c_double
        L.orc_sd_field.argtypes = [C.c_void_p, dptr, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_int, C.c_int, dptr]
        L.orc_cosmo_free.argtypes = [C.c_void_p]
        for name in ["orc_growth_D", "orc_growth_dDdy", "orc_growth_ddDddy", "orc_growth_D2", "orc_growth_dD2dy",
                     "orc_growth_ddD2ddy", "orc_growth_DLCDM"]:
            f = getattr(L, name)
            f.argtypes = [C.c_void_p, C.c_double]
            f.restype = C.c_double
        for name in ["orc_SqStd", "orc_SphiStd"]:
            f = getattr(L, name)
            f.argtypes = [C.c_void_p, C.c_double, C.c_double]
            f.restype = C.c_double
        for name in ["orc_Sq", "orc_Sphi"]:
            f = getattr(L, name)
            f.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
            f.restype = C.c_double
        L.orc_growthD_fit.argtypes = [C.c_double, C.c_double]
        L.orc_growthD_fit.restype = C.c_double
        L.orc_power_init.argtypes = [C.POINTER(Power)]
        L.orc_power_spec.argtypes = [C.POINTER(Power), C.c_double]
        L.orc_power_spec.restype = C.c_double
        L.orc_tophat_sigma2.argtypes = [C.POINTER(Power), C.c_double]
        L.orc_tophat_sigma2.restype = C.c_double
        L.orc_seedtable.argtypes = [C.c_int, C.c_uint32, u32ptr]
        L.orc_ic_2lpt.argtypes = [C.POINTER(ICParams), C.POINTER(Power), dptr, dptr, C.c_void_p, C.c_void_p]
        L.orc_ic_2lpt_from_particles.argtypes = [C.POINTER(ICParams), dptr, C.c_long, C.c_double, dptr, dptr, dptr,
                                                 C.c_void_p, C.c_void_p]
        L.orc_jbd_solve.argtypes = [C.POINTER(MG)]
        L.orc_jbd_solve.restype = C.c_double
        L.orc_phia_solve.argtypes = [C.POINTER(MG), C.c_double]
        L.orc_phicrit.argtypes = [C.POINTER(MG), C.c_double]
        L.orc_phicrit.restype = C.c_double
        L.orc_run.argtypes = [C.POINTER(RunParams), dptr, dptr, dptr, dptr, dptr, dptr]
        L.orc_run.restype = C.c_int
        L.orc_time_steps.argtypes = [C.POINTER(RunParams), C.c_int]
        L.orc_time_steps.restype = C.c_double
        L.orc_nu_create.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_nu_create.restype = C.c_void_p
        L.orc_nu_free.argtypes = [C.c_void_p]
        for name in ["orc_nu_omega_nu", "orc_nu_omega_cdm", "orc_nu_mu2"]:
            getattr(L, name).argtypes = [C.c_void_p]
            getattr(L, name).restype = C.c_double
        L.orc_nu_transfer.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.orc_nu_transfer.restype = C.c_double
        L.orc_nu_Tcb.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.orc_nu_Tcb.restype = C.c_double
        L.orc_nu_mu1.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_nu_mu1.restype = C.c_double
        L.orc_nu_pofk_cb.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_nu_pofk_cb.restype = C.c_double
        L.orc_nu_add_density.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_double, dptr, dptr]
        _lib = L
    return _lib


# ------------------------------------------------------------------ helpers
def padded_shape(N):
    return (N, N, 2 * (N // 2 + 1))


def to_complex(grid, N):
    """View an [N][N][2(N/2+1)] float64 grid as complex [N][N][N/2+1]."""
    return grid.view(np.complex128).reshape(N, N, N // 2 + 1)


def fft_r2c(real_NNN):
    N = real_NNN.shape[0]
    g = np.zeros(padded_shape(N))
    g[:, :, :N] = real_NNN
    lib().orc_fft_r2c(N, g)
    return g


def fft_c2r(ck):
    N = ck.shape[0]
    g = np.ascontiguousarray(ck.astype(np.complex128)).view(np.float64).reshape(padded_shape(N)).copy()
    lib().orc_fft_c2r(N, g)
    return g


def cic(pos, N, Ns, box):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    g = np.zeros(padded_shape(N))
    lib().orc_cic(pos.reshape(-1), pos.shape[0], N, Ns, box, g)
    return g


def pofk(deltak_grid, N, Ns, box, nbins, bintype, sub, kmin, kmax):
    cap = max(nbins, N) if nbins > 0 else N
    kb, pk, km, nm = (np.zeros(cap) for _ in range(4))
    nb = C.c_int(nbins)
    lib().orc_pofk(deltak_grid, N, Ns, box, C.byref(nb), bintype, sub, kmin, kmax, kb, pk, km, nm)
    n = nb.value
    return kb[:n], pk[:n], km[:n], nm[:n]


def forces_kspace(deltak_grid, N, box, mgk=None):
    f = [np.zeros(padded_shape(N)) for _ in range(3)]
    lib().orc_forces_kspace(deltak_grid, None if mgk is None else mgk.ctypes.data, N, box, f[0], f[1], f[2])
    return f


def interp(f, N, box, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    disp = np.zeros_like(pos)
    mean = np.zeros(3)
    lib().orc_interp(f[0], f[1], f[2], N, box, pos.reshape(-1), pos.shape[0], disp.reshape(-1), mean)
    return disp, mean


class Cosmo:
    def __init__(self, mg, init_redshift, box=0.0, nmesh=0):
        self.mg = mg
        self.h = lib().orc_cosmo_create_sd(C.byref(mg), init_redshift, box, nmesh)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cosmo_free(self.h)
            self.h = None

    def __getattr__(self, name):
        f = getattr(lib(), "orc_" + name)
        return lambda *a: f(self.h, *a)


def make_mg(model=LCDM, omega=0.267, **kw):
    m = MG()
    m.model = model
    m.omega = omega
    m.mg_active = kw.get("mg_active", 1 if model != LCDM else 0)
    m.include_screening = kw.get("include_screening", 1)
    m.use_lcdm_growth = kw.get("use_lcdm_growth", 0)
    m.fofr0 = kw.get("fofr0", 1e-5)
    m.nfofr = kw.get("nfofr", 1.0)
    m.rcH0 = kw.get("rcH0", 1.0)
    m.rsmooth = kw.get("rsmooth", 1.0)
    m.geff_const = kw.get("geff_const", 1.0)
    m.w0 = kw.get("w0", -1.0)
    m.wa = kw.get("wa", 0.0)
    m.use_w0wa = kw.get("use_w0wa", 0)
    m.beta_symm = kw.get("beta_symm", 1.0)
    m.assb_symm = kw.get("assb_symm", 0.5)
    m.range_symm = kw.get("range_symm", 1.0)
    m.smoothing_filter = kw.get("smoothing_filter", 1 if model == DGP else 0)
    m.wBD = kw.get("wBD", 100.0)
    m.Omegah2 = kw.get("Omegah2", 0.14)
    m.Omegarh2 = kw.get("Omegarh2", 4.0e-5)
    m.Omegavh2 = kw.get("Omegavh2", 0.36)
    m.scaledependent = kw.get("scaledependent", 0)
    m.sd_nk = kw.get("sd_nk", 0)
    m.sd_kmin = kw.get("sd_kmin", 0.0)
    m.sd_kmax = kw.get("sd_kmax", 0.0)
    if kw.get("nu") is not None:
        m.nu = kw["nu"].h
        m._nu_keep = kw["nu"]
    if model == JBD_GEFF:
        lib().orc_jbd_solve(C.byref(m))
    if model == MBETA and m.mg_active:
        lib().orc_phia_solve(C.byref(m), kw.get("init_redshift", 19.0))
    return m


def make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8, which=2, nu=None):
    """nu: a Neutrinos object (the CDM+baryon spectrum of its CAMB tables)."""
    p = Power()
    p.which_spectrum = which
    p.omega, p.omega_b, p.h, p.ns, p.sigma8 = omega, omega_b, h, ns, sigma8
    p.ntab = 0
    if nu is not None:
        p.nu = nu.h
        p._nu_keep = nu
    lib().orc_power_init(C.byref(p))
    return p


class Neutrinos:
    """CAMB transfer tables and Omega's of the massive-neutrino build
    (orc_nu.c).  Attach to make_mg(nu=...) / make_power(nu=...)."""

    TNU, TCDM, TB, TTOT = 0, 1, 2, 3

    def __init__(self, infofile, omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sum_mnu_ev=0.3, include=1):
        self.h = lib().orc_nu_create(str(infofile).encode(), omega, omega_b, h, ns, sum_mnu_ev, include)
        if not self.h:
            raise OSError("cannot read the transfer tables of %s" % infofile)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_nu_free(self.h)
            self.h = None

    @property
    def omega_nu(self):
        return lib().orc_nu_omega_nu(self.h)

    @property
    def omega_cdm(self):
        return lib().orc_nu_omega_cdm(self.h)

    def transfer(self, which, k, a):
        return lib().orc_nu_transfer(self.h, which, k, a)

    def mu1(self, a, k):
        return lib().orc_nu_mu1(self.h, a, k)

    def mu2(self):
        return lib().orc_nu_mu2(self.h)

    def add_density(self, a, N, box, grid, cdelta):
        lib().orc_nu_add_density(self.h, a, N, box, grid, np.ascontiguousarray(cdelta))


def ic_2lpt(N, Ns, box, seed, pw, fixed=0, inverted=0, sphere=0, rescale=1.0, want_k=False):
    ip = ICParams(N, Ns, box, seed, sphere, fixed, inverted, rescale)
    npart = Ns ** 3
    D1 = np.zeros((npart, 3))
    D2 = np.zeros((npart, 3))
    dk = np.zeros(padded_shape(N)) if want_k else None
    s2 = np.zeros(padded_shape(N)) if want_k else None
    lib().orc_ic_2lpt(C.byref(ip), C.byref(pw), D1, D2, None if dk is None else dk.ctypes.data,
                      None if s2 is None else s2.ctypes.data)
    return (D1, D2, dk, s2) if want_k else (D1, D2)


def ic_2lpt_from_particles(N, Ns, box, pos01, normfac, rescale_rk, want_k=False):
    """ReadParticlesFromFile IC: pos01 [n][3] in [0,1); rescale_rk per integer
    |k|^2 (length >= 3 (N/2)^2 + 1)."""
    ip = ICParams(N, Ns, box, 0, 0, 0, 0, 1.0)
    pos01 = np.ascontiguousarray(pos01, np.float64)
    rescale_rk = np.ascontiguousarray(rescale_rk, np.float64)
    assert len(rescale_rk) >= 3 * (N // 2) ** 2 + 1
    npart = Ns ** 3
    D1 = np.zeros((npart, 3))
    D2 = np.zeros((npart, 3))
    dk = np.zeros(padded_shape(N)) if want_k else None
    s2 = np.zeros(padded_shape(N)) if want_k else None
    lib().orc_ic_2lpt_from_particles(C.byref(ip), pos01, len(pos01), float(normfac), rescale_rk, D1, D2,
                                     None if dk is None else dk.ctypes.data, None if s2 is None else s2.ctypes.data)
    return (D1, D2, dk, s2) if want_k else (D1, D2)


FIELD_D, FIELD_dDdy, FIELD_ddDddy, FIELD_deltaD = 0, 1, 2, 3


def sd_field(cosmo, stored_k, N, Ns, box, A, AFF, fieldtype, order):
    """from_cdisp_store_to_ZA for one LPT order; stored_k is a padded complex
    grid (delta(k) for order 1, -source(k) for order 2)."""
    out = np.zeros((Ns ** 3, 3))
    lib().orc_sd_field(cosmo.h, np.ascontiguousarray(stored_k), N, Ns, box, A, AFF, fieldtype, order, out)
    return out
