"""Python host binding of libmgpicola.so (the GB300 COLA library).

Thin ctypes layer over the C ABI declared in include/mgpicola.h; it mirrors
the reference's run-parameter names and raises on every non-zero status.
There is no CPU fallback: loading fails loudly when the shared library is
missing, and mgp_create fails when no CUDA device is present.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmgpicola.so")

MODEL_LCDM, MODEL_FOFR, MODEL_DGP, MODEL_BRANSDICKE, MODEL_MBETA = 0, 1, 2, 3, 4
FILTER_NONE, FILTER_GAUSSIAN, FILTER_TOPHAT, FILTER_SHARPK = 0, 1, 2, 3

# exported symbols of include/mgpicola.h
EXPORTS = [
    "mgp_params_default", "mgp_read_parameterfile", "mgp_create", "mgp_create_with_hooks", "mgp_cosmo_eval_hooks",
    "mgp_destroy", "mgp_last_error",
    "mgp_displacement_fields", "mgp_get_displacements", "mgp_kick_drift", "mgp_step", "mgp_run", "mgp_pofk",
    "mgp_pofk_total", "mgp_pofk_rsd", "mgp_get_particles", "mgp_set_particles", "mgp_step_host", "mgp_growth", "mgp_Sq",
    "mgp_Sphi", "mgp_power_spectrum", "mgp_cosmo_eval", "mgp_cosmo_coeff", "mgp_copy_grid", "mgp_set_timing", "mgp_kernel_ms", "mgp_mark", "mgp_mark_ms", "mgp_kernel_ms_step", "mgp_set_particle_order", "mgp_set_fft_mode", "mgp_launch_count",
    "mgp_host_register", "mgp_host_unregister", "mgp_host_alloc", "mgp_host_free", "mgp_pofk_noalloc", "mgp_assign_displacement_fields",
    "mgp_growth_scaledependent", "mgp_batch_create", "mgp_batch_run", "mgp_batch_pofk", "mgp_batch_get_particles",
    "mgp_batch_ms", "mgp_batch_graph_nodes", "mgp_batch_graph_kernels", "mgp_batch_set_tuning",
    "mgp_batch_get_tuning", "mgp_batch_set_deposit_tiles", "mgp_batch_get_deposit_tiles", "mgp_batch_autotune", "mgp_output_stats", "mgp_displacement_fields_from_positions",
    "mgp_read_particle_files", "mgp_free_particles", "mgp_closure_create", "mgp_closure_destroy",
    "mgp_closure_get_weights", "mgp_closure_set_weights", "mgp_closure_set_sample", "mgp_closure_get_sample",
    "mgp_closure_forward", "mgp_closure_gradients", "mgp_closure_train_step", "mgp_closure_features",
    "mgp_closure_target", "mgp_closure_target_particles", "mgp_closure_set_particle_sample",
    "mgp_closure_get_particle_sample", "mgp_closure_set_highpass", "mgp_closure_get_highpass",
    "mgp_closure_set_scale_table", "mgp_closure_scale_at", "mgp_closure_reserve", "mgp_closure_store", "mgp_closure_load", "mgp_set_closure",
]

# field types of mgp_assign_displacement_fields (src/proto.h:155-158)
FIELD_D, FIELD_dDdy, FIELD_ddDddy, FIELD_deltaD = 0, 1, 2, 3


class Params(C.Structure):
    """struct mgp_params (include/mgpicola.h); field names are the
    reference's parameter-file keys."""
    _fields_ = [
        ("model", C.c_int), ("smoothing_filter", C.c_int), ("use_w0wa", C.c_int), ("scaledependent", C.c_int),
        ("modified_gravity_active", C.c_int), ("include_screening", C.c_int),
        ("use_lcdm_growth_factors", C.c_int), ("input_pofk_is_for_lcdm", C.c_int),
        ("input_sigma8_is_for_lcdm", C.c_int), ("inverted_initial_condition", C.c_int),
        ("amplitude_fixed_initial_condition", C.c_int),
        ("fofr0", C.c_double), ("nfofr", C.c_double), ("Rsmooth", C.c_double), ("rcH0_DGP", C.c_double),
        ("wBD", C.c_double), ("Omegah2", C.c_double), ("Omegarh2", C.c_double), ("Omegavh2", C.c_double),
        ("range_symm", C.c_double), ("assb_symm", C.c_double), ("beta_symm", C.c_double),
        ("w_0", C.c_double), ("w_a", C.c_double),
        ("pofk_compute_every_step", C.c_int), ("pofk_compute_rsd_pofk", C.c_int), ("pofk_nbins", C.c_int),
        ("pofk_bintype", C.c_int), ("pofk_subtract_shotnoise", C.c_int),
        ("pofk_kmin", C.c_double), ("pofk_kmax", C.c_double),
        ("OutputDir", C.c_char * 500), ("FileBase", C.c_char * 500), ("OutputRedshiftFile", C.c_char * 500),
        ("NumFilesWrittenInParallel", C.c_int),
        ("UseCOLA", C.c_int), ("Buffer", C.c_double), ("Nmesh", C.c_int), ("Nsample", C.c_int),
        ("Box", C.c_double), ("Init_Redshift", C.c_double), ("Seed", C.c_int), ("SphereMode", C.c_int),
        ("WhichSpectrum", C.c_int), ("WhichTransfer", C.c_int),
        ("FileWithInputSpectrum", C.c_char * 500), ("FileWithInputTransfer", C.c_char * 500),
        ("Omega", C.c_double), ("OmegaBaryon", C.c_double), ("HubbleParam", C.c_double), ("Sigma8", C.c_double),
        ("PrimordialIndex", C.c_double),
        ("UnitLength_in_cm", C.c_double), ("UnitMass_in_g", C.c_double), ("UnitVelocity_in_cm_per_s", C.c_double),
        ("InputSpectrum_UnitLength_in_cm", C.c_double),
        ("Noutputs", C.c_int), ("output_redshift", C.c_double * 64), ("output_nsteps", C.c_int * 64),
        ("sd_nk", C.c_int), ("sd_kmin", C.c_double), ("sd_kmax", C.c_double),
        ("ReadParticlesFromFile", C.c_int), ("NumInputParticleFiles", C.c_int), ("RamsesOutputNumber", C.c_int),
        ("TypeInputParticleFiles", C.c_int), ("InputParticleFileDir", C.c_char * 500),
        ("InputParticleFilePrefix", C.c_char * 500),
        ("massive_neutrinos", C.c_int), ("nu_include_massive_neutrinos", C.c_int), ("nu_SumMassNuEV", C.c_double),
        ("nu_FilenameTransferInfofile", C.c_char * 500),
    ]


class BoxParams(C.Structure):
    """struct mgp_box_params: the per-box overrides of a batch."""
    _fields_ = [("Seed", C.c_int), ("inverted_initial_condition", C.c_int),
                ("amplitude_fixed_initial_condition", C.c_int), ("fofr0", C.c_double), ("rcH0_DGP", C.c_double)]


class MGPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mgp error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """Load libmgpicola.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libmgpicola.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.mgp_last_error.restype = C.c_char_p
        L.mgp_params_default.argtypes = [C.POINTER(Params)]
        L.mgp_read_parameterfile.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(Params)]
        L.mgp_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
        L.mgp_destroy.argtypes = [vp]
        L.mgp_displacement_fields.argtypes = [vp]
        L.mgp_get_displacements.argtypes = [vp, C.c_double]
        L.mgp_kick_drift.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.mgp_step.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.mgp_run.argtypes = [vp, C.c_int]
        dp = C.POINTER(C.c_double)
        L.mgp_pofk.argtypes = [vp, C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp]
        L.mgp_pofk_total.argtypes = [vp, C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp]
        L.mgp_pofk_rsd.argtypes = [vp, C.c_double, C.c_int, C.POINTER(C.c_int)] + [dp] * 8
        L.mgp_get_particles.argtypes = [vp, vp, vp, vp, vp, C.c_size_t]
        L.mgp_set_particles.argtypes = [vp, vp, vp, vp, vp, C.c_size_t]
        L.mgp_step_host.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, vp, vp, vp, vp, C.c_size_t]
        for f in ("mgp_growth",):
            getattr(L, f).argtypes = [vp, C.c_int, C.c_double]
            getattr(L, f).restype = C.c_double
        for f in ("mgp_Sq", "mgp_Sphi"):
            getattr(L, f).argtypes = [vp, C.c_double, C.c_double, C.c_double]
            getattr(L, f).restype = C.c_double
        L.mgp_cosmo_eval.argtypes = [C.POINTER(Params), C.c_int, dp, C.c_int, dp]
        L.mgp_cosmo_eval_hooks.argtypes = [C.POINTER(Params), C.POINTER(ModelHooks), C.c_int, dp, C.c_int, dp]
        L.mgp_create_with_hooks.argtypes = [C.POINTER(Params), C.POINTER(ModelHooks), C.c_int, C.POINTER(vp)]
        L.mgp_cosmo_coeff.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, C.c_int, dp]
        L.mgp_growth_scaledependent.argtypes = [C.POINTER(Params), C.c_int, dp, dp, C.c_int, dp]
        L.mgp_assign_displacement_fields.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int)]
        L.mgp_batch_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(BoxParams), C.c_int, C.POINTER(vp)]
        L.mgp_batch_run.argtypes = [vp, C.c_int, C.c_double]
        L.mgp_batch_pofk.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp]
        L.mgp_batch_get_particles.argtypes = [vp, C.c_int, vp, vp, C.c_size_t]
        L.mgp_batch_ms.argtypes = [vp, C.c_int]
        L.mgp_batch_ms.restype = C.c_double
        L.mgp_batch_graph_nodes.argtypes = [vp]
        L.mgp_batch_graph_kernels.argtypes = [vp]
        L.mgp_batch_set_tuning.argtypes = [vp, C.POINTER(C.c_int)]
        L.mgp_batch_get_tuning.argtypes = [vp, C.POINTER(C.c_int)]
        L.mgp_batch_set_deposit_tiles.argtypes = [vp, C.c_int]
        L.mgp_batch_get_deposit_tiles.argtypes = [vp]
        L.mgp_batch_autotune.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.mgp_output_stats.argtypes = [vp, C.POINTER(C.c_int)] + [C.POINTER(C.c_double)] * 3
        L.mgp_displacement_fields_from_positions.argtypes = [vp, C.POINTER(C.c_double), C.c_size_t]
        L.mgp_read_particle_files.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_size_t)]
        L.mgp_free_particles.argtypes = [C.POINTER(C.c_double)]
        fpp = C.POINTER(C.c_float)
        dpp = C.POINTER(C.c_double)
        L.mgp_closure_create.argtypes = [C.c_int, C.c_uint, C.c_int, C.POINTER(vp)]
        L.mgp_closure_destroy.argtypes = [vp]
        L.mgp_closure_get_weights.argtypes = [vp, fpp, fpp, C.POINTER(C.c_float)]
        L.mgp_closure_set_weights.argtypes = [vp, fpp, fpp, C.c_float]
        L.mgp_closure_set_sample.argtypes = [vp, fpp, fpp]
        L.mgp_closure_get_sample.argtypes = [vp, fpp, fpp]
        L.mgp_closure_forward.argtypes = [vp, fpp]
        L.mgp_closure_gradients.argtypes = [vp, C.POINTER(C.c_double), fpp, fpp]
        L.mgp_closure_train_step.argtypes = [vp, C.c_float, C.POINTER(C.c_double)]
        L.mgp_closure_features.argtypes = [vp, vp, C.c_double]
        L.mgp_closure_target.argtypes = [vp, vp, vp, C.POINTER(C.c_double)]
        L.mgp_closure_target_particles.argtypes = [vp, vp, vp, C.c_int, C.POINTER(C.c_double)]
        L.mgp_closure_set_particle_sample.argtypes = [vp, C.c_longlong, fpp, fpp]
        L.mgp_closure_get_particle_sample.argtypes = [vp, C.POINTER(C.c_longlong), fpp, fpp]
        L.mgp_closure_reserve.argtypes = [vp, C.c_int, C.c_longlong]
        L.mgp_closure_set_highpass.argtypes = [vp, C.c_double]
        L.mgp_closure_get_highpass.argtypes = [vp]
        L.mgp_closure_get_highpass.restype = C.c_double
        L.mgp_closure_set_scale_table.argtypes = [vp, C.c_int, dpp, dpp]
        L.mgp_closure_scale_at.argtypes = [vp, C.c_double]
        L.mgp_closure_scale_at.restype = C.c_double
        L.mgp_closure_store.argtypes = [vp, C.c_int]
        L.mgp_closure_load.argtypes = [vp, C.c_int]
        L.mgp_set_closure.argtypes = [vp, vp]
        L.mgp_power_spectrum.argtypes = [vp, C.c_double]
        L.mgp_power_spectrum.restype = C.c_double
        L.mgp_copy_grid.argtypes = [vp, C.c_int, fp, C.c_size_t]
        L.mgp_set_timing.argtypes = [vp, C.c_int]
        L.mgp_kernel_ms.argtypes = [vp, C.c_char_p]
        L.mgp_kernel_ms.restype = C.c_double
        L.mgp_kernel_ms_step.argtypes = [vp, C.c_char_p, C.c_int]
        L.mgp_kernel_ms_step.restype = C.c_double
        L.mgp_mark.argtypes = [vp, C.c_int]
        L.mgp_set_particle_order.argtypes = [vp, C.c_int]
        L.mgp_set_fft_mode.argtypes = [vp, C.c_int]
        L.mgp_host_alloc.argtypes = [C.POINTER(vp), C.c_size_t]
        L.mgp_host_free.argtypes = [vp]
        L.mgp_mark_ms.argtypes = [vp, C.c_int, C.c_int]
        L.mgp_mark_ms.restype = C.c_double
        L.mgp_launch_count.argtypes = [vp]
        L.mgp_launch_count.restype = C.c_longlong
        L.mgp_host_register.argtypes = [vp, C.c_size_t]
        L.mgp_host_unregister.argtypes = [vp]
        L.mgp_pofk_noalloc.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                       C.c_double, C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp, vp]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise MGPError(rc, lib().mgp_last_error().decode(errors="replace"))


def default_params(**kw):
    p = Params()
    _check(lib().mgp_params_default(C.byref(p)))
    for k, v in kw.items():
        if isinstance(getattr(p, k), bytes):
            v = v.encode() if isinstance(v, str) else v
        setattr(p, k, v)
    return p


def read_parameterfile(fname, model=MODEL_LCDM, pofk_keys=True, read_outputs=True, use_w0wa=False,
                       read_ic_from_file=False, massive_neutrinos=False):
    """read_parameterfile + read_outputs of the reference (read_ic_from_file:
    the READICFROMFILE build's six keys are required; massive_neutrinos: the
    MASSIVE_NEUTRINOS build, which is also scale dependent, with its three
    nu_* keys)."""
    p = Params()
    p.use_w0wa = 1 if use_w0wa else 0
    p.ReadParticlesFromFile = 1 if read_ic_from_file else 0
    if massive_neutrinos:
        p.massive_neutrinos = p.scaledependent = 1
    _check(lib().mgp_read_parameterfile(fname.encode(), model, 1 if pofk_keys else 0, 1 if read_outputs else 0,
                                        C.byref(p)))
    return p


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def read_particle_files(params):
    """Positions in [0,1) of the box ([n][3]) from the IC particle files of
    params (TypeInputParticleFiles 1 RAMSES, 2 ASCII, 3 GADGET-1)."""
    ptr = C.POINTER(C.c_double)()
    n = C.c_size_t(0)
    _check(lib().mgp_read_particle_files(C.byref(params), C.byref(ptr), C.byref(n)))
    try:
        return np.ctypeslib.as_array(ptr, shape=(n.value, 3)).copy() if n.value else np.zeros((0, 3))
    finally:
        lib().mgp_free_particles(ptr)


def cosmo_eval(params, which, x):
    """Host-only growth factors (which 0-6), P(k) (which 7), mg_pofk_ratio(k,
    a = 1) (which 8) or the sigma8 enhancement at a (which 9)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    _check(lib().mgp_cosmo_eval(C.byref(params), which, _dptr(x), x.size, _dptr(out)))
    return out


_F1 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)
_F2 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_double, C.c_void_p)
_F5 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p)


class ModelHooks(C.Structure):
    """struct mgp_model_hooks: the user_defined_functions.h model functions
    as callbacks (src/user_defined_functions.h:413-904)."""
    _fields_ = [("user", C.c_void_p), ("hubble", _F1), ("dhubbleda", _F1), ("GeffoverG", _F2), ("beta_of_a", _F1),
                ("mass2_of_a", _F1), ("dmass2_of_ada", _F1), ("coupling_function", _F1), ("phi_of_a", _F1),
                ("screening_factor_potential", _F2), ("screening_factor_density", _F2), ("Factor_2LPT", _F1),
                ("second_order_kernel", _F5)]
    _SIGS = {"GeffoverG": _F2, "screening_factor_potential": _F2, "screening_factor_density": _F2,
             "second_order_kernel": _F5}

    @classmethod
    def from_functions(cls, **fns):
        """Hooks from Python functions of the reference's arguments (without
        the user pointer); the callback objects are kept on the table."""
        h = cls()
        h._keep = []
        for name, fn in fns.items():
            sig = cls._SIGS.get(name, _F1)
            cb = sig((lambda f: (lambda *a: float(f(*a[:-1]))))(fn))
            h._keep.append(cb)
            setattr(h, name, cb)
        return h


def cosmo_eval_hooks(params, hooks, which, x):
    """cosmo_eval with user model hooks; which 10-15 give hubble,
    GeffoverG(a, k = 0.1), coupling_function, mass2_of_a, phi_crit and
    Factor_2LPT at a = x as the library evaluates them."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    _check(lib().mgp_cosmo_eval_hooks(C.byref(params), C.byref(hooks) if hooks is not None else None, which, _dptr(x),
                                      x.size, _dptr(out)))
    return out


def growth_scaledependent(params, which, k, a):
    """growth_*_scaledependent(k, a) of a parameter set (scaledependent = 1)."""
    k = np.ascontiguousarray(k, dtype=np.float64)
    a = np.ascontiguousarray(np.broadcast_to(a, k.shape), dtype=np.float64)
    out = np.zeros_like(k)
    _check(lib().mgp_growth_scaledependent(C.byref(params), which, _dptr(k), _dptr(a), k.size, _dptr(out)))
    return out


def cosmo_coeff(params, kind, ai, af, aref):
    """Kick/drift coefficients on the host: COLA Sq (kind 0) / Sphi (kind 1)
    at aref, or the non-COLA SqStd (kind 2) / SphiStd (kind 3)."""
    ai, af, aref = (np.ascontiguousarray(v, dtype=np.float64) for v in (ai, af, aref))
    out = np.zeros_like(ai)
    _check(lib().mgp_cosmo_coeff(C.byref(params), kind, _dptr(ai), _dptr(af), _dptr(aref), ai.size, _dptr(out)))
    return out


def pofk_noalloc(d_deltak, Nmesh, Nsample, Box, nbins, bintype, subtract_shotnoise, kmin, kmax, stream=None):
    """Allocation-free P(k) of a caller-owned device delta(k) grid (see
    mgp_pofk_noalloc in include/mgpicola.h)."""
    cap = max(nbins, Nmesh, 1)
    k, pk, km, n = (np.zeros(cap) for _ in range(4))
    nb = C.c_int(0)
    _check(lib().mgp_pofk_noalloc(d_deltak, Nmesh, Nsample, Box, nbins, bintype, subtract_shotnoise, kmin, kmax,
                                  cap, C.byref(nb), _dptr(k), _dptr(pk), _dptr(km), _dptr(n), stream))
    m = nb.value
    return k[:m], pk[:m], km[:m], n[:m]


def host_array(shape):
    """A float32 numpy array in page-locked host memory (mgp_host_alloc);
    release it with host_free."""
    n = int(np.prod(shape))
    ptr = C.c_void_p()
    _check(lib().mgp_host_alloc(C.byref(ptr), max(4 * n, 4)))
    buf = (C.c_float * max(n, 1)).from_address(ptr.value)
    a = np.ctypeslib.as_array(buf)[:n].reshape(shape)
    _HOST[id(a)] = ptr.value
    return a


_HOST = {}


def host_free(a):
    ptr = _HOST.pop(id(a), None)
    if ptr:
        _check(lib().mgp_host_free(ptr))


def pin(arr):
    """Page-lock a numpy array for fast host<->device copies."""
    _check(lib().mgp_host_register(arr.ctypes.data, arr.nbytes))


def unpin(arr):
    _check(lib().mgp_host_unregister(arr.ctypes.data))


class Context:
    """One simulation box on one GPU (mgp_ctx)."""

    def __init__(self, params, device=0, hooks=None):
        self.params = params
        self.hooks = hooks  # the callbacks must outlive the context
        self.h = C.c_void_p()
        if hooks is None:
            _check(lib().mgp_create(C.byref(params), device, C.byref(self.h)))
        else:
            _check(lib().mgp_create_with_hooks(C.byref(params), C.byref(hooks), device, C.byref(self.h)))
        self.N = params.Nmesh
        self.Ns = params.Nsample
        self.np = params.Nsample ** 3

    def close(self):
        if self.h:
            lib().mgp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # reference entry points
    def displacement_fields(self):
        _check(lib().mgp_displacement_fields(self.h))

    def displacement_fields_from_positions(self, pos):
        """2LPT IC from the density of the given particles (Mpc/h, [n][3])."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        _check(lib().mgp_displacement_fields_from_positions(self.h, _dptr(pos), len(pos)))

    def get_displacements(self, A):
        _check(lib().mgp_get_displacements(self.h, A))

    def kick_drift(self, AI, AF, A, AFF, drift=True):
        _check(lib().mgp_kick_drift(self.h, AI, AF, A, AFF, 1 if drift else 0))

    def assign_fields(self, A, AFF, *types):
        t = (C.c_int * len(types))(*types)
        _check(lib().mgp_assign_displacement_fields(self.h, A, AFF, len(types), t))

    def step(self, A, AI, AF, AFF):
        _check(lib().mgp_step(self.h, A, AI, AF, AFF))

    def run(self, gadget=True):
        _check(lib().mgp_run(self.h, 1 if gadget else 0))

    def output_stats(self):
        """(snapshots, writer ms waiting for the GPU, writer ms on files, ms the
        calling thread was held) of mgp_run."""
        n, w, f, b = C.c_int(0), C.c_double(0), C.c_double(0), C.c_double(0)
        _check(lib().mgp_output_stats(self.h, C.byref(n), C.byref(w), C.byref(f), C.byref(b)))
        return n.value, w.value, f.value, b.value

    def pofk(self, total=False):
        """P(k) of the last density: k, P, mean |k|, mode count.  total=True
        gives the total matter spectrum of a run with massive neutrinos."""
        cap = max(self.params.pofk_nbins, self.N, 1)
        k, pk, km, n = (np.zeros(cap) for _ in range(4))
        nb = C.c_int(0)
        fn = lib().mgp_pofk_total if total else lib().mgp_pofk
        _check(fn(self.h, cap, C.byref(nb), _dptr(k), _dptr(pk), _dptr(km), _dptr(n)))
        m = nb.value
        return k[:m], pk[:m], km[:m], n[:m]

    def pofk_rsd(self, A):
        """RSD multipoles (compute_RSD_powerspectrum): k, P0, P2, P4, sigma0,
        sigma2, sigma4, n."""
        cap = max(self.params.pofk_nbins, self.N, 1)
        arrs = [np.zeros(cap) for _ in range(8)]
        nb = C.c_int(0)
        _check(lib().mgp_pofk_rsd(self.h, A, cap, C.byref(nb), *[_dptr(a) for a in arrs]))
        m = nb.value
        return tuple(a[:m] for a in arrs)

    def get_particles(self):
        pos = np.zeros((self.np, 3), np.float32)
        vel = np.zeros((self.np, 3), np.float32)
        d1 = np.zeros((self.np, 3), np.float32)
        d2 = np.zeros((self.np, 3), np.float32)
        _check(lib().mgp_get_particles(self.h, pos.ctypes.data, vel.ctypes.data, d1.ctypes.data, d2.ctypes.data,
                                       self.np))
        return pos, vel, d1, d2

    def set_particles(self, pos=None, vel=None, d1=None, d2=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (pos, vel, d1, d2)]
        ptrs = [None if a is None else a.ctypes.data for a in arrs]
        _check(lib().mgp_set_particles(self.h, *ptrs, self.np))

    def step_host(self, A, AI, AF, AFF, pos, vel, d1, d2):
        """Host-buffer step (mgp_step_host).  d1/d2 None: the LPT
        displacements on the device are kept (they are fixed after the IC)."""
        ptr = lambda a: None if a is None else a.ctypes.data
        _check(lib().mgp_step_host(self.h, A, AI, AF, AFF, ptr(pos), ptr(vel), ptr(d1), ptr(d2), self.np))

    def grid(self, which, planes=None):
        """Copy of grid `which` (its first `planes` x planes when given)."""
        nx = self.N if planes is None else int(planes)
        n = nx * self.N * 2 * (self.N // 2 + 1)
        out = np.zeros(n, np.float32)
        _check(lib().mgp_copy_grid(self.h, which, out, n))
        return out.reshape(nx, self.N, 2 * (self.N // 2 + 1))

    def growth(self, which, a):
        return lib().mgp_growth(self.h, which, a)

    def Sq(self, ai, af, aref):
        return lib().mgp_Sq(self.h, ai, af, aref)

    def Sphi(self, ai, af, aref):
        return lib().mgp_Sphi(self.h, ai, af, aref)

    def power(self, k):
        return lib().mgp_power_spectrum(self.h, k)

    def set_timing(self, on=True, history=0):
        """Stage timing of the last call; with history = n > 1 the stage
        events of the last n steps are kept (kernel_ms_step)."""
        _check(lib().mgp_set_timing(self.h, history if (on and history > 1) else (1 if on else 0)))

    def kernel_ms(self, name):
        return lib().mgp_kernel_ms(self.h, name.encode())

    def kernel_ms_step(self, name, step):
        """Stage milliseconds of step `step` from the timing history
        (set_timing(n) with n > 1)."""
        return lib().mgp_kernel_ms_step(self.h, name.encode(), step)

    def set_particle_order(self, tiles):
        """Cell-tile particle order (mgp_set_particle_order): 2 the default
        for single boxes (tile deposit, kick per tile with the arrays
        rewritten in tile order every step), 1 the tile deposit with the
        arrays in lattice order, 0 the deposit and kick in lattice order."""
        _check(lib().mgp_set_particle_order(self.h, int(tiles)))

    def set_fft_mode(self, mode):
        """Transforms of a 1024^3 single box (mgp_set_fft_mode): 1 the
        default, own strided y/x passes with the force pass fused in; 0
        cuFFT's 3D plans and the separate force pass."""
        _check(lib().mgp_set_fft_mode(self.h, int(mode)))

    def mark(self, slot):
        """Record event `slot` (0..3) on the context's stream."""
        _check(lib().mgp_mark(self.h, slot))

    def mark_ms(self, a, b):
        """Device milliseconds from mark a to mark b (waits for b)."""
        return lib().mgp_mark_ms(self.h, a, b)

    def launches(self):
        return lib().mgp_launch_count(self.h)


class Batch:
    """A batch of independent boxes run in lock step (mgp_batch_*)."""

    def __init__(self, params, boxes, device=0):
        self.p = params
        arr = (BoxParams * len(boxes))()
        for i, b in enumerate(boxes):
            arr[i] = BoxParams(int(b.get("Seed", params.Seed)), int(b.get("inverted", 0)), int(b.get("fixed", 0)),
                               float(b.get("fofr0", 0.0)), float(b.get("rcH0", 0.0)))
        self.nbox = len(boxes)
        self.h = C.c_void_p()
        _check(lib().mgp_batch_create(C.byref(params), self.nbox, arr, device, C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None):
            lib().mgp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def run(self, nsteps, z_final=0.0):
        _check(lib().mgp_batch_run(self.h, nsteps, z_final))

    def pofk(self, box, step):
        cap = max(self.p.pofk_nbins, self.p.Nmesh) if self.p.pofk_nbins > 0 else self.p.Nmesh
        k, pk, km, n = (np.zeros(cap) for _ in range(4))
        nb = C.c_int(0)
        _check(lib().mgp_batch_pofk(self.h, box, step, cap, C.byref(nb), _dptr(k), _dptr(pk), _dptr(km), _dptr(n)))
        m = nb.value
        return k[:m], pk[:m], km[:m], n[:m]

    def particles(self, box):
        n = self.p.Nsample ** 3
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        _check(lib().mgp_batch_get_particles(self.h, box, pos.ctypes.data, vel.ctypes.data, n))
        return pos, vel

    def ms(self, what=0):
        return lib().mgp_batch_ms(self.h, what)

    def graph_nodes(self):
        return lib().mgp_batch_graph_nodes(self.h)

    def graph_kernels(self):
        return lib().mgp_batch_graph_kernels(self.h)

    def tuning(self):
        t = (C.c_int * 4)()
        _check(lib().mgp_batch_get_tuning(self.h, t))
        return list(t)

    def set_tuning(self, tune):
        t = (C.c_int * 4)(*tune)
        _check(lib().mgp_batch_set_tuning(self.h, t))

    def deposit_tiles(self):
        """Deposit form: 0 lattice order, 8 or 16 the tile side in cells."""
        r = lib().mgp_batch_get_deposit_tiles(self.h)
        _check(min(r, 0))
        return r

    def set_deposit_tiles(self, side):
        _check(lib().mgp_batch_set_deposit_tiles(self.h, side))

    def autotune(self, nsteps, z_final=0.0):
        """Pick the deposit form and the launch budgets by timing runs;
        returns the best graph ms."""
        ms = C.c_double(0)
        _check(lib().mgp_batch_autotune(self.h, nsteps, z_final, C.byref(ms)))
        return ms.value


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


class Closure:
    """Learned force closure (mgp_closure_*): a 4-layer 3x3x3 CNN on an
    Nmesh^3 mesh predicting the finer-mesh force residual."""

    NW = 4 * 27 * 16 * 16
    NB = 4 * 16

    def __init__(self, Nmesh, seed=1, device=0):
        self.N = Nmesh
        self.V = Nmesh ** 3
        self.h = C.c_void_p()
        _check(lib().mgp_closure_create(Nmesh, seed, device, C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None):
            lib().mgp_closure_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def weights(self):
        w = np.zeros(self.NW, np.float32)
        b = np.zeros(self.NB, np.float32)
        s = C.c_float(0)
        _check(lib().mgp_closure_get_weights(self.h, _fptr(w), _fptr(b), C.byref(s)))
        return w.reshape(4, 27, 16, 16), b.reshape(4, 16), s.value

    def set_weights(self, w=None, b=None, scale=0.0):
        w = None if w is None else np.ascontiguousarray(w, np.float32).reshape(-1)
        b = None if b is None else np.ascontiguousarray(b, np.float32).reshape(-1)
        _check(lib().mgp_closure_set_weights(self.h, _fptr(w), _fptr(b), float(scale)))

    def set_sample(self, x=None, t=None):
        x = None if x is None else np.ascontiguousarray(x, np.float32).reshape(-1)
        t = None if t is None else np.ascontiguousarray(t, np.float32).reshape(-1)
        _check(lib().mgp_closure_set_sample(self.h, _fptr(x), _fptr(t)))

    def sample(self):
        x = np.zeros((self.V, 3), np.float32)
        t = np.zeros((self.V, 3), np.float32)
        _check(lib().mgp_closure_get_sample(self.h, _fptr(x), _fptr(t)))
        return x, t

    def forward(self):
        out = np.zeros((self.V, 3), np.float32)
        _check(lib().mgp_closure_forward(self.h, _fptr(out)))
        return out

    def gradients(self):
        gw = np.zeros(self.NW, np.float32)
        gb = np.zeros(self.NB, np.float32)
        loss = C.c_double(0)
        _check(lib().mgp_closure_gradients(self.h, C.byref(loss), _fptr(gw), _fptr(gb)))
        return loss.value, gw.reshape(4, 27, 16, 16), gb.reshape(4, 16)

    def train_step(self, lr):
        loss = C.c_double(0)
        _check(lib().mgp_closure_train_step(self.h, float(lr), C.byref(loss)))
        return loss.value

    def features(self, ctx, A):
        _check(lib().mgp_closure_features(self.h, ctx.h, float(A)))

    def target(self, fine, coarse):
        rms = C.c_double(0)
        _check(lib().mgp_closure_target(self.h, fine.h, coarse.h, C.byref(rms)))
        return rms.value

    def target_particles(self, fine, coarse, band=True):
        rms = C.c_double(0)
        _check(lib().mgp_closure_target_particles(self.h, fine.h, coarse.h, 1 if band else 0, C.byref(rms)))
        return rms.value

    def set_particle_sample(self, cells, t):
        cells = np.ascontiguousarray(cells, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 3)
        _check(lib().mgp_closure_set_particle_sample(self.h, len(cells), _fptr(cells), _fptr(t)))

    def particle_sample(self):
        n = C.c_longlong(0)
        _check(lib().mgp_closure_get_particle_sample(self.h, C.byref(n), None, None))
        cells = np.zeros((n.value, 3), np.float32)
        t = np.zeros((n.value, 3), np.float32)
        _check(lib().mgp_closure_get_particle_sample(self.h, C.byref(n), _fptr(cells), _fptr(t)))
        return cells, t

    def set_highpass(self, lambda_cells):
        _check(lib().mgp_closure_set_highpass(self.h, float(lambda_cells)))

    def highpass(self):
        return lib().mgp_closure_get_highpass(self.h)

    def set_scale_table(self, a, s):
        a = np.ascontiguousarray(a, np.float64)
        s = np.ascontiguousarray(s, np.float64)
        _check(lib().mgp_closure_set_scale_table(self.h, len(a), _dptr(a), _dptr(s)))

    def scale_at(self, A):
        return lib().mgp_closure_scale_at(self.h, float(A))

    def reserve(self, n, np_particles=0):
        _check(lib().mgp_closure_reserve(self.h, n, np_particles))

    def store(self, slot):
        _check(lib().mgp_closure_store(self.h, slot))

    def load(self, slot):
        _check(lib().mgp_closure_load(self.h, slot))

    def attach(self, ctx):
        _check(lib().mgp_set_closure(ctx.h, self.h))

    @staticmethod
    def detach(ctx):
        _check(lib().mgp_set_closure(ctx.h, None))
