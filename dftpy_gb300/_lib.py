"""ctypes binding of ``libgbofdft.so`` (the C ABI declared in include/gbofdft.h).

The product path has no CPU fallback: if the library is missing or no CUDA
device is present, every call raises ``GbofdftError``.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libgbofdft.so")

F32, F64 = 0, 1
CALC_E, CALC_V = 1, 2
KER_NONE, KER_HARTREE, KER_G2, KER_ARRAY = 0, 1, 2, 3
NE = 8
E_TF, E_VW, E_NL, E_XC, E_HARTREE, E_PSEUDO, E_EXTRA, E_TOTAL = range(8)

ERRORS = {1: ValueError, 2: RuntimeError, 3: NotImplementedError, 4: MemoryError, 5: FloatingPointError,
          6: RuntimeError}


class GbofdftError(RuntimeError):
    pass


class Lwt(ctypes.Structure):
    """Mirror of ``gbofdft_lwt``."""
    _fields_ = [("interp", ctypes.c_int), ("kdd", ctypes.c_int), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("ratio", ctypes.c_double), ("ldw", ctypes.c_double),
                ("etamax", ctypes.c_double), ("neta", ctypes.c_int), ("ktab_c", ctypes.c_void_p),
                ("ktab_end", ctypes.c_double), ("dtab_c", ctypes.c_void_p), ("dtab_end", ctypes.c_double),
                ("kfmin_opt", ctypes.c_double), ("kfmax_opt", ctypes.c_double),
                ("kfmin_state", ctypes.c_double), ("kfmax_state", ctypes.c_double),
                ("work", ctypes.c_void_p), ("work_bytes", ctypes.c_int64), ("nknots", ctypes.c_int)]


class Wgc(ctypes.Structure):
    """Mirror of ``gbofdft_wgc``."""
    _fields_ = [("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("rho0", ctypes.c_double), ("order", ctypes.c_int), ("kernels", ctypes.c_void_p),
                ("work", ctypes.c_void_p), ("work_bytes", ctypes.c_int64)]


class Functional(ctypes.Structure):
    """Mirror of ``gbofdft_functional``."""
    _fields_ = [
        ("tf", ctypes.c_int), ("tf_x", ctypes.c_double),
        ("vw", ctypes.c_int), ("vw_y", ctypes.c_double),
        ("wt", ctypes.c_int), ("wt_alpha", ctypes.c_double), ("wt_beta", ctypes.c_double),
        ("wt_kernel", ctypes.c_void_p),
        ("xc", ctypes.c_int), ("hartree", ctypes.c_int),
        ("vloc", ctypes.c_void_p), ("e_ion", ctypes.c_double), ("lwt", ctypes.POINTER(Lwt)),
        ("wgc", ctypes.POINTER(Wgc)),
    ]


class VTable(ctypes.Structure):
    """Mirror of ``gbofdft_vtable``."""
    _fields_ = [("x", ctypes.c_void_p), ("c", ctypes.c_void_p), ("m", ctypes.c_int),
                ("q4", ctypes.c_double * 5), ("dp", ctypes.c_double), ("gmin", ctypes.c_double),
                ("gmax", ctypes.c_double)]


class TnOptions(ctypes.Structure):
    """Mirror of ``gbofdft_tn_options``."""
    _fields_ = [("econv", ctypes.c_double), ("maxfun", ctypes.c_int), ("maxiter", ctypes.c_int),
                ("maxls", ctypes.c_int), ("c1", ctypes.c_double), ("c2", ctypes.c_double),
                ("xtol", ctypes.c_double), ("ncheck", ctypes.c_int), ("eps", ctypes.c_double),
                ("pred_stop", ctypes.c_double), ("eres", ctypes.c_double), ("cg_rtol", ctypes.c_double),
                ("pred_next", ctypes.c_int), ("precond", ctypes.c_int), ("time_evals", ctypes.c_int),
                ("delta", ctypes.c_void_p), ("delta_rtol", ctypes.c_double), ("res0_max", ctypes.c_double)]


class TnResult(ctypes.Structure):
    """Mirror of ``gbofdft_tn_result``."""
    _fields_ = [("energy", ctypes.c_double), ("mu", ctypes.c_double), ("converged", ctypes.c_int),
                ("n_iter", ctypes.c_int), ("n_eval_ev", ctypes.c_int), ("n_eval_v", ctypes.c_int),
                ("energies", ctypes.c_double * 8), ("history", ctypes.POINTER(ctypes.c_double)),
                ("history_cap", ctypes.c_int), ("n_history", ctypes.c_int), ("n_sync", ctypes.c_int),
                ("t_sync", ctypes.c_double), ("t_total", ctypes.c_double), ("n_eval_hess", ctypes.c_int),
                ("t_eval_timed", ctypes.c_double), ("n_eval_timed", ctypes.c_int), ("n_eval_delta", ctypes.c_int)]


_lib = None

# (name, restype, argtypes) of every exported entry point
_P = ctypes.c_void_p
_SIGS = [
    ("gbofdft_version", ctypes.c_int, []),
    ("gbofdft_launch_count", ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_last_error", ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    ("gbofdft_plan_create", ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                           ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    ("gbofdft_plan_destroy", ctypes.c_int, [_P]),
    ("gbofdft_plan_sizes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_fft_r2c", ctypes.c_int, [_P, _P, _P, _P]),
    ("gbofdft_fft_c2r", ctypes.c_int, [_P, _P, _P, _P]),
    ("gbofdft_convolve", ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P, ctypes.c_double, _P]),
    ("gbofdft_convolve_noalloc", ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                                ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P,
                                                ctypes.c_double, _P]),
    ("gbofdft_eval", ctypes.c_int, [_P, _P, ctypes.POINTER(Functional), _P, _P, ctypes.c_int, _P]),
    ("gbofdft_delta_create", ctypes.c_int, [_P, _P, ctypes.POINTER(_P)]),
    ("gbofdft_delta_destroy", ctypes.c_int, [_P]),
    ("gbofdft_eval_delta", ctypes.c_int, [_P, _P, ctypes.POINTER(Functional), ctypes.POINTER(Functional), _P, _P,
                                          ctypes.c_int, ctypes.c_int, _P]),
    ("gbofdft_wt_kernel", ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, _P, _P]),
    ("gbofdft_lwt_workspace_bytes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_wgc_workspace_bytes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_nn_conv3d", ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, _P]),
    ("gbofdft_nn_conv3d_wgrad", ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, _P, _P, _P]),
    ("gbofdft_nn_pointwise", ctypes.c_int, [ctypes.c_int, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _P]),
    ("gbofdft_nn_sqerr", ctypes.c_int, [_P, _P, ctypes.c_int64, _P, _P, _P, _P]),
    ("gbofdft_nn_sqerr_work_bytes", ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_nn_adam", ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, _P]),
    ("gbofdft_nn_to_bf16", ctypes.c_int, [_P, _P, ctypes.c_int64, _P]),
    ("gbofdft_nn_conv3d_tc_supported", ctypes.c_int, [ctypes.c_int] * 5),
    ("gbofdft_nn_conv3d_tc_pack", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, _P]),
    ("gbofdft_nn_conv3d_tc", ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, _P, _P]),
    ("gbofdft_plan_schedules", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("gbofdft_plan_set_schedule", ctypes.c_int, [_P, ctypes.c_int]),
    ("gbofdft_plan_get_schedule", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("gbofdft_wgc_kernels", ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_double, _P, _P]),
    ("gbofdft_mgp_table", ctypes.c_int, [_P, _P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, _P, _P]),
    ("gbofdft_setup_workspace_bytes", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_vloc", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(VTable), ctypes.c_int, _P, _P, ctypes.c_int,
                                    ctypes.c_int, _P, _P, ctypes.c_int64, _P, _P, _P]),
    ("gbofdft_ewald", ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_double, ctypes.c_double, _P,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int64, _P, _P]),
    ("gbofdft_density_normalize", ctypes.c_int, [_P, _P, ctypes.c_double, ctypes.c_double, _P, _P]),
    ("gbofdft_density_guess", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(VTable), ctypes.c_int, _P, _P,
                                             ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int64, _P, _P,
                                             ctypes.c_double, ctypes.c_double, _P]),
    ("gbofdft_forces_workspace_bytes", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_pp_forces", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(VTable), ctypes.c_int, _P, _P,
                                         ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int64, _P, _P]),
    ("gbofdft_ewald_forces", ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_double, ctypes.c_double, _P,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int64, _P,
                                            _P]),
    ("gbofdft_stress_workspace_bytes", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_stress_functional", ctypes.c_int, [_P, _P, ctypes.POINTER(Functional), ctypes.POINTER(ctypes.c_double),
                                                 _P, ctypes.c_int64, _P, _P]),
    ("gbofdft_pp_stress", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(VTable), ctypes.c_int, _P, _P,
                                         ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P, ctypes.c_int64, _P,
                                         _P]),
    ("gbofdft_ewald_stress", ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_double, ctypes.c_double, _P,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P,
                                            ctypes.c_int64, _P, _P]),
    ("gbofdft_tn_options_default", ctypes.c_int, [ctypes.POINTER(TnOptions)]),
    ("gbofdft_tn_workspace_bytes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_tn_hess_workspace_bytes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    ("gbofdft_optimize_tn_split", ctypes.c_int, [_P, ctypes.POINTER(Functional), _P, ctypes.POINTER(Functional), _P,
                                                 ctypes.POINTER(TnOptions), _P, ctypes.c_int64, _P, ctypes.c_int64,
                                                 ctypes.POINTER(TnResult), _P]),
    ("gbofdft_optimize_tn", ctypes.c_int, [_P, ctypes.POINTER(Functional), _P, ctypes.POINTER(TnOptions), _P,
                                           ctypes.c_int64, ctypes.POINTER(TnResult), _P]),
    ("gbofdft_dcsrch", ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.c_int64,
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int]),
]

EXPORTED = [s[0] for s in _SIGS]


def load(path=None):
    """Load the library and bind the signatures (no GPU needed to load).
    ``GBOFDFT_LIBRARY`` names another build of the library to load instead."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("GBOFDFT_LIBRARY") or LIBPATH
    if not os.path.exists(path):
        raise GbofdftError("%s is missing: build it with `python -m dftpy_gb300.build`" % path)
    L = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load().gbofdft_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    if rc != 0:
        msg = last_error()
        exc = ERRORS.get(rc, GbofdftError)
        raise exc("gbofdft%s: %s (status %d)" % ((" " + what) if what else "", msg, rc))


def check_alloc(call, what=""):
    """``check(call())`` for calls whose only side effect before a failed
    allocation can be repeated (creating a plan or delta state, building a
    kernel table).  The library allocates with ``cudaMalloc`` beside
    PyTorch's caching allocator, which keeps freed blocks reserved: on
    ``GBOFDFT_ERR_ALLOC`` the cache (and unreachable Python objects holding
    device memory) is released and the call made once more."""
    rc = call()
    if rc == 4:
        import gc
        import torch
        gc.collect()
        if torch.cuda.is_available():
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
        rc = call()
    check(rc, what)


def require_cuda():
    import torch
    if not torch.cuda.is_available():
        raise GbofdftError("dftpy_gb300 needs a CUDA device (GB300); none is visible")


def stream_ptr(stream=None):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    """Device pointer of a CUDA tensor; the C ABI takes C-contiguous buffers only."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("gbofdft: expected a CUDA tensor, got one on %s" % t.device)
    if not t.is_contiguous():
        raise ValueError("gbofdft: buffers must be C-contiguous (got strides %s)" % (tuple(t.stride()),))
    return ctypes.c_void_p(t.data_ptr())


def launch_count():
    n = ctypes.c_int64()
    check(load().gbofdft_launch_count(ctypes.byref(n)))
    return int(n.value)


def aligned_ptr(t, align=256):
    """First ``align``-byte aligned address inside a CUDA tensor's storage."""
    p = t.data_ptr()
    return ctypes.c_void_p((p + align - 1) // align * align)


def setup_workspace_bytes(plan, nat):
    n = ctypes.c_int64()
    check(load().gbofdft_setup_workspace_bytes(plan.handle, int(nat), ctypes.byref(n)), "setup_workspace_bytes")
    return int(n.value)


def stress_workspace_bytes(plan, nat):
    n = ctypes.c_int64()
    check(load().gbofdft_stress_workspace_bytes(plan.handle, int(nat), ctypes.byref(n)), "stress_workspace_bytes")
    return int(n.value)


def forces_workspace_bytes(plan, nat):
    n = ctypes.c_int64()
    check(load().gbofdft_forces_workspace_bytes(plan.handle, int(nat), ctypes.byref(n)), "forces_workspace_bytes")
    return int(n.value)


class Plan:
    """A grid plan (``gbofdft_plan``): geometry, FFT schedule, workspaces."""

    def __init__(self, nr, lattice, precision=F64, full=False):
        require_cuda()
        L = load()
        nr = [int(x) for x in nr]
        lat = [float(x) for x in list(_flat(lattice))]
        h = ctypes.c_void_p()
        check_alloc(lambda: L.gbofdft_plan_create((ctypes.c_int * 3)(*nr), (ctypes.c_double * 9)(*lat),
                                                  int(precision), 1 if full else 0, ctypes.byref(h)), "plan_create")
        self.handle = h
        self.nr = tuple(nr)
        self.precision = precision
        self.full = bool(full)
        s = (ctypes.c_int64 * 4)()
        check(L.gbofdft_plan_sizes(h, s), "plan_sizes")
        self.N, self.NG, self.n2h, self.workspace_bytes = (int(x) for x in s)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and _lib is not None:
            try:
                _lib.gbofdft_plan_destroy(h)
            except Exception:
                pass
            self.handle = None


class Delta:
    """Delta-evaluation state (``gbofdft_delta``) of an FP64 plan and an FP32
    plan on the same grid: the reference density and its FP64 convolution
    results."""

    def __init__(self, plan64, plan32):
        L = load()
        h = ctypes.c_void_p()
        check_alloc(lambda: L.gbofdft_delta_create(plan64.handle, plan32.handle, ctypes.byref(h)), "delta_create")
        self.handle = h
        self._plans = (plan64, plan32)   # the state refers to both plans

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and _lib is not None:
            try:
                _lib.gbofdft_delta_destroy(h)
            except Exception:
                pass
            self.handle = None


def _flat(lat):
    try:
        import numpy as np
        return np.asarray(lat, dtype=float).reshape(9)
    except Exception:
        return [x for row in lat for x in row]
