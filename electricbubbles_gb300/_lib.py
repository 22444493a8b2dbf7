"""ctypes binding of libeb_gb300.so (declarations in include/eb_gb300.h).

Loading fails loudly: there is no CPU fallback for any operator of this package.
"""
import ctypes
import os

from . import build as _build

EB_OK = 0
EB_HOST = 0
EB_DEVICE = 1
EB_FP64 = 0
EB_FP32 = 1
EB_SOLVE_FP64 = 0
EB_SOLVE_FP32_REFINED = 1

STATUS_NAMES = {
    0: "EB_OK", 1: "EB_ERR_ARG", 2: "EB_ERR_CUDA", 3: "EB_ERR_NOGEOM", 4: "EB_ERR_WORKSPACE",
    5: "EB_ERR_TOL", 6: "EB_ERR_NAN", 7: "EB_ERR_NOT_CONVERGED", 8: "EB_ERR_NODEVICE",
    9: "EB_ERR_TIMEOUT",
}


class EbError(RuntimeError):
    """A C-ABI call returned a status other than EB_OK."""

    def __init__(self, fn, status, msg):
        self.status = status
        super().__init__("%s -> %s: %s" % (fn, STATUS_NAMES.get(status, status), msg))


class Opts(ctypes.Structure):
    _fields_ = [("p64", ctypes.c_int), ("p32", ctypes.c_int), ("leaf64", ctypes.c_int),
                ("leaf_cap", ctypes.c_int), ("tol64", ctypes.c_double), ("tol32", ctypes.c_double),
                ("maxl", ctypes.c_int), ("gmres_tol", ctypes.c_double),
                ("inner_tol", ctypes.c_double), ("max_outer", ctypes.c_int),
                ("device", ctypes.c_int), ("graphs", ctypes.c_int), ("df64", ctypes.c_int),
                ("resid_df", ctypes.c_int), ("m2l_tc", ctypes.c_int),
                ("lap_deflate", ctypes.c_int), ("direct_max", ctypes.c_int), ("adj_df", ctypes.c_int)]


class TuneInfo(ctypes.Structure):
    _fields_ = [("leaf64", ctypes.c_int), ("leaf_cap", ctypes.c_int), ("ncand", ctypes.c_int),
                ("leaf_target", ctypes.c_int * 8), ("leaf_cap_cand", ctypes.c_int * 8),
                ("apply_us", ctypes.c_double * 8)]

    def as_dict(self):
        k = self.ncand
        return {"leaf64": self.leaf64, "leaf_cap": self.leaf_cap,
                "candidates": [{"leaf64": self.leaf_target[i], "leaf_cap": self.leaf_cap_cand[i],
                                "apply_us": self.apply_us[i]} for i in range(k)]}


class SolveInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("outer", ctypes.c_int), ("matvecs64", ctypes.c_int),
                ("matvecs32", ctypes.c_int), ("err", ctypes.c_double), ("ierr", ctypes.c_int),
                ("graph", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TreeInfo(ctypes.Structure):
    _fields_ = [("npoints", ctypes.c_int), ("levels", ctypes.c_int), ("nboxes", ctypes.c_int),
                ("nleaves", ctypes.c_int), ("v_pairs", ctypes.c_longlong),
                ("u_pairs", ctypes.c_longlong), ("p", ctypes.c_int), ("w_pairs", ctypes.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Model(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_double), ("e0", ctypes.c_double),
                ("zbond", ctypes.c_double * 2), ("mode", ctypes.c_int)]


class StageInfo(ctypes.Structure):
    _fields_ = [("lap_iters", ctypes.c_int), ("stokes_iters", ctypes.c_int),
                ("lap_err", ctypes.c_double), ("stokes_err", ctypes.c_double),
                ("flux", ctypes.c_double), ("lap_ierr", ctypes.c_int),
                ("stokes_ierr", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class AdjointInfo(ctypes.Structure):
    _fields_ = [("lap_iters", ctypes.c_int), ("stokes_iters", ctypes.c_int),
                ("lap_adj_iters", ctypes.c_int), ("stokes_adj_iters", ctypes.c_int),
                ("ierr", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# name -> (restype, argtypes); every entry is a symbol of include/eb_gb300.h
SIGNATURES = {
    "eb_version": (_I, []),
    "eb_status_string": (ctypes.c_char_p, [_I]),
    "eb_last_error": (ctypes.c_char_p, []),
    "eb_opts_default": (None, [ctypes.POINTER(Opts)]),
    "eb_ctx_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(Opts)]),
    "eb_ctx_destroy": (_I, [_P]),
    "eb_ctx_set_stream": (_I, [_P, _P]),
    "eb_ctx_sync": (_I, [_P]),
    "eb_ctx_launch_count": (ctypes.c_longlong, [_P]),
    "eb_ctx_set_profiling": (_I, [_P, _I]),
    "eb_ctx_kernel_time": (_I, [_P, _I, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_D)]),
    "eb_ctx_tree_info": (_I, [_P, ctypes.POINTER(TreeInfo)]),
    "eb_measure_fp64_peak": (_I, [_P, ctypes.POINTER(_D)]),
    "eb_measure_fp32_peak": (_I, [_P, ctypes.POINTER(_D)]),
    "eb_set_geometry": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _I]),
    "eb_extractdat": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I]),
    "eb_stokes_matvec": (_I, [_P, _I, _P, _P, _I, _I]),
    "eb_laplace_matvec": (_I, [_P, _I, _P, _P, _I, _I]),
    "eb_laplace_constraints": (_I, [_P, _I, _P, _P, _I]),
    "eb_stokes_sum": (_I, [_P, _I, _P, _I, _P, _I, _I]),
    "eb_cauchy_sum": (_I, [_P, _I, _P, _P, _P, _I, _I]),
    "eb_stokes_sum_noalloc": (_I, [_I, _P, _P, _P, _P, _I, _P, _P]),
    "eb_stokes_solve": (_I, [_P, _I, _P, _P, _I, ctypes.POINTER(SolveInfo), _I]),
    "eb_laplace_solve": (_I, [_P, _I, _P, _P, _I, ctypes.POINTER(SolveInfo), _I]),
    "eb_fdiff": (_I, [_P, _P, _P, _I]),
    "eb_pvintev": (_I, [_P, _P, _P, _I, _I]),
    "eb_dirich_neu_map": (_I, [_P, _P, _P, _P, _P, _I, _I]),
    "eb_interface_velocity": (_I, [_P, _P, _P, _D, _P, _P, _I, _I]),
    "eb_setvelf": (_I, [_P, _P, _D, _D, _P, _I]),
    "eb_setvelf_bond": (_I, [_P, _P, _D, _D, _P, _P, _P, _I]),
    "eb_set_wall": (_I, [_P, _I]),
    "eb_stokes_matvec_adjoint": (_I, [_P, _I, _P, _P, _I, _I]),
    "eb_laplace_matvec_adjoint": (_I, [_P, _I, _P, _P, _I, _I]),
    "eb_stokes_solve_adjoint": (_I, [_P, _I, _P, _P, _I, ctypes.POINTER(SolveInfo), _I]),
    "eb_laplace_solve_adjoint": (_I, [_P, _I, _P, _P, _I, ctypes.POINTER(SolveInfo), _I]),
    "eb_get_wall": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "eb_rk_f": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(Model), ctypes.POINTER(StageInfo), _I]),
    "eb_rk2_step": (_I, [_P, _I, _P, _D, _P, ctypes.POINTER(Model), ctypes.POINTER(StageInfo),
                         _I]),
    "eb_rk_f_vjp": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(Model), _P, _P,
                         ctypes.POINTER(AdjointInfo), _I]),
    "eb_rk2_step_vjp": (_I, [_P, _I, _P, _D, _P, _P, ctypes.POINTER(Model), _P,
                             ctypes.POINTER(AdjointInfo), _I]),
    "eb_deformation": (_I, [_P, _I, _P, _P, ctypes.POINTER(_D), _P, _I]),
    "eb_rk2_gradient": (_I, [_P, _I, _P, _D, _I, _P, ctypes.POINTER(Model), ctypes.POINTER(_D), _P, _P,
                             ctypes.POINTER(AdjointInfo), _I]),
    "eb_batch_define": (_I, [_P, _I, _P, _P]),
    "eb_getfourier": (_I, [_P, _I, _P, _P, _P, _P, _I]),
    "eb_double": (_I, [_P, _I, _P, _P, _P, _P, _I]),
    "eb_autotune": (_I, [_P, ctypes.POINTER(TuneInfo)]),
    "eb_bubbin_read": (_I, [ctypes.c_char_p, _I, _P, _P, _P, _P]),
    "eb_geoinit": (_I, [_I, _P, _P, _P, _P, _P, _P]),
    "eb_dumpdata": (_I, [ctypes.c_char_p, _I, _P, _D, _D, _P, _P, _P]),
    "eb_readdata": (_I, [ctypes.c_char_p, _I, ctypes.c_long, _P, _P, _P, _P, _P, _P, _P]),
    "eb_set_default_ctx": (_I, [_P]),
    "matvec_": (None, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "matvec_lapl_": (None, [_P, _P, _P, _P, _P, _P, _P, _P]),
}

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libeb_gb300.so, declaring every entry point. Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("libeb_gb300.so is not built (%s); run "
                               "electricbubbles_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn, status):
    if status != EB_OK:
        msg = _lib.eb_last_error().decode(errors="replace") if _lib is not None else ""
        raise EbError(fn, status, msg)
