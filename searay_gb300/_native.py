"""ctypes binding of libsearay_uppe.so (C ABI declared in include/searay_uppe.h).

The library is built in-tree by ``searay_gb300.build``.  There is no fallback: if the library is
missing or cannot be loaded, :func:`lib` raises.
"""
import ctypes
import pathlib

_PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = _PKG / "libsearay_uppe.so"

UPPE_OK = 0
UPPE_E_ARG = -1
UPPE_E_CUDA = -2
UPPE_E_NOMEM = -3
UPPE_E_RANGE = -4
UPPE_E_NONFINITE = -5

PREC_MIXED = 0
PREC_FP32 = 1

RATE_NONE = 0
RATE_EXPLICIT = 1
RATE_SERIES = 2

EXPORTS = ("uppe_create", "uppe_destroy", "uppe_set_stream", "uppe_set_grid", "uppe_set_material",
           "uppe_load_field", "uppe_rk4_step", "uppe_finish", "uppe_eval_rhs", "uppe_get_field",
           "uppe_check_finite", "uppe_profile_enable", "uppe_profile_read", "uppe_launch_count",
           "uppe_class_name", "uppe_step_size_noalloc", "uppe_set_chi3", "uppe_set_rotator", "uppe_set_field",
           "uppe_adjoint_rk4_step", "uppe_rk4_step_keep", "uppe_adjoint_rk4_step_kept", "uppe_adjoint_load",
           "uppe_adjoint_finish", "uppe_last_error")
NOALLOC_MAX_POINTS = 1 << 27
NCLASS = 6


class UppeConfig(ctypes.Structure):
    _fields_ = [
        ("n0", ctypes.c_int), ("n1", ctypes.c_int), ("n2", ctypes.c_int),
        ("radial_modes", ctypes.c_int), ("cylindrical", ctypes.c_int), ("precision", ctypes.c_int),
        ("dt", ctypes.c_double), ("chi3_over_nref", ctypes.c_double),
        ("nl_cut_on", ctypes.c_int), ("nl_cut_off", ctypes.c_int), ("rate_form", ctypes.c_int),
        ("field_conv", ctypes.c_double), ("rate_conv", ctypes.c_double), ("field_cutoff", ctypes.c_double),
        ("c_pre", ctypes.c_double), ("c_pow", ctypes.c_double), ("c_exp", ctypes.c_double),
        ("clog", ctypes.c_double * 6),
        ("damping", ctypes.c_double),
        ("window_cutoff", ctypes.c_int), ("window_width", ctypes.c_int),
        ("envelope", ctypes.c_int),
    ]


class UppeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH.name} is not built; run `python -m searay_gb300.build` "
                           "(the UPPE path has no CPU fallback)")
    L = ctypes.CDLL(str(LIB_PATH))
    vp = ctypes.c_void_p
    L.uppe_create.argtypes = [ctypes.POINTER(UppeConfig), ctypes.POINTER(vp)]
    L.uppe_destroy.argtypes = [vp]
    L.uppe_set_stream.argtypes = [vp, vp]
    L.uppe_set_grid.argtypes = [vp, _dp, _dp, _dp, _dp]
    L.uppe_set_material.argtypes = [vp, _dp, _dp, _dp]
    L.uppe_load_field.argtypes = [vp, vp]
    L.uppe_rk4_step.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
    L.uppe_finish.argtypes = [vp, ctypes.c_double, vp, vp, vp, vp]
    L.uppe_eval_rhs.argtypes = [vp, vp, ctypes.c_double, vp]
    L.uppe_get_field.argtypes = [vp, vp]
    L.uppe_check_finite.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.uppe_profile_enable.argtypes = [vp, ctypes.c_int]
    L.uppe_profile_read.argtypes = [vp, _dp, ctypes.POINTER(ctypes.c_longlong)]
    L.uppe_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    L.uppe_class_name.argtypes = [ctypes.c_int]
    L.uppe_class_name.restype = ctypes.c_char_p
    L.uppe_step_size_noalloc.argtypes = [vp, vp, ctypes.c_longlong, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, vp, vp]
    L.uppe_set_chi3.argtypes = [vp, ctypes.c_double]
    L.uppe_set_rotator.argtypes = [vp, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_double]
    L.uppe_set_field.argtypes = [vp, vp]
    L.uppe_adjoint_rk4_step.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, _dp]
    L.uppe_rk4_step_keep.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.uppe_adjoint_rk4_step_kept.argtypes = [vp, vp, vp, _dp]
    L.uppe_adjoint_load.argtypes = [vp, vp, vp]
    L.uppe_adjoint_finish.argtypes = [vp, ctypes.c_double, vp, vp]
    L.uppe_last_error.argtypes = [vp]
    L.uppe_last_error.restype = ctypes.c_char_p
    for name in EXPORTS:
        if name not in ("uppe_last_error", "uppe_class_name"):
            getattr(L, name).restype = ctypes.c_int
    _LIB = L
    return L


def check(rc, handle=None):
    if rc != UPPE_OK:
        msg = lib().uppe_last_error(handle)
        raise UppeError(rc, msg.decode() if msg else "unknown error")
    return rc


def dptr(a):
    """Pointer to a C-contiguous float64 NumPy array (or None)."""
    if a is None:
        return None
    assert a.dtype.name == "float64" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)
