"""ctypes binding of ``libswit_gb300.so`` (declared in include/swit_gb300.h).

The library is built in-tree by ``swit_gb300/build.py``.  There is no CPU
fallback: if the library is missing or fails to load, every entry point raises.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libswit_gb300.so")

SWIT_OK = 0
ERRORS = {-1: "SWIT_E_ARG", -2: "SWIT_E_GEOM", -3: "SWIT_E_CFL", -4: "SWIT_E_MODEL", -5: "SWIT_E_STATE",
          -6: "SWIT_E_CUDA", -7: "SWIT_E_NOMEM", -8: "SWIT_E_LIMIT", -9: "SWIT_E_TIMEOUT"}

# every symbol include/swit_gb300.h declares
EXPORTS = ("swit_create", "swit_set_model", "swit_forward", "swit_backward", "swit_gradient_l2",
           "swit_export_snapshot", "swit_import_snapshot", "swit_profile_kernels", "swit_backward_exact", "swit_query", "swit_destroy", "swit_last_error", "swit_damp_profile",
           "swit_forward_shot_static", "swit_check", "swit_misfit_l2", "swit_multi_create", "swit_multi_engine",
           "swit_multi_gradient_l2", "swit_multi_misfit_l2", "swit_multi_destroy", "swit_l2_bandwidth")


class SwitDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("nz", C.c_int32), ("npml", C.c_int32), ("nt", C.c_int32),
                ("dx", C.c_float), ("dt", C.c_float), ("free_surface", C.c_int32), ("ns", C.c_int32),
                ("ng_max", C.c_int32), ("ng", C.c_void_p), ("src_x", C.c_void_p), ("src_z", C.c_void_p),
                ("rec_x", C.c_void_p), ("rec_z", C.c_void_p), ("precision", C.c_int32), ("path", C.c_int32),
                ("shots_per_batch", C.c_int32), ("block_x", C.c_int32),
                ("kernel_variant", C.c_int32), ("checkpoint_every", C.c_int32),
                ("graph_branches", C.c_int32), ("adjoint_mode", C.c_int32), ("receiver_component", C.c_int32)]


class SwitError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "SWIT_E_?"), code, msg))
        self.code = code


_lib = None


def load(build_if_missing: bool = True):
    """Loads the engine library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("swit_gb300: CUDA engine library %s is missing; run swit_gb300/build.py" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    i = C.c_int
    sig = {
        "swit_create": ([C.POINTER(SwitDesc), C.POINTER(vp)], i),
        "swit_set_model": ([vp, vp, vp, i, vp], i),
        "swit_forward": ([vp, vp, vp, i, i, vp], i),
        "swit_backward": ([vp, vp, vp, vp, vp, i, vp], i),
        "swit_gradient_l2": ([vp, vp, vp, vp, vp, vp, vp, C.POINTER(C.c_double), i, vp], i),
        "swit_export_snapshot": ([vp, vp, vp, vp, vp, i, vp], i),
        "swit_import_snapshot": ([vp, vp, vp, vp, vp, vp, i, vp], i),
        "swit_profile_kernels": ([vp, C.POINTER(C.c_int32), C.POINTER(C.c_double), vp], i),
        "swit_backward_exact": ([vp, vp, vp, vp, C.c_int32, vp], i),
        "swit_query": ([vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                        C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)], i),
        "swit_destroy": ([vp], i),
        "swit_check": ([vp, vp], i),
        "swit_misfit_l2": ([vp, vp, vp, C.POINTER(C.c_double), C.c_int32, vp], i),
        "swit_multi_create": ([C.POINTER(SwitDesc), C.c_int32, C.POINTER(vp)], i),
        "swit_multi_engine": ([vp, C.c_int32, C.POINTER(vp)], i),
        "swit_multi_gradient_l2": ([vp, vp, vp, vp, vp, vp, C.POINTER(C.c_double), C.c_int32, vp], i),
        "swit_multi_misfit_l2": ([vp, vp, vp, vp, C.POINTER(C.c_double), C.c_int32, vp], i),
        "swit_multi_destroy": ([vp], i),
        "swit_last_error": ([], C.c_char_p),
        "swit_damp_profile": ([C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float, vp], i),
        "swit_l2_bandwidth": ([C.c_int64, C.c_int32, C.POINTER(C.c_double), vp], i),
        "swit_forward_shot_static": ([C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_int32,
                                      C.c_float, C.c_float, C.c_int32, vp, vp, vp, vp, vp, vp, vp], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def check(rc):
    if rc != SWIT_OK:
        msg = load().swit_last_error().decode(errors="replace")
        raise SwitError(rc, msg)
    return rc
