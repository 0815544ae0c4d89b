"""ctypes binding of librectv_gb300.so (the C ABI declared in include/rectv_gb300.h).

The library is built in-tree by ``rectv_gpu_gb300.build`` (or
``__graft_entry__.build()``).  Loading fails loudly if it is missing: there is
no CPU implementation behind this package.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librectv_gb300.so")

# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
_IP = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "rectv_last_error": (ctypes.c_char_p, []),
    "rectv_version": (ctypes.c_char_p, []),
    "rectv_create": (_I, [_I, _I, _I, _I, _I, _I, ctypes.POINTER(_P)]),
    "rectv_get_dims": (_I, [_P, _IP, _IP, _IP, _IP, _IP, _IP]),
    "rectv_run": (_I, [_P, _P, _P, _P, _P, _F, _F, _F, _I, _I]),
    "rectv_check_adjoints": (_I, [_P, _P, _P, _P, _P, _F, _F]),
    "rectv_free": (_I, [_P]),
    "rectv_destroy": (None, [_P]),
    "rectv_set_verbose": (_I, [_P, _I]),
    "rectv_setup_device": (_I, [_P, _P, _P, _P, _F, _F, _F, _I]),
    "rectv_iterate": (_I, [_P, _I]),
    "rectv_get_result_device": (_I, [_P, _P]),
    "rectv_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "rectv_synchronize": (_I, [_P]),
    "rectv_get_history": (_I, [_P, _P, _P, _P, _P, _IP]),
    "rectv_set_graphs": (_I, [_P, _I]),
    "rectv_op_set_geometry": (_I, [_P, _P, _P, _F]),
    "rectv_op_radonapr": (_I, [_P, _P, _P, _I, _F]),
    "rectv_op_radonapradj": (_I, [_P, _P, _P, _I, _F]),
    "rectv_op_gradient": (_I, [_P, _P, _P, _F, _I, _I]),
    "rectv_op_divergent": (_I, [_P, _P, _P, _F, _F]),
    "rectv_launch_kernel": (_I, [_P, _I, _I]),
    "rectv_kernel_cost": (_I, [_P, _I, _P, _P]),
    "rectv_get_launch_counts": (_I, [_P, _IP, _IP, _IP]),
    "rectv_get_directions": (_I, [_P, _IP, _IP]),
    "rectv_plan_directions": (_I, [_P, _I, _I, _D, _D, _IP, _IP]),
    "rectv_selftest_wait": (_I, [_P, ctypes.c_longlong, _I]),
    "rectv_autotune": (_I, [_P, _I, _IP, _IP]),
    "rectv_measure_fp32_peak": (_I, [_P, _P]),
    "rectv_get_device_bytes": (_I, [_P, _P]),
    "rectv_estimate_bytes": (_I, [_I, _I, _I, _I, _I, _P]),
    "rectv_engine_create": (_I, [_D, _I, _I, ctypes.POINTER(_P)]),
    "rectv_engine_submit": (_I, [_P, _I, _I, _I, _I, _I, _P, _P, _P, _F, _F, _F, _I, _I, _D, _P, _IP]),
    "rectv_engine_run": (_I, [_P]),
    "rectv_engine_job_info": (_I, [_P, _I, _P, _P, _P, _IP, _IP]),
    "rectv_engine_job_error": (_I, [_P, _I, ctypes.c_char_p, _I]),
    "rectv_engine_stats": (_I, [_P, _P]),
    "rectv_engine_destroy": (None, [_P]),
    "rectv_shrink_noalloc": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _F, _F, _F, _P, _P]),
    "rectv_preprocess": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I]),
    "rectv_fbp": (_I, [_P, _P, _P, _P, _F]),
    "rectv_run_init": (_I, [_P, _P, _P, _P, _P, _P, _F, _F, _F, _I, _I]),
}

_lib = None


class RectvError(RuntimeError):
    """A nonzero status from the C ABI."""

    def __init__(self, code, msg):
        super().__init__("rectv error %d: %s" % (code, msg))
        self.code = code


def load():
    """Load the shared library (once) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "librectv_gb300.so not found at %s; build it with "
            "`python -m rectv_gpu_gb300.build` (no CPU fallback exists)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != 0:
        raise RectvError(status, load().rectv_last_error().decode())
