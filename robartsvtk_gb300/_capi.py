"""ctypes binding of the C ABI in include/hmf.h (libhmf_gb300.so).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared library is missing or cannot be built.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

HMF_OK = 0
HMF_HOST = 0
HMF_DEVICE = 1
HMF_SEMANTICS_REF_CUDA = 0
HMF_SEMANTICS_REF_CPU = 1
HMF_STALL_FLOW = 0
HMF_STALL_SWEEP = 1
HMF_STALL_REVERSE_FLOW = 2
HMF_STALL_REVERSE_SWEEP = 3
HMF_FP64_PROBE_NONE = 0
HMF_FP64_PROBE_DATA = 1
HMF_FP64_PROBE_ALPHA = 2
HMF_PAGED_INPUTS_AUTO = 0
HMF_PAGED_INPUTS_HOST = 1
HMF_PAGED_INPUTS_DEVICE = 2

ERRORS = {
    -1: "HMF_ERR_INVALID_ARGUMENT",
    -2: "HMF_ERR_TREE",
    -3: "HMF_ERR_MISSING_INPUT",
    -4: "HMF_ERR_CUDA",
    -5: "HMF_ERR_OUT_OF_MEMORY",
    -6: "HMF_ERR_STATE",
}

# (name, restype, argtypes) of every symbol declared in include/hmf.h
_P = ctypes.c_void_p
_I = ctypes.c_int
SIGNATURES = [
    ("hmf_create", _I, [ctypes.POINTER(_P), _I, _I, _I, ctypes.POINTER(_I), _I, _I, _I]),
    ("hmf_destroy", _I, [_P]),
    ("hmf_set_data", _I, [_P, _I, _P, _I]),
    ("hmf_set_smoothness", _I, [_P, _I, _P, _I]),
    ("hmf_set_smoothness_scalar", _I, [_P, _I, ctypes.c_double]),
    ("hmf_set_params", _I, [_P, _I, ctypes.c_float, ctypes.c_float]),
    ("hmf_solve", _I, [_P, _P]),
    ("hmf_solve_continue", _I, [_P, _P]),
    ("hmf_get_labels", _I, [_P, _I, _P, _I, _P]),
    ("hmf_get_sink", _I, [_P, _I, _P, _I, _P]),
    ("hmf_leaf_order", _I, [_P, ctypes.POINTER(_I), _I]),
    ("hmf_device_bytes", ctypes.c_size_t, [_P]),
    ("hmf_set_timing", _I, [_P, _I]),
    ("hmf_get_stats", _I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double), _I]),
    ("hmf_last_error", ctypes.c_char_p, [_P]),
    ("hmf_create_batch", _I, [ctypes.POINTER(_P), _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _I, _I, _I]),
    ("hmf_data_term", _I, [_I, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P, _P,
                           ctypes.c_longlong, _P, _I, _P]),
    ("hmf_log_likelihood", _I, [_P, _I, ctypes.POINTER(_P), _I, ctypes.c_longlong, _I, ctypes.c_float,
                                ctypes.c_double, _I, _P, _I, _P]),
    ("hmf_create_dag", _I, [ctypes.POINTER(_P), _I, _I, _I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I),
                            ctypes.POINTER(ctypes.c_float), _I, _I]),
    ("hmf_num_volumes", _I, [_P]),
    ("hmf_batch_set_data", _I, [_P, _I, _I, _P, _I]),
    ("hmf_batch_set_smoothness", _I, [_P, _I, _I, _P, _I]),
    ("hmf_batch_get_labels", _I, [_P, _I, _I, _P, _I, _P]),
    ("hmf_batch_get_sink", _I, [_P, _I, _I, _P, _I, _P]),
    ("hmf_autotune", _I, [_P, _P]),
    ("hmf_solve_adjoint", _I, [_P, _P, _I, _I, ctypes.c_double, ctypes.POINTER(ctypes.c_double), _P]),
    ("hmf_get_data_gradient", _I, [_P, _I, _P, _I, _P]),
    ("hmf_get_alpha_gradient", _I, [_P, ctypes.POINTER(ctypes.c_double), _I]),
    ("hmf_get_adjoint_plan", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("hmf_set_adjoint_memory", _I, [_P, ctypes.c_longlong, _I]),
    ("hmf_set_zchunk", _I, [_P, _I]),
    ("hmf_get_zchunk", _I, [_P]),
    ("hmf_set_pipeline", _I, [_P, _I]),
    ("hmf_get_pipeline", _I, [_P]),
    ("hmf_set_flow_window", _I, [_P, _I]),
    ("hmf_get_flow_window", _I, [_P]),
    ("hmf_set_flow_units", _I, [_P, _I]),
    ("hmf_get_flow_units", _I, [_P]),
    ("hmf_get_adjoint_schedule", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_longlong),
                                      ctypes.POINTER(ctypes.c_longlong)]),
    ("hmf_adjoint_schedule", ctypes.c_longlong, [_I, _I, _I, ctypes.POINTER(_I), ctypes.c_longlong]),
    ("hmf_vote", _I, [_I, ctypes.POINTER(_P), ctypes.POINTER(_I), ctypes.c_longlong, _I, _P, _I, _P]),
    ("hmf_get_vote", _I, [_P, _P, _I, _P]),
    ("hmf_batch_get_vote", _I, [_P, _I, _P, _I, _P]),
    ("hmf_decomposition_energy", _I, [_I, _I, _I, ctypes.POINTER(_I), _I, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                      ctypes.POINTER(_P), _I, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double), _P]),
    ("hmf_get_energy", _I, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _I]),
    ("hmf_batch_get_energy", _I, [_P, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _I]),
    ("hmf_set_convergence_log", _I, [_P, _I]),
    ("hmf_get_convergence", _I, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _I]),
    ("hmf_set_wait_limit", _I, [_P, ctypes.c_longlong]),
    ("hmf_inject_wait_stall", _I, [_P, _I]),
    ("hmf_solve_fp64", _I, [_P, _P]),
    ("hmf_get_labels_fp64", _I, [_P, _I, _P, _I, _P]),
    ("hmf_fp64_error", _I, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _P]),
    ("hmf_fp64_loss", _I, [_P, _P, _I, ctypes.c_double, ctypes.POINTER(ctypes.c_double), _P]),
    ("hmf_set_fp64_probe", _I, [_P, _I, _I, ctypes.c_longlong, ctypes.c_double]),
    ("hmf_create_paged", _I, [ctypes.POINTER(_P), _I, _I, _I, ctypes.POINTER(_I), _I, _I, _I, ctypes.c_double]),
    ("hmf_set_paged_plan", _I, [_P, _I, _I, _I]),
    ("hmf_get_paged_plan", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                ctypes.POINTER(ctypes.c_longlong)]),
    ("hmf_paged_layout", _I, [_I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _I]),
    ("hmf_solve_noalloc", _I, [_I, _I, _I, ctypes.POINTER(_I), _I, _I, ctypes.POINTER(_P), ctypes.POINTER(_P),
                               ctypes.POINTER(ctypes.c_double), _I, ctypes.c_float, ctypes.c_float,
                               ctypes.POINTER(_P), _P]),
]

_lib = None
_lock = threading.Lock()


class HMFError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "HMF_ERR"), code, message))
        self.code = code


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libhmf_gb300.so (building it first if needed) and bind its symbols."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise FileNotFoundError("libhmf_gb300.so is not built: run robartsvtk_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, ctx=None) -> int:
    if rc < 0:
        msg = load().hmf_last_error(ctx)
        raise HMFError(rc, msg.decode() if msg else "")
    return rc
