"""ctypes binding of the engine's C ABI (include/omr_ntt.h).

The shared library is built in-tree by ``omr-ntt_gb300/build.py``.  There is
no CPU fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libomr_ntt.so")

OK = 0
STATUS = {
    0: "OK",
    -1: "INVALID_ARGUMENT",
    -2: "SIZE",
    -3: "PRECONDITION",
    -4: "CUDA",
    -5: "ALLOC",
    -6: "TIMEOUT",
    -7: "NONCANONICAL",
    -8: "DUPLICATE",
    -9: "CAPACITY",
}


class OmrNttError(RuntimeError):
    """A C-ABI call returned a non-zero omr_ntt_status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


_lib = None

_c = ctypes
_SIGS = {
    "omr_ntt_domain_create": (_c.c_int, [_c.c_int, _c.c_uint32, _c.POINTER(_c.c_void_p)]),
    "omr_ntt_domain_destroy": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_domain_info": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_int), _c.POINTER(_c.c_uint64),
                                        _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint64)]),
    "omr_ntt_domain_check": (_c.c_int, [_c.c_void_p, _c.c_void_p]),
    "omr_ntt_domain_twiddles": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p]),
    "omr_ntt_encoder_name": (_c.c_char_p, [_c.c_int]),
    "omr_ntt_encoder_supports": (_c.c_int, [_c.c_int, _c.c_uint32]),
    "omr_ntt_encoder_plan": (_c.c_int, [_c.c_int, _c.c_int, _c.c_uint32]),
    "omr_ntt_encode": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_uint64, _c.c_void_p, _c.c_uint64,
                                   _c.c_void_p]),
    "omr_ntt_encode_host": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_uint64, _c.c_void_p, _c.c_uint64]),
    "omr_ntt_forward": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p, _c.c_void_p, _c.c_uint64,
                                    _c.c_void_p]),
    "omr_ntt_inverse": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p, _c.c_void_p, _c.c_uint64,
                                    _c.c_void_p]),
    "omr_ntt_forward_noalloc": (_c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_uint64,
                                            _c.c_void_p]),
    "omr_ntt_forward_host": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p, _c.c_uint64]),
    "omr_ntt_inverse_host": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p, _c.c_uint64]),
    "omr_ntt_partial": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_uint64, _c.c_void_p, _c.c_void_p,
                                    _c.c_void_p, _c.c_void_p]),
    "omr_ntt_partial_host": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_uint64, _c.c_void_p,
                                         _c.c_void_p, _c.c_void_p]),
    "omr_ntt_check_canonical": (_c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_uint64, _c.c_void_p]),
    "omr_ntt_plan_count": (_c.c_int, [_c.c_int, _c.c_uint32]),
    "omr_ntt_plan_describe": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_int, _c.c_char_p, _c.c_size_t]),
    "omr_ntt_plan_passes": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_int, _c.c_uint64,
                                        _c.POINTER(_c.c_uint64), _c.c_int]),
    "omr_ntt_plan_run_pass": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_int, _c.c_int, _c.c_void_p,
                                          _c.c_void_p, _c.c_void_p, _c.c_uint64, _c.c_void_p]),
    "omr_ntt_candidates": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_int, _c.c_uint64,
                                       _c.POINTER(_c.c_int), _c.POINTER(_c.c_int), _c.c_int]),
    "omr_ntt_run_candidate": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_int, _c.c_int, _c.c_uint64,
                                          _c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_uint64,
                                          _c.c_void_p]),
    "omr_ntt_tune_point": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_uint64, _c.c_int, _c.c_uint64,
                                       _c.c_int, _c.c_uint64, _c.POINTER(_c.c_float), _c.c_int]),
    "omr_ntt_planner_set": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_uint64, _c.c_int, _c.c_uint64,
                                        _c.c_int, _c.c_int]),
    "omr_ntt_planner_get": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_uint64, _c.c_int, _c.c_uint64,
                                        _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    "omr_ntt_planner_clear": (_c.c_int, []),
    "omr_ntt_planner_save": (_c.c_int, [_c.c_char_p]),
    "omr_ntt_planner_load": (_c.c_int, [_c.c_char_p]),
    "omr_ntt_batch_create": (_c.c_int, [_c.POINTER(_c.c_void_p)]),
    "omr_ntt_batch_destroy": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_batch_add": (_c.c_int, [_c.c_void_p, _c.c_int, _c.c_uint32, _c.c_int, _c.c_int,
                                      _c.c_uint64, _c.c_void_p, _c.c_uint64, _c.c_uint64]),
    "omr_ntt_batch_build": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_batch_info": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64),
                                       _c.POINTER(_c.c_uint64)]),
    "omr_ntt_batch_run": (_c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_void_p]),
    "omr_ntt_batch_check": (_c.c_int, [_c.c_void_p, _c.c_void_p]),
    "omr_ntt_batch_inject_stall": (_c.c_int, [_c.c_void_p, _c.c_uint32]),
    "omr_ntt_batch_run_per_request": (_c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_void_p]),
    "omr_ntt_plan_class_count": (_c.c_int, []),
    "omr_ntt_plan_class_candidate": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_int, _c.c_uint64, _c.c_int,
                                                 _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    "omr_ntt_planner_use_mlp": (_c.c_int, [_c.c_int]),
    "omr_ntt_mlp_features": (_c.c_int, [_c.c_int, _c.c_uint32, _c.c_uint64, _c.c_int, _c.c_uint64,
                                         _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_create": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int, _c.c_uint64, _c.POINTER(_c.c_void_p)]),
    "omr_ntt_mlp_destroy": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_mlp_param_count": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_mlp_get_params": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_set_params": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_forward": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_float), _c.c_int, _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_gradients": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_float), _c.POINTER(_c.c_float),
                                          _c.POINTER(_c.c_float), _c.c_int, _c.POINTER(_c.c_float),
                                          _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_fit": (_c.c_int, [_c.c_void_p, _c.POINTER(_c.c_float), _c.POINTER(_c.c_float),
                                    _c.POINTER(_c.c_float), _c.c_int, _c.c_int, _c.c_int, _c.c_float,
                                    _c.c_uint64, _c.POINTER(_c.c_float)]),
    "omr_ntt_mlp_install": (_c.c_int, [_c.c_void_p]),
    "omr_ntt_mlp_load": (_c.c_int, [_c.c_char_p, _c.POINTER(_c.c_void_p)]),
    "omr_ntt_last_error": (_c.c_char_p, []),
    "omr_ntt_version": (_c.c_char_p, []),
}


def lib():
    """Load the engine library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OmrNttError(-4, f"engine library not built: {LIB_PATH} (run build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def declared_symbols():
    return list(_SIGS)


def check(rc: int):
    if rc != OK:
        msg = lib().omr_ntt_last_error()
        raise OmrNttError(rc, msg.decode() if msg else "")
    return rc
