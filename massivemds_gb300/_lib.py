"""ctypes binding of libmdsx.so (the C ABI declared in include/mdsx.h).

There is no fallback: if the CUDA library is missing or cannot be loaded, every
engine call raises. Build it with ``massivemds_gb300.build.build()`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB_PATH

MDSX_OK = 0
STATUS_NAMES = {
    1: "MDSX_EINVAL",
    2: "MDSX_ENOMEM",
    3: "MDSX_ECUDA",
    4: "MDSX_ETIMEOUT",
    5: "MDSX_ESTATE",
    6: "MDSX_EUNSUPPORTED",
}

# Every symbol include/mdsx.h declares, with (restype, argtypes).
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_i, _sz, _l = ctypes.c_int, ctypes.c_size_t, ctypes.c_long
SIGNATURES = {
    "mdsx_create": (_i, [_i, _i, _l, _i, ctypes.POINTER(_vp)]),
    "mdsx_create_rows": (_i, [_i, _i, _l, _i, _i, _i, ctypes.POINTER(_vp)]),
    "mdsx_get_row_range": (_i, [_vp, _ip, _ip]),
    "mdsx_destroy": (_i, [_vp]),
    "mdsx_update_locations": (_i, [_vp, _i, _dp, _sz]),
    "mdsx_get_sum_of_increments": (_i, [_vp, _dp]),
    "mdsx_get_log_likelihood_gradient": (_i, [_vp, _dp, _sz]),
    "mdsx_store_state": (_i, [_vp]),
    "mdsx_restore_state": (_i, [_vp]),
    "mdsx_accept_state": (_i, [_vp]),
    "mdsx_set_pairwise_data": (_i, [_vp, _dp, _sz]),
    "mdsx_set_pairwise_data_f32": (_i, [_vp, _fp, _sz]),
    "mdsx_set_parameters": (_i, [_vp, _dp, _sz]),
    "mdsx_make_dirty": (_i, [_vp]),
    "mdsx_get_internal_dimension": (_i, [_vp, _ip]),
    "mdsx_get_log_likelihood": (_i, [_vp, _dp]),
    "mdsx_last_error": (ctypes.c_char_p, [_vp]),
    "mdsx_set_stream": (_i, [_vp, _vp]),
    "mdsx_update_locations_device": (_i, [_vp, _vp, _sz]),
    "mdsx_evaluate_device": (_i, [_vp, _vp, _vp]),
    "mdsx_last_launch_count": (_i, [_vp, _ip]),
    "mdsx_set_sweep_schedule": (_i, [_vp, _i]),
    "mdsx_get_sweep_schedule": (_i, [_vp, _ip]),
    "mdsx_selftest_bounded_wait": (_i, [ctypes.c_double, _i, _ip]),
    "mdsx_selftest_math_f64": (_i, [_dp, _sz, _dp, _i]),
    "mdsx_hmc_run": (_i, [_vp, _vp, _dp, _dp, _dp, _vp]),
    "mdsx_sweep_f32_noalloc": (_i, [_vp, ctypes.c_longlong, _vp, _i, _i, ctypes.c_double, _i, _vp, _vp, _vp]),
    "mdsx_version": (ctypes.c_char_p, []),
    "mdsx_inject_fault": (_i, [_i, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "mdsx_surrogate_create": (_i, [_vp, _i, _i, _i, _i, ctypes.c_ulonglong, ctypes.POINTER(_vp)]),
    "mdsx_surrogate_destroy": (None, [_vp]),
    "mdsx_surrogate_last_error": (ctypes.c_char_p, [_vp]),
    "mdsx_surrogate_info": (_i, [_vp, _ip, _dp]),
    "mdsx_surrogate_landmarks": (_i, [_vp, _ip]),
    "mdsx_surrogate_parameters": (_i, [_vp, _i, _i, _fp, _fp]),
    "mdsx_surrogate_add_state": (_i, [_vp, _dp, _dp, _i, ctypes.c_ulonglong]),
    "mdsx_surrogate_training_rows": (_i, [_vp, _i, _i, _fp, _fp, _fp]),
    "mdsx_surrogate_train": (_i, [_vp, _i, _i, ctypes.c_double, ctypes.c_ulonglong, _dp]),
    "mdsx_surrogate_batch_gradient": (_i, [_vp, _ip, _i, _dp]),
    "mdsx_surrogate_gradient": (_i, [_vp, _dp, _dp]),
    "mdsx_batch_create": (_i, [_l, _i, ctypes.POINTER(_vp)]),
    "mdsx_batch_destroy": (None, [_vp]),
    "mdsx_batch_last_error": (ctypes.c_char_p, [_vp]),
    "mdsx_batch_instance_count": (_i, [_vp]),
    "mdsx_batch_add_instance": (_i, [_vp, _i, _i, _ip]),
    "mdsx_batch_set_pairwise_data": (_i, [_vp, _i, _dp, _sz]),
    "mdsx_batch_set_pairwise_data_f32": (_i, [_vp, _i, _fp, _sz]),
    "mdsx_batch_set_parameters": (_i, [_vp, _i, _dp, _sz]),
    "mdsx_batch_update_locations": (_i, [_vp, _i, _i, _dp, _sz]),
    "mdsx_batch_make_dirty": (_i, [_vp]),
    "mdsx_batch_get_sum_of_increments": (_i, [_vp, _i, _dp]),
    "mdsx_batch_get_log_likelihood": (_i, [_vp, _i, _dp]),
    "mdsx_batch_get_log_likelihood_gradient": (_i, [_vp, _i, _dp, _sz]),
    "mdsx_batch_evaluate": (_i, [_vp]),
    "mdsx_batch_evaluate_device": (_i, [_vp, _vp, _vp]),
    "mdsx_batch_tune": (_i, [_vp, _i, _ip]),
    "mdsx_batch_group_shape": (_i, [_vp, _i, _ip, _ip, _ip, _ip]),
    "mdsx_batch_force_shape": (_i, [_vp, _i, _i, _i, _i]),
    "mdsx_test_gemm_bf16": (_i, [_i, _i, _i, _i, _i, ctypes.POINTER(ctypes.c_ushort),
                                 ctypes.POINTER(ctypes.c_ushort), _fp]),
}

_lib = None


class MdsxError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: str | None = None):
    """Load libmdsx.so (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"libmdsx.so not found at {path}: the CUDA engine is not built "
            "(run massivemds_gb300.build.build()); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, handle=None) -> None:
    if status != MDSX_OK:
        msg = load().mdsx_last_error(handle)
        raise MdsxError(status, msg.decode() if msg else "")
