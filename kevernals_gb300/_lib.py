"""ctypes binding of libkvtomo.so (the C ABI declared in include/kvtomo.h).

The library is built in-tree by kevernals_gb300.build; loading fails loudly
when it is missing -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkvtomo.so")

KV_OK = 0
STATUS_NAMES = {0: "KV_OK", 1: "KV_ERR_INVALID_ARG", 2: "KV_ERR_GEOMETRY", 3: "KV_ERR_OOM",
                4: "KV_ERR_CUDA", 5: "KV_ERR_TIMEOUT", 6: "KV_ERR_NUMERIC",
                7: "KV_ERR_UNSUPPORTED", 8: "KV_ERR_NO_DEVICE"}

FAMILY = {"rc": 0, "exact": 1}
STORAGE = {"f32": 0, "bf16": 1, "f16": 2}
MEM_HOST, MEM_DEVICE = 0, 1

# Every symbol include/kvtomo.h declares, with its ctypes signature.
ITER_CB = C.CFUNCTYPE(C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p)


class KvGeometry(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
                ("n_views", C.c_int32), ("nu", C.c_int32), ("nv", C.c_int32),
                ("du", C.c_float), ("dv", C.c_float),
                ("src", C.POINTER(C.c_float)), ("det_origin", C.POINTER(C.c_float)),
                ("fulcrum_z", C.c_float)]


_vp = C.c_void_p
SIGNATURES = {
    "kv_version": ([], C.c_char_p),
    "kv_status_string": ([C.c_int], C.c_char_p),
    "kv_ctx_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
    "kv_ctx_destroy": ([_vp], C.c_int),
    "kv_ctx_set_stream": ([_vp, _vp], C.c_int),
    "kv_sync": ([_vp], C.c_int),
    "kv_ctx_last_error": ([_vp], C.c_char_p),
    "kv_ctx_set_timing": ([_vp, C.c_int], C.c_int),
    "kv_ctx_timing_read": ([_vp, C.c_char_p, C.c_size_t], C.c_int),
    "kv_plan_create": ([_vp, C.POINTER(KvGeometry), C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
    "kv_plan_destroy": ([_vp], C.c_int),
    "kv_plan_volume_elems": ([_vp], C.c_size_t),
    "kv_plan_proj_elems": ([_vp], C.c_size_t),
    "kv_forward": ([_vp, _vp, _vp, C.c_int], C.c_int),
    "kv_forward_single": ([_vp, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "kv_back": ([_vp, _vp, _vp, C.c_int], C.c_int),
    "kv_sensitivity": ([_vp, _vp, C.c_int], C.c_int),
    "kv_shift_and_add": ([_vp, _vp, _vp, C.c_int], C.c_int),
    "kv_fbp": ([_vp, _vp, _vp, C.c_int32, C.c_int], C.c_int),
    "kv_shift_and_add_shifts": ([C.POINTER(KvGeometry), C.c_int, _vp], C.c_int),
    "kv_uniform_volume": ([_vp, _vp, C.c_int], C.c_int),
    "kv_phantom_ellipsoids": ([_vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float,
                               C.c_float, _vp, C.c_int32, _vp, C.c_int], C.c_int),
    "kv_mlem": ([_vp, _vp, _vp, C.c_int, C.c_float, C.c_int, ITER_CB, _vp], C.c_int),
    "kv_sart": ([_vp, _vp, _vp, C.c_int, C.c_float, C.c_int, ITER_CB, _vp], C.c_int),
    "kv_residual": ([_vp, _vp, _vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)],
                    C.c_int),
    "kv_batch_mlem": ([_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.c_int,
                       C.c_float, C.c_int], C.c_int),
    "kv_plan_autotune": ([_vp], C.c_int),
    "kv_plan_get_tuning": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "kv_plan_set_tuning": ([_vp, C.c_int, C.c_int], C.c_int),
    "kv_plan_get_slab": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                          C.POINTER(C.c_int)], C.c_int),
    "kv_plan_set_slab": ([_vp, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "kv_plan_get_back_shape": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "kv_plan_set_back_shape": ([_vp, C.c_int, C.c_int], C.c_int),
    "kv_plan_get_back_staging": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)], C.c_int),
    "kv_plan_set_back_staging": ([_vp, C.c_int, C.c_int], C.c_int),
    "kv_warm_ratio": ([_vp, _vp, _vp, _vp, C.c_size_t, C.POINTER(C.c_double)], C.c_int),
    "kv_warm_normalize": ([_vp, _vp, _vp, _vp, C.c_size_t], C.c_int),
    "kv_warm_fill": ([_vp, _vp, _vp, _vp, C.c_float, _vp, C.c_size_t], C.c_int),
    "kv_conv3_bf16": ([_vp, _vp, C.c_int32, _vp, C.c_int32, _vp, _vp, C.c_int32, _vp, C.c_int32, C.c_int32,
                       C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "kv_unet_create": ([_vp, C.c_uint64, C.POINTER(_vp)], C.c_int),
    "kv_unet_destroy": ([_vp], C.c_int),
    "kv_unet_num_params": ([_vp], C.c_size_t),
    "kv_unet_forward": ([_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_int], C.c_int),
    "kv_unet_train_step": ([_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                            C.POINTER(C.c_float), C.c_int], C.c_int),
    "kv_unet_gradients": ([_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_float),
                           _vp, C.c_int], C.c_int),
    "kv_unet_get_state": ([_vp, _vp, C.POINTER(C.c_int64)], C.c_int),
    "kv_unet_set_state": ([_vp, _vp, C.c_int64], C.c_int),
    "kv_residual_noalloc": ([_vp, _vp, _vp, C.POINTER(C.c_double), C.POINTER(C.c_double)],
                            C.c_int),
}

_lib = None


def lib():
    """Loads libkvtomo.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                "g.build()\"` (kevernals_gb300.build.build()); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


class KvError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
