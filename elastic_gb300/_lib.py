"""ctypes binding of libelastic_rtm.so (the C-ABI in include/elastic_rtm.h).

There is no fallback: if the shared library is missing or cannot be loaded,
every call raises.  Build it with ``python -m elastic_gb300.build`` (or
``__graft_entry__.build()``).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libelastic_rtm.so")

_c_int, _c_float, _c_double = ctypes.c_int, ctypes.c_float, ctypes.c_double
_P = ctypes.c_void_p

# name -> (restype, argtypes); one line per entry point of include/elastic_rtm.h
SIGNATURES = {
    "rtm_last_error": (ctypes.c_char_p, []),
    "rtm_last_status": (_c_int, []),
    "rtm_set_exact": (None, [_c_int]),
    "rtm_set_kernel_version": (None, [_c_int]),
    "rtm_op3_c_": (None, [_c_int] * 4 + [_P] * 10),
    "rtm_op3_dev_noalloc": (_c_int, [_c_int] * 3 + [_P] * 11),
    "rtm_gpu_init": (None, [_c_int] * 3),
    "rtm_gpu_copy_in": (None, [_c_int] * 3 + [_P] * 10),
    "rtm_gpu_copy_out": (None, [_c_int] * 3 + [_P] * 5),
    "rtm_gpu_func": (None, [_c_int] * 4 + [_P] * 12),
    "rtm_gpu_final": (None, []),
    "rtm_model_op_c_": (_c_int, [_c_int, _c_int, _c_float, _c_float] + [_P] * 8),
    "rtm_source_c_": (_c_int, [_c_int, _c_float, _c_float, _c_int, _P]),
    "rtm_abc_c_": (_c_int, [_c_int, _P]),
    "rtm_fwd_c_": (_c_int, [_c_int, _c_int, _c_int, _c_float, _c_int, _c_int, _c_int] + [_P] * 11),
    "rtm_image_init_c_": (_c_int, [_c_int, _c_int, _c_int, _c_float, _c_float] + [_P] * 8),
    "rtm_model_delta_c_": (_c_int, [_c_int, _c_int, _P, _P, _P]),
    "rtm_image_op_c_": (_c_int, [_c_int] * 4 + [_P] * 14),
    "rtm_born_scatter_c_": (_c_int, [_c_int] * 5 + [_P] * 15),
    "rtm_op3_full_c_": (_c_int, [_c_int] * 6 + [_P] * 15),
    "rtm_op_c_": (_c_int, [_c_int] * 4 + [_c_float, _c_float] + [_c_int] * 3 + [_c_float, _c_int, _c_int]
                  + [_P] * 11 + [_c_int, _c_int]),
    "rtm_op_d_": (_c_int, [_c_int] * 4 + [_c_double, _c_double] + [_c_int] * 3 + [_c_double, _c_int, _c_int]
                  + [_P] * 11 + [_c_int, _c_int]),
    "rtm_velocity_jacobian_c_": (_c_int, [_c_int] * 3 + [_P] * 9),
    "rtm_velocity_jacobian_d_": (_c_int, [_c_int] * 3 + [_P] * 9),
    "rtm_velocity_model_c_": (_c_int, [_c_int] * 2 + [_P] * 5),
    "rtm_velocity_model_d_": (_c_int, [_c_int] * 2 + [_P] * 5),
    "rtm_model_c_": (_c_int, [_c_int] * 3 + [_c_float] * 2 + [_c_int] * 3 + [_c_float] + [_c_int] * 2 + [_P] * 8),
    "rtm_born_migrate_c_": (_c_int, [_c_int] * 3 + [_c_float] * 2 + [_c_int] * 3 + [_c_float] + [_c_int] * 3
                            + [_P] * 3 + [_c_int] + [_P] * 4 + [_c_int]),
    "rtm_lsrtm_c_": (_c_int, [_c_int] * 3 + [_c_float] * 3 + [_c_int] * 3 + [_P, _P, _c_int, _c_int] + [_P] * 4
                     + [_c_int, _P, _P]),
    "rtm_lsrtm_d_": (_c_int, [_c_int] * 3 + [_c_double] * 3 + [_c_int] * 3 + [_P, _P, _c_int, _c_int] + [_P] * 4
                     + [_c_int, _P, _P]),
    "unet_create": (ctypes.c_void_p, [_c_int, _c_int, _c_int, ctypes.c_uint]),
    "unet_destroy": (None, [_P]),
    "unet_num_params": (ctypes.c_longlong, [_P]),
    "unet_layer_info": (_c_int, [_P, _c_int, _P]),
    "unet_get_params": (_c_int, [_P, _P]),
    "unet_set_params": (_c_int, [_P, _P]),
    "unet_set_gemm": (_c_int, [_c_int]),
    "unet_forward": (_c_int, [_P, _P, _c_int, _P, _c_int]),
    "unet_loss_grad": (_c_int, [_P, _P, _P, _c_int, _c_int, _P, _P]),
    "unet_train_step": (_c_int, [_P, _P, _P, _c_int, _c_int, _c_float, _c_float, _c_float, _c_float, _P]),
    "rtm_batch_create": (ctypes.c_void_p, [_c_int, _c_int, _c_int, _c_float, _c_float, _c_float, _c_int, _c_int]
                         + [_P] * 3 + [_c_int] + [_P] * 5 + [_c_int, _c_int, _c_int]),
    "rtm_batch_migrate": (_c_int, [_P, _c_int, _c_int, _P, _c_int, _P, _c_int]),
    "rtm_batch_stats": (_c_int, [_P, _P]),
    "rtm_batch_autotune": (_c_int, [_P, _c_int, _c_int, _c_int]),
    "rtm_batch_set": (_c_int, [_P, _c_int, _c_int]),
    "rtm_batch_set_checkpoint": (_c_int, [_P, _c_int]),
    "rtm_batch_set_tma": (_c_int, [_P, _c_int]),
    "rtm_batch_set_march": (_c_int, [_P, _c_int]),
    "rtm_batch_set_test_stall": (_c_int, [_P, _c_int]),
    "rtm_debug_march_plan": (_c_int, [_c_int, _P, _c_int, _c_int, _P, _c_int, _P]),
    "rtm_batch_set_stages": (_c_int, [_P, _c_int, _c_int, _c_int, _c_int]),
    "rtm_batch_destroy": (None, [_P]),
    "rtm_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "rtm_host_free": (None, [_P]),
    "acoustic3d_fwd_c_": (_c_int, [_c_int] * 4 + [_c_float] * 3 + [_P, _c_int, _c_float, _c_int, _c_int, _c_int, _P,
                                   _c_int, _P, _P, _P, _c_int, _P]),
    "acoustic3d_rtm_c_": (_c_int, [_c_int] * 4 + [_c_float] * 3 + [_P, _c_int, _c_float, _c_int, _c_int, _c_int, _P,
                                   _c_int, _P, _c_int, _P, _c_int, _P]),
    "acoustic3d_set": (_c_int, [_c_int, _c_int]),
    "acoustic3d_set_kernel": (_c_int, [_c_int]),
    "rtm3d_gpu_init": (None, [_c_int] * 3),
    "rtm3d_gpu_func": (None, [_c_int] * 3 + [_P] * 35),
    "rtm3d_gpu_final": (None, []),
    "rtm3d_set_exact": (_c_int, [_c_int]),
    "rtm3d_set_kernel": (_c_int, [_c_int]),
    "rtm3d_step_dev": (_c_int, [_c_int] * 3 + [_P] * 4 + [_c_int]),
    "pml_born_c_": (_c_int, [_c_int] * 3 + [_c_float] * 2 + [_c_int] * 3 + [_c_float] + [_c_int] * 6 + [_P] * 8),
    "pml_born_dev": (_c_int, [_c_int] * 3 + [_c_float] * 2 + [_c_int] * 3 + [_c_float] + [_c_int] * 6 + [_P] * 4),
    "pml_born_launches": (ctypes.c_longlong, []),
    "pml_set_kernel": (_c_int, [_c_int]),
    "pml_set_test_stall": (_c_int, [_c_int]),
    "rtm_debug_umma_desc": (_c_int, [_c_int, _c_int, _c_int, _c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.c_uint, _P]),
    "rtm_debug_umma_probe": (_c_int, [_c_int, ctypes.c_uint, ctypes.c_uint, _P, _P, _P]),
    "rtm_debug_umma_probe_sw": (_c_int, [_c_int, _c_int, _P, _P, _P]),
    "rtm_debug_umma_probe2": (_c_int, [_c_int] * 5 + [ctypes.c_uint, ctypes.c_uint, _P, _P, _P]),
}

_lib = None


class RtmError(RuntimeError):
    pass


def load():
    """Load the CUDA library (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RtmError(f"{LIB_PATH} is missing: build it with elastic_gb300.build.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ptr(a):
    """Pointer to a C-contiguous numpy array (or a torch tensor's data_ptr)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data_as(ctypes.c_void_p)
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported array type {type(a)}")


def check(status):
    """Raise RtmError for a non-zero status of an int-returning entry point."""
    if status != 0:
        msg = load().rtm_last_error().decode(errors="replace")
        raise RtmError(f"status {status}: {msg}")
    return status


def check_void():
    """Raise RtmError when the last void drop-in call failed."""
    check(load().rtm_last_status())
