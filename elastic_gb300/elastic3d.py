"""The 3D elastic kernel of the reference's kernel_3d_test
(rtm3d_* of include/elastic_rtm.h).

Planes are padded (ny+10, nx+10, nz+10) float32 arrays (z fastest), fields
in the order Vy, Vx, Vz, syy, sxx, szz, sxy, sxz, syz, coefficients m1_y,
m1_x, m1_z, m2, m3, m2m3.
"""
import ctypes

import numpy as np

from ._lib import check, load

FIELDS = ("vy", "vx", "vz", "syy", "sxx", "szz", "sxy", "sxz", "syz")
COEFS = ("m1y", "m1x", "m1z", "m2", "m3", "m2m3")


KERNELS = {"cell": 0, "paired": 1, "paired-prefetch": 3, "paired-bound": 5, "paired-prefetch-bound": 7}


def set_kernel(kind="paired-bound"):
    """Step kernel form (every form gives the same bits)."""
    check(load().rtm3d_set_kernel(KERNELS[kind]))


def _ptrs(arrs):
    P = ctypes.c_void_p * len(arrs)
    return P(*[(a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data) for a in arrs])


def step(inp, in1, out, m, exact=True):
    """One step through the reference-shaped drop-in (host planes; out is
    updated in place).  Returns {copy in, step, copy out} seconds."""
    L = load()
    ny, nx, nz = (d - 10 for d in out[0].shape)
    arrs = list(inp) + list(in1) + list(out) + list(m)
    for a in arrs:
        assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.shape == out[0].shape
    t = np.zeros(3, np.float32)
    check(L.rtm3d_set_exact(1 if exact else 0))
    L.rtm3d_gpu_init(ny, nz, nx)
    check(L.rtm_last_status())
    try:
        L.rtm3d_gpu_func(ny, nz, nx, *[a.ctypes.data_as(ctypes.c_void_p) for a in arrs], None,
                         t.ctypes.data_as(ctypes.c_void_p))
        check(L.rtm_last_status())
    finally:
        L.rtm3d_gpu_final()
    return t


def step_dev(inp, in1, out, m, exact=True):
    """One step on device tensors (torch, float32, contiguous, padded)."""
    ny, nx, nz = (d - 10 for d in out[0].shape)
    check(load().rtm3d_step_dev(ny, nz, nx, _ptrs(inp), _ptrs(in1), _ptrs(out), _ptrs(m), 1 if exact else 0))
