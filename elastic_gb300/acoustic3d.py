"""3D acoustic 10th-order propagator and 3D RTM with reverse-time restart
(C-ABI acoustic3d_* of include/elastic_rtm.h).

Volumes are numpy arrays (or device tensors with on_device=True) shaped
[n3, n2, n1] (y, x, z; z fastest).  Positions are 1-based (z, x, y).
"""
import numpy as np

from ._lib import check, load, ptr

F32 = np.float32


def set_shape(tile_x=16, ychunks=0):
    check(load().acoustic3d_set(tile_x, ychunks))


KERNELS = {"slab": 0, "ring": 1, "pipelined": 2, "slab-paired": 3}


def set_kernel(kind="slab"):
    """Step kernel for n1 % 4 == 0: "slab" (default: every operand by bulk
    tensor copies issued slices ahead, y taps from an unrolled register
    queue), "slab-paired" (the same with paired FP32 instructions in fast
    arithmetic), "ring" (every tap from a ring of copied slices) or
    "pipelined" (cp.async halo, shifted register queue)."""
    check(load().acoustic3d_set_kernel(KERNELS[kind]))


def forward(vel2, d, damp_a, damp_b, src, wavelet, zr, record=True, on_device=False):
    """Returns (traces [nt, n3, n2] or None, level nt-2, level nt-1, device ms)."""
    n3, n2, n1 = vel2.shape
    nt = len(wavelet)
    w = np.ascontiguousarray(wavelet, F32)
    if on_device:
        import torch
        dev = vel2.device
        data = torch.zeros((nt, n3, n2), dtype=torch.float32, device=dev) if record else None
        l0 = torch.zeros_like(vel2)
        l1 = torch.zeros_like(vel2)
    else:
        vel2 = np.ascontiguousarray(vel2, F32)
        data = np.zeros((nt, n3, n2), F32) if record else None
        l0, l1 = np.zeros_like(vel2), np.zeros_like(vel2)
    ms = np.zeros(1, np.float64)
    zs, xs, ys = src
    check(load().acoustic3d_fwd_c_(n1, n2, n3, nt, d[0], d[1], d[2], ptr(vel2), damp_a, damp_b, zs, xs, ys, ptr(w),
                                   zr if record else 0, ptr(data), ptr(l0), ptr(l1), int(on_device), ptr(ms)))
    return data, l0, l1, float(ms[0])


def rtm(vel2, d, damp_a, damp_b, src, wavelet, zr, traces, jt=1, on_device=False):
    """Image of the traces [nt, n3, n2]; returns (image, device ms)."""
    n3, n2, n1 = vel2.shape
    nt = len(wavelet)
    w = np.ascontiguousarray(wavelet, F32)
    if on_device:
        import torch
        img = torch.zeros_like(vel2)
    else:
        vel2 = np.ascontiguousarray(vel2, F32)
        traces = np.ascontiguousarray(traces, F32)
        img = np.zeros_like(vel2)
    ms = np.zeros(1, np.float64)
    zs, xs, ys = src
    check(load().acoustic3d_rtm_c_(n1, n2, n3, nt, d[0], d[1], d[2], ptr(vel2), damp_a, damp_b, zs, xs, ys, ptr(w), zr,
                                   ptr(traces), jt, ptr(img), int(on_device), ptr(ms)))
    return img, float(ms[0])
