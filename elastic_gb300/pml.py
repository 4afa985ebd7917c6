"""Split-field PML Born modelling (pml_born_* of include/elastic_rtm.h).

The reference's working_Src/born.f90 program: background and scattered
(Born) elastic wavefields with a split-field PML, Ricker source, receiver
lines and snapshots, bit-identical to the reference's CPU execution.

Model planes are float32 [nx, nz] arrays (the Fortran (nz, nx) layout, z
fastest); grid indices are 1-based as in the reference.
"""
import ctypes

import numpy as np

from ._lib import check, load

SEIS = ("Vx", "Vz", "P", "Vx_b", "Vz_b", "P_b")


def params(dx, Tt, fp=25.0, dtseis=0.002):
    """nt, dt, nsource, nseis as the reference's main program derives them
    from the grid step, the propagation time Ttime, the peak frequency and
    the trace sampling (working_Src/born.f90:67-73, 251, 255)."""
    F = np.float32
    dt = F(F(F(0.2) * F(dx)) / F(F(np.sqrt(F(2.0))) * F(2000.0)))
    x = F(F(F(F(np.sqrt(F(6.0))) / F(3.14159265)) / F(fp)) / dt)
    return {"nt": int(F(F(Tt) / dt)), "dt": float(dt), "nsource": 4 * int(np.floor(x + 0.5)),
            "nseis": int(F(F(Tt) / F(dtseis)) + F(1))}


def _addr(a):
    return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[_addr(a) for a in arrs])


def born(vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource, nsource, fp, nsnap, nseis, abc, zrec,
         free_surface=False, lame=False):
    """elastic_init + elastic_op on host arrays.  Returns (seis, snap): six
    receiver lines [nx-2abc, nseis] (Vx, Vz, P, Vx_b, Vz_b, P_b) and six
    snapshot cubes [nsnap, nx, nz]."""
    L = load()
    nx, nz = vp0.shape
    m = [np.ascontiguousarray(x, np.float32) for x in (vp0, vs0, rho0, dvp, dvs, drho)]
    for x in m:
        if x.shape != (nx, nz):
            raise ValueError("model planes must share one [nx, nz] shape")
    seis = [np.zeros((nx - 2 * abc, nseis), np.float32) for _ in range(6)]
    snap = [np.zeros((nsnap, nx, nz), np.float32) for _ in range(6)]
    F = ctypes.c_float
    check(L.pml_born_c_(nz, nx, nt, F(dx), F(dt), xsource, zsource, nsource, F(fp), nsnap, nseis, abc, zrec,
                        int(free_surface), int(lame), *[x.ctypes.data_as(ctypes.c_void_p) for x in m],
                        _ptrs(seis), _ptrs(snap)))
    return seis, snap


def born_dev(model, seis, snap, dx, dt, nt, xsource, zsource, nsource, fp, abc, zrec, free_surface=False,
             lame=False, stream=None):
    """The same on device tensors (torch, float32, contiguous): model = six
    [nx, nz] planes (vp0, vs0, rho0, dvp, dvs, drho); seis six
    [nx-2abc, nseis], snap six [nsnap, nx, nz] tensors, overwritten.  Work is
    queued on `stream` (a torch.cuda.Stream, default: the current one)."""
    nx, nz = model[0].shape
    nseis, nsnap = seis[0].shape[1], snap[0].shape[0]
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    F = ctypes.c_float
    check(load().pml_born_dev(nz, nx, nt, F(dx), F(dt), xsource, zsource, nsource, F(fp), nsnap, nseis, abc, zrec,
                              int(free_surface), int(lame), _ptrs(model), _ptrs(seis), _ptrs(snap),
                              ctypes.c_void_p(stream.cuda_stream)))


KERNELS = {"rows4": 0, "cell": 1, "rows4-prefetch": 2, "cell-prefetch": 3, "tile": 4, "tile-prefetch": 6,
           "cell-prefetch-b5": 3 + 5 * 16, "cell-prefetch-b6": 3 + 6 * 16, "cell-prefetch-b8": 3 + 8 * 16,
           "fused": 8}


def set_kernel(kind="cell-prefetch-b6"):
    """Step kernel form (every form gives the same bits): tiles staged by
    bulk tensor copies, four rows per thread, or one cell per thread; with or
    without an L2 prefetch of each thread's first-touch lines."""
    check(load().pml_set_kernel(KERNELS[kind]))


def set_test_stall(on):
    """Test hook: the staged-tile form's first launch waits on a flag that
    nothing sets and the call returns status 4 (see pml_set_test_stall)."""
    check(load().pml_set_test_stall(1 if on else 0))


def launches():
    """Kernels launched by the last call."""
    return int(load().pml_born_launches())
