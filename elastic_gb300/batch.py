"""Batched multi-shot RTM (the C-ABI's rtm_batch_* entry points).

Shots sit on their own subgrids of a full model; groups of shots are migrated
together on the GPU (see csrc/batch.cu).  Traces and images may be host numpy
arrays or device tensors (anything with ``data_ptr()``).
"""
import ctypes

import numpy as np

from ._lib import RtmError, check, load, ptr


class BatchRTM:
    def __init__(self, nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, zsrc, zrec, comp_mask=3,
                 group_max=4, nsource=250, exact_adjoint=False):
        lib = load()
        self.nz, self.nx, self.nt = nz, nx, nt
        self.nxs = np.ascontiguousarray(nxs, np.int32)
        self.nshots = len(self.nxs)
        self.comp_mask = comp_mask
        self.ncomp = bin(comp_mask & 31).count("1")
        self.group_max = min(group_max, self.nshots)
        arrs = [np.ascontiguousarray(a, np.float32) for a in (rho, lam, mu)]
        ints = [np.ascontiguousarray(a, np.int32) for a in (x0, nxs, xsrc, zsrc, zrec)]
        self._keep = arrs + ints
        h = lib.rtm_batch_create(nz, nx, nt, dx, dt, fp, nsource, abc, *[ptr(a) for a in arrs], self.nshots,
                                 *[ptr(a) for a in ints], comp_mask, group_max, 1 if exact_adjoint else 0)
        if not h:
            raise RtmError(lib.rtm_last_error().decode())
        self.h = ctypes.c_void_p(h)

    def trace_count(self, s0, ns):
        """Number of floats of the traces of shots [s0, s0+ns)."""
        return int(self.ncomp * self.nt * self.nxs[s0:s0 + ns].sum())

    def groups(self):
        """Consecutive groups of at most group_max shots."""
        return [(s, min(self.group_max, self.nshots - s)) for s in range(0, self.nshots, self.group_max)]

    def migrate(self, shot0, nshot, traces, image, traces_on_device=False, image_on_device=False):
        check(load().rtm_batch_migrate(self.h, shot0, nshot, ptr(traces), int(traces_on_device), ptr(image),
                                       int(image_on_device)))

    def stats(self):
        out = np.zeros(48, np.float64)
        check(load().rtm_batch_stats(self.h, ptr(out)))
        return dict(fwd_ms=out[0], adj_ms=out[1], cells=int(out[2]), kernels=int(out[3]), total_ms=out[4],
                    tile_x=int(out[5]), work_items=int(out[6]), tile_x_adj=int(out[7]),
                    tune_ms_fwd=list(out[8:11]), tune_ms_adj=list(out[11:14]),
                    stages=int(out[14]), stages_adj=int(out[15]), threads=int(out[40]), threads_adj=int(out[41]),
                    checkpoint=int(out[42]), tma=bool(out[43]), march=bool(out[44]), tune_ms_march=out[45],
                    march_adj=bool(out[46]), tune_ms_march_adj=out[47],
                    # per tile width 8, 16, 32: [1 stage, 2 stages, 1 stage 512 threads, 2 stages 512 threads]
                    tune_ms_fwd_variants=[list(out[16 + 4 * i:20 + 4 * i]) for i in range(3)],
                    tune_ms_adj_variants=[list(out[28 + 4 * i:32 + 4 * i]) for i in range(3)])

    def autotune(self, shot0=0, nshot=None, steps=20):
        """Pick the fastest tile width per pass on the geometry of a group."""
        nshot = self.group_max if nshot is None else nshot
        check(load().rtm_batch_autotune(self.h, shot0, nshot, steps))
        return self.stats()

    def set_graph(self, use_graph, tile_x=0):
        check(load().rtm_batch_set(self.h, 1 if use_graph else 0, tile_x))
        self._graph = use_graph

    def set_tile(self, tile_x):
        check(load().rtm_batch_set(self.h, 1 if getattr(self, "_graph", True) else 0, tile_x))

    def set_stages(self, fwd, adj, threads_fwd=256, threads_adj=256):
        """Staging buffers per CTA (1 or 2) and threads per CTA (256, or 512
        at tile widths >= 16) of the forward and adjoint step."""
        check(load().rtm_batch_set_stages(self.h, fwd, adj, threads_fwd, threads_adj))

    def set_tma(self, on):
        """Stage the step kernels' tiles with tensor-memory-access loads."""
        check(load().rtm_batch_set_tma(self.h, int(bool(on))))

    def set_march(self, mode):
        """Passes by the marching kernels: -1 the autotuner's choice per pass
        (on until autotune has run), else a bit mask -- 1 forward, 2 adjoint
        (0: tile kernels for both)."""
        check(load().rtm_batch_set_march(self.h, int(mode)))

    def set_test_stall(self, on):
        """Test hook: make the next migrations' first forward marching launch
        wait on a flag that nothing sets, so they return status 4."""
        check(load().rtm_batch_set_test_stall(self.h, int(bool(on))))

    def set_checkpoint(self, interval):
        """0: keep every level's FP16 snapshots; k: checkpoint the forward
        state every k levels and recompute segments in the adjoint pass."""
        check(load().rtm_batch_set_checkpoint(self.h, interval))

    def close(self):
        if getattr(self, "h", None):
            load().rtm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
