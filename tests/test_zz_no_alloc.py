"""rtm_op3_dev_noalloc, the allocation-free entry point.

It serves callers that cannot allocate device memory where they migrate
(their own allocator owns the device heap, or an allocation there would
synchronise or fail): they pass device buffers, the library uses a fixed
scratch array.  This file is collected last on purpose, so that a run which
stops at the first failure has already run every other test.

The test calls the entry point through the C-ABI twice in a row (different
sizes and data, so the second call must not depend on what the first left
in the shared scratch) and compares each result with rtm_op3_c_, the
existing host-buffer entry point, in exact arithmetic: the outputs must be
bit-identical, the tolerance of every exact-mode parity test here.  A
third call, repeating the second (so no kernel is loaded for the first time
during it), must leave the device's free memory unchanged.
"""
import numpy as np
import pytest

from elastic_gb300 import rtm as R
from elastic_gb300._lib import check, load, ptr

pytestmark = pytest.mark.gpu


def _case(nz, nx, nt, seed):
    rng = np.random.default_rng(seed)
    C = [(0.05 * rng.standard_normal((nx, nz))).astype(np.float32) for _ in range(5)]
    H = [rng.standard_normal((nt, nx, nz)).astype(np.float32) for _ in range(5)]
    return C, H


def test_noalloc_matches_rtm_op3_c_on_two_calls():
    import torch

    lib = load()
    R.set_exact(True)
    for nz, nx, nt, seed in [(48, 60, 24, 1), (37, 29, 15, 2)]:
        C, H = _case(nz, nx, nt, seed)
        ref = [h.copy() for h in H]
        R.rtm_op3(nt, nz, nx, 1, *ref, *C)  # existing entry point, host buffers
        Hd = [torch.from_numpy(h).cuda() for h in H]
        Cd = [torch.from_numpy(c).cuda() for c in C]
        torch.cuda.synchronize()
        check(lib.rtm_op3_dev_noalloc(nt, nz, nx, *[ptr(t) for t in Hd], *[ptr(t) for t in Cd], None))
        for got, want in zip(Hd, ref):
            np.testing.assert_array_equal(got.cpu().numpy(), want)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    check(lib.rtm_op3_dev_noalloc(nt, nz, nx, *[ptr(t) for t in Hd], *[ptr(t) for t in Cd], None))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = load()
    z = np.zeros(4, np.float32)
    st = lib.rtm_op3_dev_noalloc(10, 1024, 1024, *[ptr(z)] * 10, None)
    assert st == 1
    assert b"exceeds the fixed scratch" in lib.rtm_last_error()
