"""The GPU step of the reference's 3D elastic kernel test (rtm3d_* of the
C-ABI) against the oracle (bit for bit in exact arithmetic, which the
reference's own check pins, tests/test_k3_oracle.py), through the device
entry point and the reference-shaped drop-in; and the reference's own test
main run with its GPU hand-off served by this library."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from elastic_gb300 import elastic3d as E

pytestmark = pytest.mark.gpu

SIZES = [(7, 9, 13), (20, 33, 40), (16, 70, 100)]


def planes(ny, nx, nz, seed, halo_zero=True):
    rng = np.random.default_rng(seed)
    shape = (ny + 10, nx + 10, nz + 10)

    def one():
        a = rng.uniform(-1.0, 1.0, shape).astype(np.float32)
        if halo_zero:
            b = np.zeros(shape, np.float32)
            b[5:-5, 5:-5, 5:-5] = a[5:-5, 5:-5, 5:-5]
            a = b
        return a
    inp = [one() for _ in range(9)]
    in1 = [one() for _ in range(9)]
    out = [one() for _ in range(9)]
    m = [one() for _ in range(6)]
    return inp, in1, out, m


@pytest.fixture(params=list(E.KERNELS))
def kernel(request):
    E.set_kernel(request.param)
    yield request.param
    E.set_kernel()


@pytest.mark.parametrize("size", SIZES, ids=lambda s: "%dx%dx%d" % s)
@pytest.mark.parametrize("halo_zero", [True, False], ids=["zero_halo", "random_halo"])
def test_step_dev_exact_equals_oracle(size, halo_zero, kernel):
    import torch
    ny, nx, nz = size
    inp, in1, out, m = planes(ny, nx, nz, seed=ny * nx + nz, halo_zero=halo_zero)
    want = O.k3_step(inp, in1, [o.copy() for o in out], m)
    d = lambda L: [torch.from_numpy(a).cuda() for a in L]
    dout = d(out)
    E.step_dev(d(inp), d(in1), dout, d(m), exact=True)
    torch.cuda.synchronize()
    for k in range(9):
        np.testing.assert_array_equal(dout[k].cpu().numpy(), want[k], err_msg=E.FIELDS[k])


@pytest.mark.parametrize("size", SIZES[:2], ids=lambda s: "%dx%dx%d" % s)
def test_drop_in_exact_equals_oracle_and_fast_is_close(size):
    ny, nx, nz = size
    inp, in1, out, m = planes(ny, nx, nz, seed=7 + nz)
    want = O.k3_step(inp, in1, [o.copy() for o in out], m)
    got = [o.copy() for o in out]
    t = E.step(inp, in1, got, m, exact=True)
    assert np.all(t >= 0)
    for k in range(9):
        np.testing.assert_array_equal(got[k], want[k], err_msg=E.FIELDS[k])
    fast = [o.copy() for o in out]
    E.step(inp, in1, fast, m, exact=False)
    for k in range(9):
        e = np.linalg.norm(fast[k].astype(np.float64) - want[k]) / np.linalg.norm(want[k])
        assert e < 1e-6, (E.FIELDS[k], e)


def test_reference_test_main_passes_with_gpu_step():
    """kernel_3d_test's own main (200^3, its CPU step, func_check at 1e-13)
    with rtm_gpu_init/func/final renamed to this library's rtm3d_gpu_*."""
    root = O.ref_root()
    if not root or not os.path.isdir(os.path.join(root, "kernel_3d_test")):
        pytest.skip("reference sources not present")
    subprocess.run(["make", "-s", "-C", O.HERE, "k3gpu", "REFROOT=" + os.path.abspath(root)], check=True)
    err = O.k3_reference_check(binary=os.path.join(O.HERE, "_ref", "k3_check_gpu"))
    print(err[-800:])
    assert err.count("Check Okay") == 9
