"""The plain single-shot RTM case at full size, on the GPU, against the
reference's own Fortran path.

400 x 200 cells, dx = dz = 10 m, dt = 1 ms, nt = 2000, 40-cell sponge, 15 Hz
Ricker explosive source at (x, z) = (2000 m, 50 m), 400 receivers at
z = 50 m.  With the grid origin at 0 m these are the reference's 1-based
indices xsource = 201, zsource = zrec = 6 (row 5 would leave the Vz trace
identically zero: Vz is only updated from row 6 on, W/rtmlib-mod.f90 Az, Bz).
Three-layer smoothed migration model; the Born model is the 5% Gaussian blob
that the true model adds.  The Born data are recorded on all five
components; the RTM migrates the Vx and Vz gathers with the stress traces
zeroed.

The reference outputs come from executing the reference's Fortran modules
and its C recursion (tests/golden/make_golden_f90.py, ref90_config1.npz):
the Born gathers as SHA-256 digests of their float32 bytes, the images in
full, and the float64 oracle's images and relative errors.

Exact mode (the drop-ins' default) must reproduce the reference's bits;
fast mode must agree within 1e-5 relative L2.  Each output's relative L2
error against the float64 oracle is printed.
"""
import hashlib
import os

import numpy as np
import pytest

from elastic_gb300 import rtm as R

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RTOL_FAST = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def cfg():
    return dict(np.load(os.path.join(HERE, "golden", "ref90_config1.npz")))


def run(cfg, exact):
    nz, nx, nt, abc, zsrc, xsrc, zrec = (int(v) for v in cfg["geom"])
    dx, dt, fp = (float(v) for v in cfg["phys"])
    R.set_exact(exact)
    try:
        op = R.RtmOperator(nz, dx, nx, dx, dt, xsrc, zsrc, zrec, fp, nt, abc, cfg["rho"], cfg["lam"], cfg["mu"])
        dm = [np.array(x) for x in cfg["dm"]]
        born = [np.zeros((nx, nt), np.float32) for _ in range(5)]
        assert op.rtm_op(False, *dm, *born) == 0
        gathers = [born[0].copy(), born[1].copy()] + [np.zeros((nx, nt), np.float32) for _ in range(3)]
        img = [np.zeros((nx, nz), np.float32) for _ in range(3)]
        assert op.rtm_op(True, *img, *gathers) == 0
    finally:
        R.set_exact(True)
    return born, img


NAMES_D = ["Vx", "Vz", "sigmaxx", "sigmazz", "sigmaxz"]
NAMES_I = ["drho", "dlambda", "dmu"]


def test_config1_exact_equals_reference_fortran(cfg):
    born, img = run(cfg, exact=True)
    for k in range(5):
        assert digest(born[k]) == str(cfg["born_sha256"][k]), "Born %s differs from the reference" % NAMES_D[k]
        print("Born %-8s bit-identical to the reference; rel. L2 vs float64 oracle %.2e"
              % (NAMES_D[k], cfg["born_err_f64"][k]))
    assert float(np.abs(born[1]).max()) > 0, "the Vz trace must be recorded"
    for k in range(3):
        np.testing.assert_array_equal(img[k], cfg["image"][k], err_msg=NAMES_I[k])
        print("image %-8s bit-identical to the reference; rel. L2 vs float64 oracle %.2e"
              % (NAMES_I[k], rel_l2(img[k], cfg["image_f64"][k])))


def test_config1_fast_mode_within_tolerance(cfg):
    born_x, img_x = run(cfg, exact=True)
    born, img = run(cfg, exact=False)
    for k in range(2):
        e = rel_l2(born[k], born_x[k])
        print("Born %-8s fast vs reference rel. L2 %.2e" % (NAMES_D[k], e))
        assert e <= RTOL_FAST
    for k in range(3):
        e = rel_l2(img[k], cfg["image"][k])
        e64 = rel_l2(img[k], cfg["image_f64"][k])
        print("image %-8s fast vs reference rel. L2 %.2e; vs float64 oracle %.2e" % (NAMES_I[k], e, e64))
        assert e <= RTOL_FAST
