"""GPU parity of the 2D elastic path: every entry point of the C-ABI against
the oracle on the same seeded inputs.  Exact mode must be bit-identical to the
oracle (which is itself bit-identical to the reference C where the reference
can be run); fast mode must agree to 1e-5 relative L2 (the tolerance of the
project's parity bar)."""
import os

import numpy as np
import pytest

import oracle as O
from elastic_gb300 import rtm as R
from elastic_gb300._lib import load

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RTOL_FAST = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def model(nz, nx, seed=0, dtype=np.float32):
    """Three-layer model with a Gaussian blob: Vp 2000/2800/3500, Vs=Vp/1.73,
    Gardner density."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :]
    vp = np.where(z < nz // 3, 2000.0, np.where(z < 2 * nz // 3, 2800.0, 3500.0)) * np.ones((nx, 1))
    xx, zz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    vp *= 1 + 0.05 * np.exp(-((xx - nx * rng.uniform(0.3, 0.7)) ** 2 + (zz - nz / 2) ** 2) / (2 * (nz / 8) ** 2))
    vs = vp / 1.73
    rho = 310.0 * vp ** 0.25
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    return rho.astype(dtype), lam.astype(dtype), mu.astype(dtype)


@pytest.fixture(autouse=True, params=[1, 2], ids=["v1", "v2"])
def exact_mode(request):
    """Every test runs with both step-kernel generations (v2 applies where the
    planes are 16-byte aligned, e.g. nz % 4 == 0; elsewhere both run v1)."""
    R.set_exact(True)
    R.set_kernel_version(request.param)
    yield
    R.set_exact(True)
    R.set_kernel_version(0)


def test_rtm_op3_c_matches_reference_golden_vectors():
    g = np.load(os.path.join(HERE, "golden", "rtm_op3_c_ref.npz"))
    nf, nt, nx, nz = g["hin"].shape
    H = [np.ascontiguousarray(h) for h in g["hin"]]
    C = [np.ascontiguousarray(c) for c in g["coefs"]]
    R.rtm_op3(nt, nz, nx, 1, *H, *C)
    for a, b in zip(H, g["hout"]):
        np.testing.assert_array_equal(a, b)


def test_rtm_op3_c_matches_reference_digests_at_several_sizes():
    """rtm_op3_c_ on the GPU reproduces the reference's output bit for bit on
    an odd grid, one and a half 128-row strips over several column tiles,
    and the single-shot grid (200 x 400) over 60 levels (inputs from
    tests/golden/detgen.py, digests from the reference, make_golden.py)."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import detgen
    from make_golden import sizes_inputs
    g = np.load(os.path.join(HERE, "golden", "rtm_op3_c_sizes.npz"))
    for key in g.files:
        nz, nx, nt = (int(v) for v in key.split("x"))
        coefs, H = sizes_inputs(nz, nx, nt)
        R.rtm_op3(nt, nz, nx, 1, *H, *coefs)
        assert detgen.digest(H) == str(g[key]), key


@pytest.mark.parametrize("nz,nx,nt", [(37, 45, 20), (11, 13, 9), (64, 48, 12), (70, 33, 7)])
def test_rtm_op3_c_exact_random(nz, nx, nt):
    rng = np.random.default_rng(nz + nx)
    C = [(0.05 * rng.standard_normal((nx, nz))).astype(np.float32) for _ in range(5)]
    H = [rng.standard_normal((nt, nx, nz)).astype(np.float32) for _ in range(5)]
    ref = [h.copy() for h in H]
    O.rtm_op3_c(ref, C)
    R.rtm_op3(nt, nz, nx, 1, *H, *C)
    for a, b in zip(H, ref):
        np.testing.assert_array_equal(a, b)


def test_rtm_op3_c_fast_mode_tolerance():
    nz, nx, nt = 60, 70, 40
    rng = np.random.default_rng(5)
    C = [(0.05 + 0.02 * rng.random((nx, nz))).astype(np.float32) for _ in range(5)]
    H = [rng.standard_normal((nt, nx, nz)).astype(np.float32) for _ in range(5)]
    ref = [h.copy() for h in H]
    O.rtm_op3_c(ref, C)
    R.set_exact(False)
    R.rtm_op3(nt, nz, nx, 1, *H, *C)
    for a, b in zip(H, ref):
        assert rel_l2(a, b) < RTOL_FAST


def _pad(a, nz, nx, nt=None):
    """The reference's padded layout: (nz+10,nx+10[,nt+10]) with +5 offsets."""
    if nt is None:
        out = np.zeros((nx + 10, nz + 10), np.float32)
        out[5:5 + nx, 5:5 + nz] = a
    else:
        out = np.zeros((nt + 10, nx + 10, nz + 10), np.float32)
        out[5:5 + nt, 5:5 + nx, 5:5 + nz] = a
    return out


def _masked(C, nz, nx):
    m = [np.zeros_like(c) for c in C]
    m[0][5:nx - 5, 4:nz - 5] = C[0][5:nx - 5, 4:nz - 5]   # m1_x
    m[1][4:nx - 5, 5:nz - 5] = C[1][4:nx - 5, 5:nz - 5]   # m1_z
    m[2][4:nx - 5, 4:nz - 5] = C[2][4:nx - 5, 4:nz - 5]   # aux_m2
    m[3][5:nx - 5, 5:nz - 5] = C[3][5:nx - 5, 5:nz - 5]   # aux_m3
    m[4][4:nx - 5, 4:nz - 5] = C[4][4:nx - 5, 4:nz - 5]   # aux_m2m3
    return m


def test_rtm_gpu_func_internal_layer():
    """The reference's C->CUDA layer: levels nt-3..nt-9 by the C loop, the
    rest by rtm_gpu_func on padded arrays (W/rtmlib-modC.c:120-279)."""
    nz, nx, nt = 40, 60, 30
    rng = np.random.default_rng(11)
    C = [(0.05 * rng.standard_normal((nx, nz))).astype(np.float32) for _ in range(5)]
    H = [rng.standard_normal((nt, nx, nz)).astype(np.float32) for _ in range(5)]
    full = [h.copy() for h in H]
    O.rtm_op3_c(full, C)
    # emulate the C part: levels nt-3 .. nt-9 from the oracle (3-level windows)
    part = [h.copy() for h in H]
    for it in range(nt - 3, nt - 10, -1):
        w = [p[it:it + 3].copy() for p in part]
        O.rtm_op3_c(w, C)
        for f in range(5):
            part[f][it] = w[f][0]
    P = [_pad(p, nz, nx, nt) for p in part]
    M = [_pad(m, nz, nx) for m in _masked(C, nz, nx)]
    lib = load()
    from elastic_gb300._lib import ptr, check_void
    import ctypes
    tps = np.zeros(1, np.float64)
    lib.rtm_gpu_init(nt, nz, nx)
    check_void()
    lib.rtm_gpu_func(nt - 10, nt, nz, nx, *[ptr(p) for p in P], *[ptr(m) for m in M], None, ptr(tps))
    check_void()
    lib.rtm_gpu_final()
    for f in range(5):
        np.testing.assert_array_equal(P[f][5:5 + nt, 5:5 + nx, 5:5 + nz], full[f])
    assert tps[0] > 0


def test_model_op_exact():
    nz, nx = 50, 61
    rho, lam, mu = model(nz, nx, 1)
    mu[3:7, 10:12] = 0.0  # liquid patch exercises the mu==0 branch
    got = R.model_op(rho, lam, mu, 10.0, 1e-3)
    m1x, m1z, m2, m3 = O.model_op(rho, lam, mu)
    ref = O.rtmmod_init(m1x, m1z, m2, m3, np.float32(10.0), np.float32(1e-3))
    for a, b in zip(got[:5], ref):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(got[5], m2)
    np.testing.assert_array_equal(got[6], m3)


def _setup(nz, nx, nt, abc, seed=0):
    rho, lam, mu = model(nz, nx, seed)
    coefs = list(O.coefficients(rho, lam, mu, np.float32(10.0), np.float32(1e-3)))
    return rho, lam, mu, coefs


@pytest.mark.parametrize("nz,nx,nt,abc", [(60, 80, 120, 12), (45, 37, 60, 20), (90, 50, 40, 40)])
def test_forward_history_exact(nz, nx, nt, abc):
    rho, lam, mu, coefs = _setup(nz, nx, nt, abc)
    src = O.source_op2(nt, np.float32(1e-3), np.float32(40.0), 40)
    filt = O.abc_init(abc)
    ref = O.forward(coefs, nt, np.float32(1e-3), 6, nx // 2, src, abc, filt)
    got = R.forward(coefs, nt, 1e-3, nx // 2, 6, abc, src)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
    assert np.abs(ref[0]).max() > 0


def test_image_init_and_image_op_exact():
    nz, nx, nt, abc = 40, 52, 50, 10
    rho, lam, mu, coefs = _setup(nz, nx, nt, abc)
    src = O.source_op2(nt, np.float32(1e-3), np.float32(40.0), 30)
    H = O.forward(coefs, nt, np.float32(1e-3), 6, 20, src, abc, O.abc_init(abc))
    S_ref = O.image_init(H[0], H[1], np.float32(10.0), np.float32(1e-3))
    S = R.image_init(H[0], H[1], 10.0, 1e-3)
    for a, b in zip(S, S_ref):
        np.testing.assert_array_equal(a, b)
    rng = np.random.default_rng(2)
    dm = [rng.standard_normal((nx, nz)).astype(np.float32) for _ in range(3)]
    np.testing.assert_array_equal(np.stack(R.image_op2(False, S, images=dm)), np.stack(O.image_fwd(*dm, S_ref)))
    A = [rng.standard_normal((nt, nx, nz)).astype(np.float32) for _ in range(5)]
    np.testing.assert_array_equal(np.stack(R.image_op2(True, S, H=A)), np.stack(O.image_adj(A, S_ref)))


def test_model_delta_exact():
    nz, nx = 30, 33
    rng = np.random.default_rng(9)
    d1 = rng.uniform(-1, 1, (nx, nz)).astype(np.float32)
    d2 = rng.uniform(-0.01, 1, (nx, nz)).astype(np.float32)
    d3 = rng.uniform(-0.01, 1, (nx, nz)).astype(np.float32)
    got = R.model_delta(d1, d2, d3)
    ref = O.model_delta(d1, d2, d3)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def test_born_scatter_exact():
    nz, nx, nt, abc = 40, 48, 60, 10
    rho, lam, mu, coefs = _setup(nz, nx, nt, abc)
    rng = np.random.default_rng(4)
    H = [rng.standard_normal((nt, nx, nz)).astype(np.float32) * 1e-3 for _ in range(5)]
    Href = [h.copy() for h in H]
    Dref = O.born_scatter(Href, coefs, 7, abc, O.abc_init(abc))
    Hg, D = R.born_scatter(H, coefs, 7, abc)
    for a, b in zip(Hg, Href):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(D, Dref):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("exact_adjoint", [False, True])
def test_rtm_op3_full_exact(exact_adjoint):
    nz, nx, nt, abc = 36, 44, 70, 10
    rho, lam, mu, coefs = _setup(nz, nx, nt, abc)
    rng = np.random.default_rng(8)
    D = [rng.standard_normal((nx, nt)).astype(np.float32) for _ in range(5)]
    ref = O.rtm_op3(D, coefs, nz, 6, exact=exact_adjoint, abc=abc)
    got = R.rtm_op3_full(D, coefs, nz, 6, abc=abc, exact_adjoint=exact_adjoint)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def _op(adj, nz, nx, nt, abc, dm, D, dtype=np.float32, linear=False, exact_adjoint=False):
    rho, lam, mu = model(nz, nx, 3, dtype)
    op = R.RtmOperator(nz, 10.0, nx, 10.0, 1e-3, nx // 2, 6, 6, 40.0, nt, abc, rho, lam, mu, nsource=40,
                       dtype=dtype, linear=linear, exact_adjoint=exact_adjoint)
    dm = [np.array(x, dtype) for x in dm]  # fresh arrays: outputs are written in place
    D = [np.array(x, dtype) for x in D]
    assert op.rtm_op(adj, *dm, *D) == 0
    return rho, lam, mu, dm, D


def test_rtm_op_rtm_exact():
    nz, nx, nt, abc = 40, 56, 90, 12
    rng = np.random.default_rng(12)
    D = [rng.standard_normal((nx, nt)).astype(np.float32) for _ in range(5)]
    dm0 = [np.zeros((nx, nz), np.float32) for _ in range(3)]
    rho, lam, mu, dm, _ = _op(True, nz, nx, nt, abc, dm0, D)
    ref, _ = O.rtm_op2(True, rho, lam, mu, dm0, D, np.float32(10.0), np.float32(1e-3), nt, 6, nx // 2, 6,
                       np.float32(40.0), abc, 40)
    for a, b in zip(dm, ref):
        np.testing.assert_array_equal(a, b)
    assert np.abs(ref[0]).max() > 0


def test_rtm_op_born_exact():
    nz, nx, nt, abc = 40, 56, 90, 12
    rng = np.random.default_rng(13)
    dm_in = [rng.uniform(0.0, 0.2, (nx, nz)).astype(np.float32) for _ in range(3)]
    D0 = [np.zeros((nx, nt), np.float32) for _ in range(5)]
    rho, lam, mu, dm, D = _op(False, nz, nx, nt, abc, dm_in, D0)
    ref_dm, ref_D = O.rtm_op2(False, rho, lam, mu, dm_in, D0, np.float32(10.0), np.float32(1e-3), nt, 6, nx // 2, 6,
                              np.float32(40.0), abc, 40)
    for a, b in zip(D, ref_D):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(dm, ref_dm):  # dlambda/dmu averaged in place as in the reference
        np.testing.assert_array_equal(a, b)


def test_fp64_dot_product_gpu():
    """Adjoint dot-product test of the linear Born operator and its exact
    (sponged) adjoint, both on the GPU in FP64: holds to 1e-6 (observed
    ~1e-13)."""
    nz, nx, nt, abc = 40, 48, 80, 12
    rng = np.random.default_rng(21)
    m = [rng.standard_normal((nx, nz)) for _ in range(3)]
    d = [rng.standard_normal((nx, nt)) for _ in range(5)]
    _, _, _, _, Lm = _op(False, nz, nx, nt, abc, m, [np.zeros((nx, nt))] * 5, np.float64, linear=True)
    _, _, _, Ltd, _ = _op(True, nz, nx, nt, abc, [np.zeros((nx, nz))] * 3, d, np.float64, exact_adjoint=True)
    lhs = sum(float(np.vdot(a, b)) for a, b in zip(Lm, d))
    rhs = sum(float(np.vdot(a, b)) for a, b in zip(m, Ltd))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_rtm_op_matches_reference_fortran_fixtures():
    """Born gathers and RTM images through the drop-in rtm_op_c_ equal the
    reference's own Fortran path (translated and executed, fixtures from
    tests/golden/make_golden_f90.py) bit for bit: an odd grid and one that
    crosses the kernels' 128-row strips and several column tiles."""
    g = np.load(os.path.join(HERE, "golden", "ref90_small.npz"))
    for name in sorted({k.split("/")[0] for k in g.files}):
        p = {k.split("/")[1]: g[k] for k in g.files if k.startswith(name + "/")}
        nz, nx, nt, abc, zsrc, xsrc, zrec = (int(v) for v in p["geom"])
        dx, dt, fp = (float(v) for v in p["phys"])
        op = R.RtmOperator(nz, dx, nx, dx, dt, xsrc, zsrc, zrec, fp, nt, abc, p["rho"], p["lam"], p["mu"])
        dm = [np.array(x) for x in p["dm"]]
        D = [np.zeros((nx, nt), np.float32) for _ in range(5)]
        assert op.rtm_op(False, *dm, *D) == 0
        np.testing.assert_array_equal(np.stack(D), p["born"], err_msg=name)
        img = [np.zeros((nx, nz), np.float32) for _ in range(3)]
        D = [np.array(x) for x in p["born"]]
        assert op.rtm_op(True, *img, *D) == 0
        np.testing.assert_array_equal(np.stack(img), p["image"], err_msg=name)
