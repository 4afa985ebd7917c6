"""LSRTM (CGLS on the linear Born operator with its exact adjoint) on the
GPU against a CGLS written here over the oracle's FP64 operators."""
import numpy as np
import pytest

import oracle as O
from elastic_gb300 import rtm as R
from elastic_gb300 import synth

pytestmark = pytest.mark.gpu

NZ, NX, NT, DX, DT, FP, ABC, NS, ZREC = 40, 48, 150, 10.0, 1e-3, 25.0, 10, 40, 5
XSRC, ZSRC = np.array([15, 34], np.int32), np.array([5, 6], np.int32)


def model():
    vp = synth.smooth_random_model(NZ, NX, DX, 60.0, 2000.0, 3000.0, seed=11)
    return [np.ascontiguousarray(a, np.float64) for a in synth.lame_from_vp(vp)]


def L(rho, lam, mu, m):
    """Linear Born data of all shots, FP64 oracle (rtm_op2, exact=True)."""
    zero_d = [np.zeros((NX, NT)) for _ in range(5)]
    return np.stack([np.stack(O.rtm_op2(False, rho, lam, mu, list(m), zero_d, DX, DT, NT, int(ZSRC[s]), int(XSRC[s]),
                                        ZREC, FP, ABC, NS, exact=True)[1]) for s in range(len(XSRC))])


def LT(rho, lam, mu, d):
    """Exact adjoint of L summed over shots, FP64 oracle."""
    zero_m = [np.zeros((NX, NZ)) for _ in range(3)]
    out = np.zeros((3, NX, NZ))
    for s in range(len(XSRC)):
        out += np.stack(O.rtm_op2(True, rho, lam, mu, zero_m, list(d[s]), DX, DT, NT, int(ZSRC[s]), int(XSRC[s]),
                                  ZREC, FP, ABC, NS, exact=True)[0])
    return out


def problem(dtype):
    """Born data of a Gaussian density perturbation plus 5% seeded noise.
    (The Lame parameters are ~1e9 times larger than the density, so unscaled
    CGLS only makes progress on a density-dominated residual.)"""
    rho, lam, mu = model()
    ix, iz = np.meshgrid(np.arange(NX), np.arange(NZ), indexing="ij")
    blob = np.exp(-((ix - 24.0) ** 2 + (iz - 22.0) ** 2) / 20.0)
    m_true = [0.05 * rho * blob, np.zeros_like(lam), np.zeros_like(mu)]
    d = L(rho, lam, mu, m_true)
    rng = np.random.default_rng(12)
    d = d + 0.05 * np.std(d) * rng.standard_normal(d.shape)
    return [np.ascontiguousarray(a, dtype) for a in (rho, lam, mu)] + [np.ascontiguousarray(d, dtype)]


def oracle_cgls(rho, lam, mu, data, niter):
    """CGLS for min ||L m - d|| over all shots with the FP64 oracle
    operators."""
    rho, lam, mu = (np.asarray(a, np.float64) for a in (rho, lam, mu))

    x = np.zeros((3, NX, NZ))
    r = data.astype(np.float64).copy()
    resid = [np.linalg.norm(r)]
    s = LT(rho, lam, mu, r)
    p = s.copy()
    gamma = np.vdot(s, s)
    for _ in range(niter):
        q = L(rho, lam, mu, p)
        alpha = gamma / np.vdot(q, q)
        x += alpha * p
        r -= alpha * q
        resid.append(np.linalg.norm(r))
        s = LT(rho, lam, mu, r)
        gnew = np.vdot(s, s)
        p = s + (gnew / gamma) * p
        gamma = gnew
    return x, np.array(resid)


@pytest.fixture(scope="module")
def reference():
    rho, lam, mu, data = problem(np.float64)
    return oracle_cgls(rho, lam, mu, data, 4)


def rel_errs(dm, x_ref):
    return [float(np.linalg.norm(dm[i].astype(np.float64) - x_ref[i]) / np.linalg.norm(x_ref[i])) for i in range(3)]


def test_lsrtm_fp64_matches_oracle_cgls(reference):
    x_ref, r_ref = reference
    rho, lam, mu, data = problem(np.float64)
    dm, resid = R.lsrtm(rho, lam, mu, data, XSRC, ZSRC, ZREC, DX, DT, NT, FP, ABC, niter=4, nsource=NS,
                        dtype=np.float64)
    errs = rel_errs(dm, x_ref)
    print("fp64 LSRTM vs oracle CGLS: model rel err per parameter", errs, "resid", resid, r_ref)
    np.testing.assert_allclose(resid, r_ref, rtol=1e-9)
    assert max(errs) < 1e-8
    assert np.all(np.diff(resid) < 0)


def test_lsrtm_fp32_close_to_fp64_oracle(reference):
    x_ref, r_ref = reference
    rho, lam, mu, data = problem(np.float32)
    dm, resid = R.lsrtm(rho, lam, mu, data, XSRC, ZSRC, ZREC, DX, DT, NT, FP, ABC, niter=4, nsource=NS)
    errs = rel_errs(dm, x_ref)
    print("fp32 LSRTM vs FP64 oracle CGLS: model rel err per parameter", errs, "resid", resid, r_ref)
    # float32 operators (rounding ~1e-7 per operation over nt steps) and CG's
    # sensitivity to them: each parameter agrees to this relative L2
    assert max(errs) < 2e-3
    np.testing.assert_allclose(resid, r_ref, rtol=1e-3)


def test_lsrtm_zero_iterations_and_zero_data():
    rho, lam, mu, data = problem(np.float32)
    dm, resid = R.lsrtm(rho, lam, mu, data, XSRC, ZSRC, ZREC, DX, DT, NT, FP, ABC, niter=0, nsource=NS)
    assert not dm.any()
    assert resid[0] == pytest.approx(np.linalg.norm(data.astype(np.float64)), rel=1e-6)
    dm, resid = R.lsrtm(rho, lam, mu, np.zeros_like(data), XSRC, ZSRC, ZREC, DX, DT, NT, FP, ABC, niter=3,
                        nsource=NS)
    assert not dm.any() and not resid.any()
