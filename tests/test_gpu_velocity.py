"""Velocity parameterisation (lame=.false.): GPU images and Born gathers
against the reference's velocity imaging condition and velocity Born sources
(W/image-mod-rtm.f90:182-225) restated literally here, per time level, over
the oracle's FP64 source and adjoint histories."""
import numpy as np
import pytest

import oracle as O
from elastic_gb300 import rtm as R
from elastic_gb300 import synth

pytestmark = pytest.mark.gpu

# receivers on row 12: Vz and sigmaxz are only updated from row 6 on, so a
# shallower row would record zeros for them
NZ, NX, NT, ABC, ZREC, XSRC, ZSRC, NS = 40, 48, 100, 8, 12, 24, 6, 30
DX, DT, FP = 10.0, 1e-3, 30.0


def models():
    vp = synth.smooth_random_model(NZ, NX, DX, 80.0, 1900.0, 3300.0, seed=5)
    vs = vp / 1.8
    rho = 310.0 * vp ** 0.25
    return [np.ascontiguousarray(a, np.float64) for a in (rho, vp, vs)]


def histories(rho, vp, vs):
    lam, mu = rho * (vp ** 2 - 2 * vs ** 2), rho * vs ** 2
    coefs = list(O.coefficients(rho, lam, mu, DX, DT))
    src = O.source_op2(NT, DT, FP, NS, dtype=np.float64)
    filt = O.abc_init(ABC, np.float64)
    H = O.forward(coefs, NT, DT, ZSRC, XSRC, src, ABC, filt)
    S = O.image_init(H[0], H[1], DX, DT)
    return coefs, filt, S


def vel_images_reference(rho, vp, vs, A, S):
    """image_op2(adj), lame=.false., W/image-mod-rtm.f90:182-198"""
    m1, m2, m3 = rho, vp, vs
    dm1, dm2, dm3 = (np.zeros_like(rho) for _ in range(3))
    Vx, Vz, sxx, szz, sxz = A
    S1, S2, S3, S4, S5, S6 = S
    for it in range(NT):
        dm1 += (Vx[it] * S1[it]) + (Vz[it] * S2[it]) \
            - (sxx[it] * (m2 * m2 * S4[it] + (m2 * m2 - 2.0 * m3 * m3) * S5[it])) \
            - (szz[it] * (m2 * m2 * S5[it] + (m2 * m2 - 2.0 * m3 * m3) * S4[it])) \
            - (sxz[it] * (m3 * m3 * S6[it]))
        dm2 -= (sxx[it] * (2.0 * m1 * m2 * S3[it])) + (szz[it] * (2.0 * m1 * m2 * S3[it]))
        dm3 += (sxx[it] * (4.0 * m1 * m3 * S5[it])) + (szz[it] * (4.0 * m1 * m3 * S4[it])) \
            - (sxz[it] * (2.0 * m1 * m3 * S6[it]))
    return dm1, dm2, dm3


def vel_sources_reference(rho, vp, vs, dm, S):
    """image_op2(forward), lame=.false., W/image-mod-rtm.f90:199-222"""
    m1, m2, m3 = rho, vp, vs
    d1, d2, d3 = dm
    S1, S2, S3, S4, S5, S6 = S
    H = [np.zeros((NT, NX, NZ)) for _ in range(5)]
    for it in range(NT):
        H[0][it] = d1 * S1[it]
        H[1][it] = d1 * S2[it]
        H[2][it] = -(d1 * (m2 * m2 * S4[it] + (m2 * m2 - 2.0 * m3 * m3) * S5[it])) \
            - (d2 * (2.0 * m1 * m2 * S3[it])) + (d3 * (4.0 * m1 * m3 * S5[it]))
        H[3][it] = -(d1 * (m2 * m2 * S5[it] + (m2 * m2 - 2.0 * m3 * m3) * S4[it])) \
            - (d2 * (2.0 * m1 * m2 * S3[it])) + (d3 * (4.0 * m1 * m3 * S4[it]))
        H[4][it] = -(d1 * (m3 * m3 * S6[it])) - (d3 * (2.0 * m1 * m3 * S6[it]))
    return H


def rel(a, b):
    nb = np.linalg.norm(b)
    assert nb > 0, "reference is all zero"
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / nb)


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 2e-4)])
def test_velocity_images_match_reference_condition(dtype, tol):
    rho, vp, vs = models()
    coefs, filt, S = histories(rho, vp, vs)
    rng = np.random.default_rng(1)
    D = [rng.standard_normal((NX, NT)) for _ in range(5)]
    A = O.rtm_op3(D, coefs, NZ, ZREC, exact=False, abc=ABC, filt=filt)
    ref = vel_images_reference(rho, vp, vs, A, S)
    op = R.RtmOperator(NZ, DX, NX, DX, DT, XSRC, ZSRC, ZREC, FP, NT, ABC, rho, vp, vs, nsource=NS, dtype=dtype,
                       lame=False)
    im = [np.zeros((NX, NZ), dtype) for _ in range(3)]
    op.rtm_op(True, *im, *[np.ascontiguousarray(d, dtype) for d in D])
    errs = [rel(a, b) for a, b in zip(im, ref)]
    print(dtype.__name__, "velocity images rel L2", errs)
    assert max(errs) < tol


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 2e-4)])
def test_velocity_born_matches_reference_sources(dtype, tol):
    rho, vp, vs = models()
    coefs, filt, S = histories(rho, vp, vs)
    rng = np.random.default_rng(2)
    dm = [0.05 * rho * rng.standard_normal((NX, NZ)), 0.05 * vp * rng.standard_normal((NX, NZ)),
          0.05 * vs * rng.standard_normal((NX, NZ))]
    Hs = vel_sources_reference(rho, vp, vs, dm, S)
    ref = O.born_scatter(Hs, coefs, ZREC, ABC, filt)
    op = R.RtmOperator(NZ, DX, NX, DX, DT, XSRC, ZSRC, ZREC, FP, NT, ABC, rho, vp, vs, nsource=NS, dtype=dtype,
                       lame=False, linear=True)
    D = [np.zeros((NX, NT), dtype) for _ in range(5)]
    op.rtm_op(False, *[np.ascontiguousarray(x, dtype) for x in dm], *D)
    errs = [rel(a, b) for a, b in zip(D, ref)]
    print(dtype.__name__, "velocity Born gathers rel L2", errs)
    assert max(errs) < tol


def test_velocity_jacobian_pair_is_a_transpose():
    """<J x, y> = <x, J^T y> per cell, in FP64."""
    rho, vp, vs = models()
    rng = np.random.default_rng(3)
    x = [rng.standard_normal((NX, NZ)) for _ in range(3)]
    y = [rng.standard_normal((NX, NZ)) for _ in range(3)]
    Jx = R.velocity_jacobian(False, rho, vp, vs, *x)
    JTy = R.velocity_jacobian(True, rho, vp, vs, *y)
    lhs = sum(float(np.vdot(a, b)) for a, b in zip(Jx, y))
    rhs = sum(float(np.vdot(a, b)) for a, b in zip(x, JTy))
    assert lhs == pytest.approx(rhs, rel=1e-12)
