"""The oracle against an execution of the reference's own Fortran.

The reference's RTM and Born path (2d_rtm_restart/Src_working/
rtm-mod-adj.f90:132-496 with model-mod.f90, source-mod.f90, abc-mod.f90,
rtmlib-mod.f90, image-mod-rtm.f90 and the C recursion rtmlib-modC.c) runs
here through oracle/f90c.py, which translates the Fortran modules to C as
they are written (no Fortran compiler exists in this image).  Every
intermediate array the modules keep is compared with the oracle's restated
functions bit for bit: coefficients (model_op, rtmmod_init, aux_*_c), the
Ricker table, the sponge filter, the five source-wavefield histories, the
imaging operators S1..S6, the Born gathers and the images.

The committed fixtures made from the same execution
(tests/golden/make_golden_f90.py) carry the pin to machines without the
reference tree; tests/test_oracle.py and the GPU tests read them.
"""
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

pytestmark = pytest.mark.skipif(not O.ref90_available(), reason="reference tree not present")

F = np.float32


def _model(nz, nx, seed):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :]
    vp = np.where(z < nz // 2, 2000.0, 2800.0) * (1 + 0.03 * rng.standard_normal((nx, nz)))
    vs = vp / 1.73
    if seed % 2:
        vs[:, : nz // 4] = 0.0  # a fluid top: mu = 0 takes model_op's zero branch
    rho = (310.0 * vp ** 0.25).astype(F)
    lam = (rho * (vp ** 2 - 2 * vs ** 2)).astype(F)
    mu = (rho * vs ** 2).astype(F)
    return rho, lam, mu


# (nz, nx, nt, abc, zsrc, xsrc, zrec): odd sizes, a sponge that covers most
# of a small grid, acquisition inside and below the sponge, nt below and
# above the progress bar's 59 levels
CASES = [
    (37, 45, 260, 8, 12, 23, 12),
    (40, 48, 300, 10, 5, 24, 5),
    (64, 71, 280, 20, 25, 30, 26),
    (33, 130, 257, 4, 9, 100, 7),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%dx%dx%d_abc%d" % c[:4])
def test_reference_rtm_equals_oracle_at_every_stage(case):
    nz, nx, nt, abc, zsrc, xsrc, zrec = case
    dx, dt, fp = 10.0, 1e-3, 15.0
    rho, lam, mu = _model(nz, nx, seed=nz + nx)
    rng = np.random.default_rng(nt)
    D = [rng.standard_normal((nx, nt)).astype(F) for _ in range(5)]
    zero = [np.zeros((nx, nz), F) for _ in range(3)]
    r = O.ref90_rtm(True, rho, lam, mu, zero, D, dx, dt, nt, zsrc, xsrc, zrec, fp, abc, forward=True,
                    state=O.REF90_STATE)

    # a1, a2: model_op, rtmmod_init, aux_*_c
    coefs = O.coefficients(rho, lam, mu, F(dx), F(dt))
    names = ["m1_x", "m1_z", "aux_m2_c", "aux_m3_c", "aux_m2m3_c"]
    for c, n in zip(coefs, names):
        np.testing.assert_array_equal(r["rtm_mod_adj." + n], c, err_msg=n)
    # a3, a4: Ricker table (nsource = 250, rtm-mod-adj.f90:100) and sponge filter
    src = O.source_op2(nt, F(dt), F(fp), 250)
    np.testing.assert_array_equal(r["rtm_mod_adj.source"], src)
    filt = O.abc_init(abc)
    np.testing.assert_array_equal(r["abc_mod.filter"], filt)
    # a5, a6: forward operators inside the source-wavefield loop
    H = O.forward(coefs, nt, F(dt), zsrc, xsrc, src, abc, filt)
    for k in range(5):
        np.testing.assert_array_equal(r["fwd"][k], H[k], err_msg="history %d" % k)
    # a7: image_init
    S = O.image_init(H[0], H[1], F(dx), F(dt))
    for k in range(6):
        np.testing.assert_array_equal(r["image_mod_rtm.s%d" % (k + 1)], S[k], err_msg="S%d" % (k + 1))
    # a10, a11, a13: rtm_op3 (F90 first levels + C recursion) and the imaging condition
    img, _ = O.rtm_op2(True, rho, lam, mu, zero, D, F(dx), F(dt), nt, zsrc, xsrc, zrec, F(fp), abc, 250)
    for k in range(3):
        np.testing.assert_array_equal(r["dm"][k], img[k], err_msg="image %d" % k)


@pytest.mark.parametrize("case", CASES[:3], ids=lambda c: "%dx%dx%d_abc%d" % c[:4])
def test_reference_born_equals_oracle(case):
    """a8, a9: model_delta, the Born secondary sources and the scattered loop."""
    nz, nx, nt, abc, zsrc, xsrc, zrec = case
    dx, dt, fp = 10.0, 1e-3, 15.0
    rho, lam, mu = _model(nz, nx, seed=nz + nx + 1)
    rng = np.random.default_rng(nz)
    dm = [(0.05 * rng.standard_normal((nx, nz)) * m).astype(F) for m in (rho, lam, mu)]
    dm[0][:, :3] = 0.05  # below model_delta's 0.1 threshold: zeroed density averages
    D0 = [np.zeros((nx, nt), F) for _ in range(5)]
    r = O.ref90_rtm(False, rho, lam, mu, dm, D0, dx, dt, nt, zsrc, xsrc, zrec, fp, abc)
    _, D = O.rtm_op2(False, rho, lam, mu, dm, D0, F(dx), F(dt), nt, zsrc, xsrc, zrec, F(fp), abc, 250)
    for k in range(5):
        np.testing.assert_array_equal(r["D"][k], D[k], err_msg="gather %d" % k)


def test_reference_lambda_mu_are_averaged_in_place():
    """rtm_init hands lambda and mu to model_op, which replaces them by their
    harmonic averages (model-mod.f90:65-88); the oracle's model_op returns
    the same averaged planes."""
    nz, nx = 30, 26
    rho, lam, mu = _model(nz, nx, seed=3)
    r = O.ref90_rtm(True, rho, lam, mu, [np.zeros((nx, nz), F)] * 3, [np.zeros((nx, 260), F)] * 5, 10.0, 1e-3,
                    260, 10, 13, 10, 15.0, 6, state=["model_mod.m2", "model_mod.m3"])
    _, _, m2, m3 = O.model_op(rho, lam, mu)
    np.testing.assert_array_equal(r["model_mod.m2"], m2)
    np.testing.assert_array_equal(r["model_mod.m3"], m3)


def test_reference_fixtures_are_current():
    """The committed fixtures equal a fresh execution of the reference."""
    g = np.load(os.path.join(GOLD, "ref90_small.npz"))
    for name in sorted({k.split("/")[0] for k in g.files}):
        p = {k.split("/")[1]: g[k] for k in g.files if k.startswith(name + "/")}
        nz, nx, nt, abc, zsrc, xsrc, zrec = (int(v) for v in p["geom"])
        dx, dt, fp = (float(v) for v in p["phys"])
        r = O.ref90_rtm(False, p["rho"], p["lam"], p["mu"], list(p["dm"]), [np.zeros((nx, nt), F)] * 5,
                        dx, dt, nt, zsrc, xsrc, zrec, fp, abc)
        np.testing.assert_array_equal(np.stack(r["D"]), p["born"])
        r = O.ref90_rtm(True, p["rho"], p["lam"], p["mu"], [np.zeros((nx, nz), F)] * 3, list(p["born"]),
                        dx, dt, nt, zsrc, xsrc, zrec, fp, abc)
        np.testing.assert_array_equal(np.stack(r["dm"]), p["image"])


def _velocity_helpers():
    import importlib.util
    spec = importlib.util.spec_from_file_location("velocity_gpu_test", os.path.join(HERE, "test_gpu_velocity.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("adj", [True, False])
def test_velocity_imaging_restatement_equals_reference(adj):
    """The velocity-parameterisation imaging condition and Born sources
    (lame=.false., W/image-mod-rtm.f90:182-225) that tests/test_gpu_velocity.py
    holds the GPU to, against the reference's own image_init, image_init2 and
    image_op2 executed on the same float32 histories: equal to float32
    rounding (the restatement sums in float64)."""
    tv = _velocity_helpers()
    rho, vp, vs = tv.models()
    coefs, filt, _ = tv.histories(rho, vp, vs)
    src = O.source_op2(tv.NT, tv.DT, tv.FP, tv.NS, dtype=np.float64)
    H = O.forward(coefs, tv.NT, tv.DT, tv.ZSRC, tv.XSRC, src, tv.ABC, filt)
    f32 = lambda a: np.asarray(a, F)
    f64 = lambda a: np.asarray(a, F).astype(np.float64)
    m = [f32(rho), f32(vp), f32(vs)]
    S = [x.astype(np.float64) for x in O.image_init(f32(H[0]), f32(H[1]), F(tv.DX), F(tv.DT))]
    rng = np.random.default_rng(2)
    if adj:
        A = [f32(rng.standard_normal(H[0].shape)) for _ in range(5)]
        got = O.ref90_image(True, False, m, f32(H[0]), f32(H[1]), tv.DX, tv.DT, H=A)
        want = tv.vel_images_reference(f64(rho), f64(vp), f64(vs), [a.astype(np.float64) for a in A], S)
    else:
        dm = [f32(rng.standard_normal(rho.shape)) for _ in range(3)]
        got = O.ref90_image(False, False, m, f32(H[0]), f32(H[1]), tv.DX, tv.DT, dm=dm)
        want = tv.vel_sources_reference(f64(rho), f64(vp), f64(vs), [d.astype(np.float64) for d in dm], S)
    for a, b in zip(got, want):
        assert np.linalg.norm(b) > 0
        assert np.linalg.norm(a - b) <= 2e-6 * np.linalg.norm(b)
