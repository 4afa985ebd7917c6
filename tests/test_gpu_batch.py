"""GPU tests of the batched multi-shot RTM (FP16 source snapshots, fused
Kahan imaging, CUDA-graph time loop) against the oracle's full-history FP32
RTM of every shot on its subgrid, stacked."""
import numpy as np
import pytest

import oracle as O
from elastic_gb300 import rtm as R
from elastic_gb300 import synth
from elastic_gb300._lib import RtmError
from elastic_gb300.batch import BatchRTM

pytestmark = pytest.mark.gpu

# FP16 snapshots perturb the source wavefield by ~2^-12 of its per-level
# maximum; the stacked images agree with the FP32 full-history oracle to
# this relative L2 (observed values are printed by the test).
RTOL_SNAP = 5e-3

# The marching adjoint sums the two pairs of coefficient x field products
# that share a stencil before differencing them (a23*sxx + a2*szz under the
# x difference of Vx, a2*sxx + a23*szz under the z difference of Vz); against
# the tile kernel, which differences each product, the images agree to this
# relative L2 (observed values are printed).
RTOL_REASSOC = 1e-5


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def survey(nshots=5, nz=48, nx=200, nt=160, seed=1, spacing=24, wmin=50, wmax=96):
    vp = synth.smooth_random_model(nz, nx, 10.0, 150.0, 1800.0, 3500.0, seed=seed)
    rho, lam, mu = synth.lame_from_vp(vp)
    x0, nxs, xsrc = synth.uneven_survey(nx, nshots, spacing, wmin, wmax, seed=seed)
    rng = np.random.default_rng(seed)
    traces = [[(rng.standard_normal((w, nt))).astype(np.float32) for _ in range(2)] for w in nxs]
    return rho, lam, mu, x0, nxs, xsrc, traces


def oracle_stack(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, dtype=np.float32):
    img = [np.zeros((nx, nz), np.float64) for _ in range(3)]
    for s in range(len(nxs)):
        a, w = int(x0[s] - 1), int(nxs[s])
        D = [traces[s][0], traces[s][1]] + [np.zeros((w, nt), np.float32)] * 3
        D = [np.ascontiguousarray(d, dtype) for d in D]
        sl = lambda m: np.ascontiguousarray(m[a:a + w], dtype)
        dm, _ = O.rtm_op2(True, sl(rho), sl(lam), sl(mu), [np.zeros((w, nz), dtype)] * 3, D, dtype(dx), dtype(dt),
                          int(nt), int(zs), int(xsrc[s] - a), int(zr), dtype(fp), int(abc), int(ns))
        for i in range(3):
            img[i][a:a + w] += dm[i]
    return img


def run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group, graph=True,
              tile_x=0, tune=False, stages=None, march=None):
    n = len(nxs)
    eng = BatchRTM(nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, np.full(n, zs), np.full(n, zr),
                   comp_mask=3, group_max=group, nsource=ns)
    if tune:
        eng.autotune(0, group, steps=4)
    eng.set_graph(graph, tile_x)
    if stages:
        eng.set_stages(*stages)
    if march is not None:
        eng.set_march(march)
    image = np.zeros(3 * nz * nx, np.float32)
    for s0, k in eng.groups():
        flat = np.concatenate([np.concatenate([traces[s][c].ravel() for c in range(2)]) for s in range(s0, s0 + k)])
        eng.migrate(s0, k, flat, image)
    st = eng.stats()
    eng.close()
    return image.reshape(3, nx, nz), st


@pytest.mark.parametrize("version", [1, 2])
def test_batch_matches_oracle_stack(version):
    R.set_kernel_version(version)
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 48, 200, 160, 10.0, 1e-3, 30.0, 12, 6, 6, 40
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nz=nz, nx=nx, nt=nt)
    img, st = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=2)
    ref32 = oracle_stack(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns)
    ref64 = oracle_stack(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, np.float64)
    errs32 = [rel_l2(img[i], ref32[i]) for i in range(3)]
    errs64 = [rel_l2(img[i], ref64[i]) for i in range(3)]
    print("batch vs FP32 oracle", errs32, "vs FP64 oracle", errs64, st)
    R.set_kernel_version(0)
    assert max(errs32) < RTOL_SNAP
    assert max(errs64) < RTOL_SNAP
    # v2 folds the FP32 partial images into the compensated totals every 32
    # levels (one extra launch each)
    assert st["kernels"] == 2 * nt + (0 if version == 1 else -(-nt // 32))


def test_batch_graph_and_grouping_are_bit_identical():
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 40, 180, 90, 10.0, 1e-3, 30.0, 10, 6, 6, 40
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=4, nz=nz, nx=nx, nt=nt, seed=3)
    a, _ = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=4)
    b, _ = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=1,
                     graph=False)
    np.testing.assert_array_equal(a, b)


def test_batch_tile_widths_and_autotuner_are_bit_identical():
    """The tile width (chosen by hand or by the autotuner) does not change
    the arithmetic of any cell."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 40, 180, 60, 10.0, 1e-3, 30.0, 10, 6, 6, 40
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=3, nz=nz, nx=nx, nt=nt, seed=5)
    ref, _ = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=3, tile_x=8,
                       march=0)
    for tx, stages in ((16, None), (8, (2, 2)), (16, (2, 2)), (16, (1, 2, 512, 512)), (32, (2, 1, 512, 512))):
        # two staging buffers (next tile staged during the current one) do
        # not change the arithmetic either; where they do not fit the
        # launcher keeps one
        img, _ = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=3,
                           tile_x=tx, stages=stages, march=0)
        np.testing.assert_array_equal(img, ref)
    # the autotuner may also pick the marching kernels (forward bit for
    # bit, adjoint to rounding)
    img, st = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=3,
                        tune=True)
    assert max(rel_l2(img[i], ref[i]) for i in range(3)) < RTOL_REASSOC
    assert st["tile_x"] in (8, 16, 32) and st["tile_x_adj"] in (8, 16, 32)
    # -1 marks a tile width that does not fit in shared memory
    assert all(t > 0 or t == -1 for t in st["tune_ms_fwd"] + st["tune_ms_adj"])
    assert max(st["tune_ms_fwd"]) > 0 and max(st["tune_ms_adj"]) > 0
    assert st["stages"] in (1, 2) and st["stages_adj"] in (1, 2)
    assert all(t > 0 or t == -1 for row in st["tune_ms_fwd_variants"] + st["tune_ms_adj_variants"] for t in row)
    assert st["threads"] in (256, 512) and st["threads_adj"] in (256, 512)


def test_batch_staging_depth_with_several_tiles_per_cta_is_bit_identical():
    """A grid large enough that every CTA loops over several work items, so
    the two-stage path prefetches the next tile while computing the current
    one; one and two staging buffers give the same image, bit for bit."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 700, 1200, 24, 10.0, 1e-3, 30.0, 20, 8, 8, 20
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=3, nz=nz, nx=nx, nt=nt, seed=7, spacing=300, wmin=300,
                                                 wmax=400)
    for tx in (8, 16):
        ref, st = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=3,
                            tile_x=tx, stages=(1, 1), march=0)
        assert st["work_items"] > 2 * 152  # more work items than resident CTAs
        assert np.isfinite(ref).all() and np.abs(ref).max() > 0
        for stages in ((2, 2), (1, 1, 512, 512), (2, 2, 512, 512)):
            if tx == 8 and len(stages) > 2:
                continue  # 512 threads need tile width >= 16
            img, _ = run_batch(rho, lam, mu, x0, nxs, xsrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=3,
                               tile_x=tx, stages=stages, march=0)
            np.testing.assert_array_equal(img, ref)


@pytest.mark.parametrize("interval", [7, 13, 59, 60])
def test_batch_checkpoint_restart_is_bit_identical(interval):
    """Checkpointing the forward state every `interval` levels and
    recomputing each segment in the adjoint pass reproduces the images of
    the all-levels snapshot store bit for bit (the recomputation is the same
    deterministic forward recursion, snapshot scales included)."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 40, 180, 60, 10.0, 1e-3, 30.0, 10, 6, 6, 40
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=3, nz=nz, nx=nx, nt=nt, seed=9)

    def run(k):
        n = len(nxs)
        eng = BatchRTM(nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, np.full(n, zs), np.full(n, zr),
                       comp_mask=3, group_max=3, nsource=ns)
        if k:
            eng.set_checkpoint(k)
        image = np.zeros(3 * nz * nx, np.float32)
        for s0, g in eng.groups():
            flat = np.concatenate([np.concatenate([traces[s][c].ravel() for c in range(2)]) for s in range(s0, s0 + g)])
            eng.migrate(s0, g, flat, image)
        st = eng.stats()
        eng.close()
        return image, st

    ref, st0 = run(0)
    img, st = run(interval)
    assert st0["checkpoint"] == 0 and st["checkpoint"] == interval
    np.testing.assert_array_equal(img, ref)
    assert np.abs(ref).max() > 0


@pytest.mark.parametrize("tile,stages,interval", [(8, (1, 1), 0), (16, (2, 2), 0), (8, (2, 1), 7), (32, (1, 1), 0)])
def test_batch_tma_staging_is_bit_identical(tile, stages, interval):
    """Staging the step tiles with tensor-memory-access loads (zeros from the
    hardware fill and the guard columns) gives the images of the per-thread
    asynchronous copies bit for bit, with one or two staging buffers and in
    checkpoint-restart mode; most CTAs walk several work items (nz 700)."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 700, 700, 40, 10.0, 1e-3, 30.0, 20, 8, 8, 20
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=3, nz=nz, nx=nx, nt=nt, seed=11, spacing=200, wmin=150,
                                                 wmax=260)

    def run(tma):
        n = len(nxs)
        eng = BatchRTM(nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, np.full(n, zs), np.full(n, zr),
                       comp_mask=3, group_max=3, nsource=ns)
        eng.set_graph(True, tile)
        eng.set_stages(*stages)
        if interval:
            eng.set_checkpoint(interval)
        eng.set_tma(tma)
        eng.set_march(0)  # the tile kernels, staged both ways
        image = np.zeros(3 * nz * nx, np.float32)
        for s0, g in eng.groups():
            flat = np.concatenate([np.concatenate([traces[s][c].ravel() for c in range(2)]) for s in range(s0, s0 + g)])
            eng.migrate(s0, g, flat, image)
        st = eng.stats()
        eng.close()
        return image, st

    ref, st0 = run(False)
    img, st = run(True)
    assert st["tma"] and not st0["tma"]
    np.testing.assert_array_equal(img, ref)
    assert np.abs(ref).max() > 0


@pytest.mark.parametrize("nz,nx,nt,interval", [(40, 180, 60, 0), (300, 900, 40, 0), (700, 700, 40, 7), (280, 900, 40, 0),
                                                (800, 700, 40, 7)])
def test_batch_marching_kernels_match_tile_kernels(nz, nx, nt, interval):
    """The passes by the marching kernels (one CTA per SM walking 128-row
    strips in 8-column chunks through rings of staged columns and adjoint
    products): the forward gives the tile kernel's images bit for bit, the
    adjoint agrees to rounding; one strip narrower than the grid of CTAs,
    several strips with a partial last one, thin last strips (24 and 32
    rows) that the adjoint marches in bands, checkpoint-restart mode; the
    autotuner times them beside the tile variants."""
    dx, dt, fp, abc, zs, zr, ns = 10.0, 1e-3, 30.0, 20 if nz > 100 else 10, 8, 8, 20
    wmin, wmax, spacing = (50, 96, 24) if nx < 300 else (150, 400, 200)
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=3, nz=nz, nx=nx, nt=nt, seed=13, spacing=spacing, wmin=wmin,
                                                 wmax=wmax)

    def run(march, tune=False):
        n = len(nxs)
        eng = BatchRTM(nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, np.full(n, zs), np.full(n, zr),
                       comp_mask=3, group_max=3, nsource=ns)
        if interval:
            eng.set_checkpoint(interval)
        if tune:
            eng.autotune(0, 3, steps=2)
        eng.set_march(march)
        image = np.zeros(3 * nz * nx, np.float32)
        for s0, g in eng.groups():
            flat = np.concatenate([np.concatenate([traces[s][c].ravel() for c in range(2)]) for s in range(s0, s0 + g)])
            eng.migrate(s0, g, flat, image)
        st = eng.stats()
        eng.close()
        return image.reshape(3, nx, nz), st

    ref, st0 = run(0)
    fwd, st1 = run(1)
    both, st3 = run(3)
    assert not st0["march"] and not st0["march_adj"]
    assert st1["march"] and not st1["march_adj"]
    assert st3["march"] and st3["march_adj"]
    np.testing.assert_array_equal(fwd, ref)
    assert np.abs(ref).max() > 0
    errs = [rel_l2(both[i], ref[i]) for i in range(3)]
    print("marching adjoint vs tile adjoint, rel. L2 per image:", errs)
    assert max(errs) < RTOL_REASSOC
    if nz == 300:
        img, st = run(-1, tune=True)
        assert st["tune_ms_march"] > 0 and st["tune_ms_march_adj"] > 0
        assert max(rel_l2(img[i], ref[i]) for i in range(3)) < RTOL_REASSOC


def test_survey_geometry_group_vs_fp64_oracle():
    """One 4-shot group of the 64-shot survey at its full geometry -- 2000 x
    800 grid, dx = 5 m, dt = 0.5 ms, smooth random background (1800-4000 m/s,
    200 m correlation), subgrids 600-2000 cells wide, source and receivers at
    row 10, 40-cell sponge -- over a truncated window of nt = 600 levels, on
    the marching kernels with FP16 source snapshots, against the float64
    oracle's RTM of every shot (ora_rtm_lowmem, the reference's algorithm in
    double precision), stacked.  The traces are the Vx, Vz gathers that the
    drop-in Born operator models from a dipping-reflector perturbation of the
    background between rows 46 and 90 (just below the sponge: its
    reflections reach the receivers within the window).  Each image's
    relative L2 error is printed."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 800, 2000, 600, 5.0, 5e-4, 15.0, 40, 10, 10, 250
    vp = synth.smooth_random_model(nz, nx, dx, 200.0, 1800.0, 4000.0, seed=2)
    rho, lam, mu = synth.lame_from_vp(vp)
    x0, nxs, xsrc = synth.uneven_survey(nx, 64, 15, 600, 2000, seed=2)
    # the group of four consecutive shots with the widest subgrids
    s0 = max(range(0, 64, 4), key=lambda s: int(nxs[s:s + 4].sum()))
    sel = list(range(s0, s0 + 4))
    refl = synth.dipping_reflectivity(nz, nx, seed=2, top=46, bottom=90)
    traces = []
    for s in sel:
        a, w = int(x0[s] - 1), int(nxs[s])
        sl = lambda m: np.ascontiguousarray(m[a:a + w])
        op = R.RtmOperator(nz, dx, w, dx, dt, int(xsrc[s] - a), zs, zr, fp, nt, abc, sl(rho), sl(lam), sl(mu),
                           nsource=ns, linear=True)
        dm = [np.ascontiguousarray((refl[a:a + w] * m[a:a + w]).astype(np.float32)) for m in (rho, lam, mu)]
        D = [np.zeros((w, nt), np.float32) for _ in range(5)]
        R.set_exact(False)
        try:
            assert op.rtm_op(False, *dm, *D) == 0
        finally:
            R.set_exact(True)
        traces.append([D[0], D[1]])
        assert np.abs(D[0]).max() > 0 and np.abs(D[1]).max() > 0
    sx0, snx, ssrc = x0[sel], nxs[sel], xsrc[sel]
    img, st = run_batch(rho, lam, mu, sx0, snx, ssrc, traces, nz, nx, nt, dx, dt, fp, abc, zs, zr, ns, group=4,
                        march=3)
    assert st["march"] and st["march_adj"]
    ref = [np.zeros((nx, nz)) for _ in range(3)]
    for k, s in enumerate(sel):
        a, w = int(x0[s] - 1), int(nxs[s])
        sl = lambda m: np.ascontiguousarray(m[a:a + w], np.float64)
        D = [traces[k][0].astype(np.float64), traces[k][1].astype(np.float64)] + [np.zeros((w, nt))] * 3
        dm = O.rtm_lowmem(sl(rho), sl(lam), sl(mu), D, dx, dt, nt, zs, int(xsrc[s] - a), zr, fp, abc, ns)
        for i in range(3):
            ref[i][a:a + w] += dm[i]
    assert min(np.abs(r).max() for r in ref) > 0
    errs = [rel_l2(img[i], ref[i]) for i in range(3)]
    print("survey-geometry group (widths %s, nt=%d): image rel. L2 vs float64 oracle drho %.2e dlambda %.2e "
          "dmu %.2e" % (list(map(int, snx)), nt, *errs))
    assert max(errs) < RTOL_SNAP


def test_batch_wait_timeout_returns_status_4_and_recovers():
    """The timeout path of the bounded device waits.  With the test hook on,
    the first forward marching launch waits on a device flag that nothing
    sets: its wait gives up after about a second (before any copy is
    issued), the chunk waits of its compute warps run out as well, the
    kernels record it in the engine's error flag and rtm_batch_migrate
    returns RTM_ERR_TIMEOUT (4).  With the hook off the same engine migrates
    the same group again and its image equals that of a migration before the
    timeout bit for bit; the drop-in path still matches the oracle."""
    nz, nx, nt, dx, dt, fp, abc, zs, zr, ns = 40, 160, 60, 10.0, 1e-3, 30.0, 10, 6, 6, 40
    rho, lam, mu, x0, nxs, xsrc, traces = survey(nshots=2, nz=nz, nx=nx, nt=nt, seed=5, spacing=40, wmin=60,
                                                 wmax=80)
    eng = BatchRTM(nz, nx, nt, dx, dt, fp, abc, rho, lam, mu, x0, nxs, xsrc, np.full(2, zs), np.full(2, zr),
                   comp_mask=3, group_max=2, nsource=ns)
    eng.set_march(3)
    flat = np.concatenate([np.concatenate([t[0].ravel(), t[1].ravel()]) for t in traces])
    before = np.zeros(3 * nz * nx, np.float32)
    eng.migrate(0, 2, flat, before)
    eng.set_test_stall(True)
    with pytest.raises(RtmError, match="status 4"):
        eng.migrate(0, 2, flat, np.zeros(3 * nz * nx, np.float32))
    eng.set_test_stall(False)
    after = np.zeros(3 * nz * nx, np.float32)
    eng.migrate(0, 2, flat, after)
    eng.close()
    np.testing.assert_array_equal(after, before)
    assert np.abs(before).max() > 0
    # the library's other entry points are unaffected
    rng = np.random.default_rng(3)
    C = [(0.05 * rng.standard_normal((48, 40))).astype(np.float32) for _ in range(5)]
    H = [rng.standard_normal((12, 48, 40)).astype(np.float32) for _ in range(5)]
    ref = [h.copy() for h in H]
    O.rtm_op3_c(ref, C)
    R.set_exact(True)
    R.rtm_op3(12, 40, 48, 1, *H, *C)
    for a, b in zip(H, ref):
        np.testing.assert_array_equal(a, b)
