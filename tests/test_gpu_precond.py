"""Learned preconditioner workflow: the batched Born/migration entry point
agrees bit for bit with rtm_op (linear Born, exact adjoint); a U-Net trained
on the GPU from the project's own (reflectivity, migrated image) pairs
lowers the Born data residual of held-out migrations below plain RTM's and
below 10 iterations of plain LSRTM."""
import numpy as np
import pytest

from elastic_gb300 import precond as PC
from elastic_gb300 import rtm as R

pytestmark = pytest.mark.gpu

NX = NZ = 64
# 0.8 s of record: reflections from the bottom of the 640 m window return
NT, DX, DT, FP, ABC, NS = 800, 10.0, 1e-3, 25.0, 10, 40


def problem(comp_mask=3):
    rho, lam, mu = PC.background_window(NX, NZ, nz_model=NZ, smooth_cells=2.0)
    return PC.Problem(rho, lam, mu, DX, DT, NT, NX // 2 + 1, 5, 5, FP, ABC, NS, comp_mask=comp_mask)


def test_born_migrate_matches_rtm_op():
    pb = problem(comp_mask=31)
    rng = np.random.default_rng(0)
    r = PC.random_reflectivity(rng, 2, NX, NZ, ABC + 2)
    dm = r * pb.bg[None]
    data, img = pb.born_migrate(dm)
    for k in range(2):
        D = [np.zeros((NX, NT), np.float32) for _ in range(5)]
        m = [np.ascontiguousarray(dm[k, i]) for i in range(3)]
        op = R.RtmOperator(NZ, DX, NX, DX, DT, pb.xsrc, pb.zsrc, pb.zrec, FP, NT, ABC, pb.rho, pb.lam, pb.mu,
                           nsource=NS, linear=True, exact_adjoint=True)
        op.rtm_op(False, *m, *D)
        np.testing.assert_array_equal(np.stack(D), data[k])
        im = [np.zeros((NX, NZ), np.float32) for _ in range(3)]
        op.rtm_op(True, *im, *[np.ascontiguousarray(data[k, c]) for c in range(5)])
        np.testing.assert_array_equal(np.stack(im), img[k])
    # migration of given data equals the image of the combined call
    np.testing.assert_array_equal(pb.migrate(data), img)


def test_component_mask_zeroes_unrecorded_gathers():
    pb = problem(comp_mask=3)
    rng = np.random.default_rng(4)
    dm = PC.random_reflectivity(rng, 1, NX, NZ, ABC + 2) * pb.bg[None]
    full = problem(comp_mask=31)
    d3, d31 = pb.born(dm), full.born(dm)
    np.testing.assert_array_equal(d3[:, :2], d31[:, :2])
    assert not d3[:, 2:].any()
    # migration ignores the unrecorded components of its input
    np.testing.assert_array_equal(pb.migrate(d31), pb.migrate(d3))


def test_learned_preconditioner_beats_rtm_and_lsrtm_on_held_out_pairs():
    """Trained on 768 (reflectivity, migrated image) pairs of the Vx/Vz
    survey; on 8 held-out pairs the learned estimate (with its least-squares
    scale) has a lower Born data residual than RTM with its best scale and
    than 10 iterations of plain LSRTM."""
    pb = problem()
    rng = np.random.default_rng(1)
    ntrain, ntest = 768, 8
    r = PC.random_reflectivity(rng, ntrain + ntest, NX, NZ, ABC + 2)
    dm = r * pb.bg[None]
    data, img = pb.born_migrate(dm)
    pc = PC.Preconditioner(NX, NZ, batch=32, seed=0, margin=ABC + 2)
    pc.fit_scales(img[:ntrain])
    losses = pc.train(img[:ntrain], r[:ntrain], steps=1500, lr=1e-3)
    zero_loss = float(np.mean((pc.out_scale * r[:ntrain]) ** 2))
    d_test, img_test = data[ntrain:], img[ntrain:]
    m_nn = pc.apply(img_test, pb.bg)
    res_nn = PC.scaled_residual(pb, m_nn, d_test)
    res_rtm = PC.scaled_residual(pb, img_test, d_test)
    ls = [pb.lsrtm(d_test[k], 10) for k in range(2)]
    res_ls = np.array([x[1][-1] / x[1][0] for x in ls])
    print("train loss", losses[0], "->", np.mean(losses[-50:]), "(zero prediction", zero_loss, ")")
    print("Born residual: learned", res_nn, "RTM (best scale)", res_rtm, "LSRTM-10", res_ls)
    assert np.mean(losses[-50:]) < 0.5 * zero_loss
    assert np.mean(res_nn) < np.mean(res_rtm)
    assert np.mean(res_nn[:2]) < np.mean(res_ls)
