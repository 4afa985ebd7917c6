"""GPU U-Net (BF16 tensor-core GEMMs, FP32 accumulation) against the float64
oracle: forward output, loss and per-layer gradients; Adam training reduces
the loss."""
import numpy as np
import pytest

import unet_oracle as U
from elastic_gb300.unet import UNet, set_gemm

pytestmark = pytest.mark.gpu

# BF16 activations (8-bit mantissa, relative rounding 2^-9 per value) through
# 15 layers: outputs and gradients agree with the float64 oracle (fed the same
# BF16-rounded weights and input) to these relative L2 errors
RTOL_OUT = 2e-2
RTOL_GRAD = 6e-2


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def setup(H=32, W=32, n=2, seed=3):
    net = UNet(H, W, n, seed=seed)
    table, nparam = U.layer_table(H, W)
    assert net.layer_table() == table and net.nparam == nparam
    rng = np.random.default_rng(seed)
    p = net.get_params().astype(np.float64)
    for r in table:  # non-zero biases exercise the bias paths
        p[r[6]:r[6] + r[2]] = 0.05 * rng.standard_normal(r[2])
    p = U.bf16_round(p)  # the GPU computes with BF16 weights
    net.set_params(p.astype(np.float32))
    x = U.bf16_round(rng.standard_normal((n, H, W, 3))).astype(np.float32)
    t = rng.standard_normal((n, H, W, 3)).astype(np.float32)
    return net, table, p, x, t


@pytest.fixture(autouse=True, params=["tcgen05_tma", "tcgen05", "mma_sync"])
def gemm_path(request):
    """Every test runs with each GEMM kernel of the forward and
    backward-data passes."""
    set_gemm(request.param)
    yield request.param
    set_gemm()


@pytest.mark.parametrize("hw", [(64, 64, 2), (256, 256, 1), (128, 256, 1)])
def test_gemm_paths_agree(hw):
    """The GEMM kernels accumulate the same BF16 products in FP32 in
    different orders: network outputs and gradients agree closely (the BF16
    rounding of activations can flip on either side of a tie).  The sizes
    take the bulk-copy convolution through its whole-row tiles (W <= 128)
    and its row-segment tiles (W = 256)."""
    H, W, n = hw
    net, table, p, x, t = setup(H=H, W=W, n=n, seed=5)
    out = {}
    for kind in ("tcgen05_tma", "tcgen05", "mma_sync"):
        set_gemm(kind)
        y = net.forward(x)
        _, g = net.loss_grad(x, t)
        out[kind] = (y, g)
    y_ms, g_ms = out["mma_sync"]
    assert np.abs(y_ms).max() > 0
    for kind in ("tcgen05_tma", "tcgen05"):
        e_y, e_g = rel(out[kind][0], y_ms), rel(out[kind][1], g_ms)
        print("%s vs mma.sync at %dx%d: output rel. L2 %.2e, gradient %.2e" % (kind, H, W, e_y, e_g))
        assert e_y < 5e-3 and e_g < 2e-2
    net.close()


def test_unet_forward_matches_oracle():
    net, table, p, x, t = setup()
    y = net.forward(x)
    ref, _ = U.forward(p, x.astype(np.float64), table)
    e = rel(y, ref)
    print("forward rel L2", e)
    assert e < RTOL_OUT
    net.close()


def test_unet_gradients_match_oracle():
    net, table, p, x, t = setup()
    loss, g = net.loss_grad(x, t)
    rl, rg = U.loss_grad(p, x.astype(np.float64), t.astype(np.float64), table)
    print("loss", loss, rl)
    assert loss == pytest.approx(rl, rel=RTOL_OUT)
    errs = []
    for i, r in enumerate(table):
        ks, ci, co, coutp, kp, woff, boff = r[:7]
        ew = rel(g[woff:woff + coutp * kp], rg[woff:woff + coutp * kp])
        eb = rel(g[boff:boff + co], rg[boff:boff + co])
        errs.append((i, round(ew, 4), round(eb, 4)))
    print("per-layer gradient rel L2 (weights, bias):", errs)
    assert max(max(e[1], e[2]) for e in errs) < RTOL_GRAD
    # padding of the weight matrices gets no gradient
    for r in table:
        ks, ci, co, coutp, kp, woff = r[:6]
        Wg = g[woff:woff + coutp * kp].reshape(coutp, kp)
        assert not Wg[:, ks * ks * ci:].any() and not Wg[co:].any()
    net.close()


def test_unet_adam_training_reduces_loss():
    H = W = 32
    net = UNet(H, W, 4, seed=1)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((4, H, W, 3)).astype(np.float32)
    # a smooth, learnable target: a local average of the input
    k = np.ones((3, 3)) / 9.0
    t = np.zeros_like(x)
    for dy in range(3):
        for dx in range(3):
            t += k[dy, dx] * np.roll(np.roll(x, dy - 1, axis=1), dx - 1, axis=2)
    losses = [net.train_step(x, t, lr=1e-3) for _ in range(150)]
    print("loss", losses[0], "->", losses[-1])
    assert losses[-1] < 0.2 * losses[0]
    net.close()
