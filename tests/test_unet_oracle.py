"""The U-Net oracle (float64 numpy, hand-written backward) against float64
torch autograd of the same network: pins the oracle that the GPU gradient
check relies on."""
import numpy as np
import pytest

import unet_oracle as U

torch = pytest.importorskip("torch")
F = torch.nn.functional


def torch_net(params, x, t, table):
    Wb = U.unpack(params, table)
    Ws = [(torch.tensor(W, dtype=torch.float64, requires_grad=True), torch.tensor(b, dtype=torch.float64,
                                                                                  requires_grad=True)) for W, b in Wb]

    def conv(i, inp):
        W, b = Ws[i]
        ks, ci, co = table[i][0], table[i][1], table[i][2]
        k = W.reshape(co, ks, ks, ci).permute(0, 3, 1, 2)  # (co, ci, ky, kx)
        y = F.conv2d(inp, k, b, padding=ks // 2)
        return F.leaky_relu(y, U.LEAK) if i != 14 else y

    up = lambda z: F.interpolate(z, scale_factor=2, mode="nearest")
    pool = lambda z: F.avg_pool2d(z, 2)
    xt = torch.tensor(np.transpose(x, (0, 3, 1, 2)), dtype=torch.float64)
    a0 = conv(0, xt); a1 = conv(1, a0)
    a2 = conv(2, pool(a1)); a3 = conv(3, a2)
    a4 = conv(4, pool(a3)); a5 = conv(5, a4)
    a6 = conv(6, pool(a5)); a7 = conv(7, a6)
    a8 = conv(8, torch.cat([up(a7), a5], 1)); a9 = conv(9, a8)
    a10 = conv(10, torch.cat([up(a9), a3], 1)); a11 = conv(11, a10)
    a12 = conv(12, torch.cat([up(a11), a1], 1)); a13 = conv(13, a12)
    out = conv(14, a13)
    tt = torch.tensor(np.transpose(t, (0, 3, 1, 2)), dtype=torch.float64)
    loss = torch.mean((out - tt) ** 2)
    loss.backward()
    grad = np.zeros(len(params))
    for (W, b), row in zip(Ws, table):
        ks, ci, co, coutp, kp, woff, boff = row[:7]
        full = np.zeros((coutp, kp))
        full[:co, :ks * ks * ci] = W.grad.numpy()
        grad[woff:woff + coutp * kp] = full.ravel()
        grad[boff:boff + co] = b.grad.numpy()
    return float(loss), grad, np.transpose(out.detach().numpy(), (0, 2, 3, 1))


def test_unet_oracle_matches_torch_autograd():
    H = W = 16
    table, n = U.layer_table(H, W)
    rng = np.random.default_rng(0)
    params = np.zeros(n)
    for ks, ci, co, coutp, kp, woff, boff, _, _ in table:
        Wf = np.zeros((coutp, kp))
        Wf[:co, :ks * ks * ci] = rng.standard_normal((co, ks * ks * ci)) * np.sqrt(2.0 / (ks * ks * ci))
        params[woff:woff + coutp * kp] = Wf.ravel()
        params[boff:boff + co] = 0.1 * rng.standard_normal(co)
    x = rng.standard_normal((2, H, W, 3))
    t = rng.standard_normal((2, H, W, 3))
    loss, grad = U.loss_grad(params, x, t, table)
    out, _ = U.forward(params, x, table)
    tl, tg, tout = torch_net(params, x, t, table)
    np.testing.assert_allclose(out, tout, rtol=1e-10, atol=1e-12)
    assert loss == pytest.approx(tl, rel=1e-12)
    np.testing.assert_allclose(grad, tg, rtol=1e-9, atol=1e-14)


def test_unet_layer_table_sizes():
    table, n = U.layer_table(256, 256)
    assert 0.85e6 < n < 0.95e6  # ~0.9M parameters
    assert [r[3] for r in table] == [32, 32, 64, 64, 96, 96, 128, 128, 96, 96, 64, 64, 32, 32, 8]
    assert all(r[4] % 32 == 0 for r in table)
