"""CPU oracle (test infrastructure only) of the learned image preconditioner:
the 4-level 3->3 channel U-Net of elastic_gb300/csrc/unet.cu in float64
numpy, forward and hand-written backward, on the same flat parameter vector.

There is no reference implementation of this network (lgan/elastic only
intends an iterative solver, 2d_rtm_restart/Src_working/rtm-mod-adj.f90:5-7);
the oracle is pinned instead by a float64 torch autograd check in the CPU
tests.  Layout conventions (shared with the CUDA code):
  * images NHWC (n, H, W, C);
  * a 3x3 layer's weights [coutp][kp], k = (ky*3 + kx)*cin + ci, zero beyond
    9*cin, then the bias [coutp]; the 1x1 output layer [8][32] + bias [8]
    (rows >= 3 unused);
  * concatenation order [upsampled coarse level | skip].
"""
import numpy as np

CH = (32, 64, 96, 128)
LEAK = 0.1  # negative-side slope of the leaky ReLU


def layer_table(H, W, cin=3, cout=3, ch=CH):
    """(ks, cin, cout, coutp, kp, woff, boff, H, W) per layer, in order
    e1a e1b e2a e2b e3a e3b ba bb d3a d3b d2a d2b d1a d1b out."""
    c = ch
    spec = [(3, cin, c[0], 0), (3, c[0], c[0], 0), (3, c[0], c[1], 1), (3, c[1], c[1], 1), (3, c[1], c[2], 2),
            (3, c[2], c[2], 2), (3, c[2], c[3], 3), (3, c[3], c[3], 3), (3, c[3] + c[2], c[2], 2), (3, c[2], c[2], 2),
            (3, c[2] + c[1], c[1], 1), (3, c[1], c[1], 1), (3, c[1] + c[0], c[0], 0), (3, c[0], c[0], 0),
            (1, c[0], cout, 0)]
    out, off = [], 0
    for ks, ci, co, lvl in spec:
        coutp = 8 if ks == 1 else co
        kp = (9 * ci + 31) // 32 * 32 if ks == 3 else (ci + 31) // 32 * 32
        woff = off
        off += coutp * kp
        boff = off
        off += coutp
        out.append((ks, ci, co, coutp, kp, woff, boff, H >> lvl, W >> lvl))
    return out, off


def unpack(params, table):
    """[(Wk (cout, ks*ks*cin), b (cout))] from the flat vector."""
    res = []
    for ks, ci, co, coutp, kp, woff, boff, _, _ in table:
        Wf = np.asarray(params[woff:woff + coutp * kp], np.float64).reshape(coutp, kp)
        res.append((Wf[:co, :ks * ks * ci].copy(), np.asarray(params[boff:boff + co], np.float64).copy()))
    return res


def im2col3(x):
    """x (n,H,W,C) -> cols (n*H*W, 9C), column (ky*3+kx)*C + c, zero padding 1."""
    n, H, W, C = x.shape
    xp = np.zeros((n, H + 2, W + 2, C))
    xp[:, 1:-1, 1:-1] = x
    cols = np.empty((n, H, W, 9, C))
    for ky in range(3):
        for kx in range(3):
            cols[:, :, :, ky * 3 + kx] = xp[:, ky:ky + H, kx:kx + W]
    return cols.reshape(n * H * W, 9 * C)


def col2im3(cols, shape):
    """Adjoint of im2col3."""
    n, H, W, C = shape
    c = cols.reshape(n, H, W, 9, C)
    xp = np.zeros((n, H + 2, W + 2, C))
    for ky in range(3):
        for kx in range(3):
            xp[:, ky:ky + H, kx:kx + W] += c[:, :, :, ky * 3 + kx]
    return xp[:, 1:-1, 1:-1].copy()


def pool(x):
    n, H, W, C = x.shape
    return x.reshape(n, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_bwd(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(g):
    n, H, W, C = g.shape
    return g.reshape(n, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward(params, x, table):
    """Returns (output (n,H,W,3), cache)."""
    Wb = unpack(params, table)
    cache = {}
    a = {}

    def conv(i, inp):
        Wk, b = Wb[i]
        ks = table[i][0]
        n, H, W, C = inp.shape
        cols = im2col3(inp) if ks == 3 else inp.reshape(-1, C)
        z = cols @ Wk.T + b
        cache[i] = (inp, cols)
        y = np.where(z > 0, z, LEAK * z) if i != 14 else z
        return y.reshape(n, H, W, -1)

    a[0] = conv(0, np.asarray(x, np.float64))
    a[1] = conv(1, a[0])
    a[2] = conv(2, pool(a[1]))
    a[3] = conv(3, a[2])
    a[4] = conv(4, pool(a[3]))
    a[5] = conv(5, a[4])
    a[6] = conv(6, pool(a[5]))
    a[7] = conv(7, a[6])
    a[8] = conv(8, np.concatenate([up(a[7]), a[5]], axis=3))
    a[9] = conv(9, a[8])
    a[10] = conv(10, np.concatenate([up(a[9]), a[3]], axis=3))
    a[11] = conv(11, a[10])
    a[12] = conv(12, np.concatenate([up(a[11]), a[1]], axis=3))
    a[13] = conv(13, a[12])
    out = conv(14, a[13])
    cache["a"] = a
    return out, cache


def loss_grad(params, x, t, table):
    """Mean squared error and its gradient, flat like params."""
    out, cache = forward(params, x, table)
    a = cache["a"]
    Wb = unpack(params, table)
    t = np.asarray(t, np.float64)
    d = out - t
    loss = float(np.mean(d * d))
    grad = np.zeros(len(params))
    n = x.shape[0]

    def conv_bwd(i, gy, y):
        """gy: gradient of layer i's output (n,H,W,cout); y its output."""
        ks, ci, co, coutp, kp, woff, boff, H, W = table[i]
        g = gy.reshape(-1, co)
        if i != 14:
            g = g * np.where(y.reshape(-1, co) > 0, 1.0, LEAK)
        inp, cols = cache[i]
        dW = g.T @ cols
        full = np.zeros((coutp, kp))
        full[:co, :dW.shape[1]] = dW
        grad[woff:woff + coutp * kp] = full.ravel()
        grad[boff:boff + co] = g.sum(axis=0)
        dcols = g @ Wb[i][0]
        if ks == 3:
            return col2im3(dcols, inp.shape)
        return dcols.reshape(inp.shape)

    c = CH
    g_out = 2.0 * d / d.size
    g13 = conv_bwd(14, g_out, out)
    g12 = conv_bwd(13, g13, a[13])
    gcat0 = conv_bwd(12, g12, a[12])
    g11 = up_bwd(gcat0[..., :c[1]])
    g1 = gcat0[..., c[1]:].copy()
    g10 = conv_bwd(11, g11, a[11])
    gcat1 = conv_bwd(10, g10, a[10])
    g9 = up_bwd(gcat1[..., :c[2]])
    g3 = gcat1[..., c[2]:].copy()
    g8 = conv_bwd(9, g9, a[9])
    gcat2 = conv_bwd(8, g8, a[8])
    g7 = up_bwd(gcat2[..., :c[3]])
    g5 = gcat2[..., c[3]:].copy()
    g6 = conv_bwd(7, g7, a[7])
    gp2 = conv_bwd(6, g6, a[6])
    g5 = g5 + pool_bwd(gp2)
    g4 = conv_bwd(5, g5, a[5])
    gp1 = conv_bwd(4, g4, a[4])
    g3 = g3 + pool_bwd(gp1)
    g2 = conv_bwd(3, g3, a[3])
    gp0 = conv_bwd(2, g2, a[2])
    g1 = g1 + pool_bwd(gp0)
    g0 = conv_bwd(1, g1, a[1])
    conv_bwd(0, g0, a[0])
    del n
    return loss, grad


def bf16_round(x):
    """Round float values to bfloat16 (nearest-even), returned as float64."""
    f = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((f + 0x7FFF + ((f >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)
