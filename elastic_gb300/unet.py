"""Learned image-domain preconditioner (4-level 3->3 channel U-Net, BF16
tensor-core training and inference kernels in libelastic_rtm.so)."""
import ctypes

import numpy as np

from ._lib import check, load, ptr


GEMMS = {"mma_sync": 0, "tcgen05": 1, "tcgen05_tma": 2}


def set_gemm(kind="tcgen05_tma"):
    """GEMM kernel of the forward and backward-data passes: "tcgen05_tma"
    (default: tcgen05 MMAs, 3x3 convolutions fed by bulk tensor copies of
    shifted activation boxes), "tcgen05" (operands gathered by threads) or
    "mma_sync"."""
    check(load().unet_set_gemm(GEMMS[kind]))


class UNet:
    """unet_create/unet_* of the C-ABI.  Images are float32 NHWC
    (n, H, W, 3); parameters one flat float32 vector."""

    NLAYERS = 15

    def __init__(self, H, W, max_batch, seed=0):
        self.H, self.W, self.max_batch = H, W, max_batch
        self.h = load().unet_create(H, W, max_batch, seed)
        if not self.h:
            check(3)
        self.nparam = int(load().unet_num_params(self.h))

    def layer_table(self):
        out = []
        info = np.zeros(9, np.int64)
        for i in range(self.NLAYERS):
            check(load().unet_layer_info(self.h, i, ptr(info)))
            out.append(tuple(int(v) for v in info))
        return out

    def get_params(self):
        w = np.zeros(self.nparam, np.float32)
        check(load().unet_get_params(self.h, ptr(w)))
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.shape == (self.nparam,)
        check(load().unet_set_params(self.h, ptr(w)))

    def _x(self, x):
        if hasattr(x, "data_ptr"):
            return x, 1
        return np.ascontiguousarray(x, np.float32), 0

    def forward(self, x):
        x, dev = self._x(x)
        n = x.shape[0]
        if dev:
            import torch
            y = torch.empty((n, self.H, self.W, 3), dtype=torch.float32, device=x.device)
        else:
            y = np.zeros((n, self.H, self.W, 3), np.float32)
        check(load().unet_forward(self.h, ptr(x), n, ptr(y), dev))
        return y

    def loss_grad(self, x, t):
        x, dev = self._x(x)
        t, _ = self._x(t)
        loss = ctypes.c_double(0)
        g = np.zeros(self.nparam, np.float32)
        check(load().unet_loss_grad(self.h, ptr(x), ptr(t), x.shape[0], dev, ctypes.byref(loss), ptr(g)))
        return loss.value, g

    def train_step(self, x, t, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        x, dev = self._x(x)
        t, _ = self._x(t)
        loss = ctypes.c_double(0)
        check(load().unet_train_step(self.h, ptr(x), ptr(t), x.shape[0], dev, lr, beta1, beta2, eps,
                                     ctypes.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            load().unet_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
