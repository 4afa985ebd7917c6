"""Learned image-domain preconditioner: training pairs from the project's own
Born modelling and migration, U-Net training on the GPU, and evaluation by
the Born data residual against plain RTM and LSRTM.

A problem is one shot over a window of the background model.  Its Born
operator L maps a model perturbation (drho, dlambda, dmu) to the recorded
receiver gathers; the migrated image of a perturbation is L^T L dm (exact
adjoint).  The network maps the normalised 3-channel migrated image to the
relative perturbation r = dm / background (the reflectivity), i.e. it learns
an approximation of the inverse of the Born Hessian L^T L.

Image layout for the network: (n, nx, nz, 3) float32 (H = nx, W = nz).
Model planes follow the rest of the package: (nx, nz) per parameter.
"""
import time

import numpy as np

from . import rtm as R
from ._lib import check, load, ptr
from .unet import UNet


def smooth(a, sigma):
    """Separable Gaussian smoothing of a (nx, nz) plane (edge-replicating)."""
    if sigma <= 0:
        return a
    r = int(3 * sigma)
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k /= k.sum()
    out = np.asarray(a, np.float64)
    for ax in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[ax] = (r, r)
        p = np.pad(out, pad, mode="edge")
        out = sum(k[i] * np.take(p, np.arange(i, i + out.shape[ax]), axis=ax) for i in range(2 * r + 1))
    return out


def background_window(nx=256, nz=256, nz_model=200, smooth_cells=5.0):
    """Migration background: the three-layer model of the single-shot
    configuration (Vp 2000/2800/3500 m/s on nz_model rows), Gaussian-smoothed,
    as a (nx, nz) window extended below row nz_model by repeating the last row
    (a 256-cell window is deeper than the 200-row model)."""
    from . import synth
    vp = synth.layered_model(nz_model, nx, blob=0.0)
    if nz > nz_model:
        vp = np.concatenate([vp, np.repeat(vp[:, -1:], nz - nz_model, axis=1)], axis=1)
    vp = smooth(vp[:, :nz], smooth_cells)
    return synth.lame_from_vp(vp)


def random_reflectivity(rng, n, nx, nz, margin, amp=0.1, nlayers=(4, 10), nspikes=(2, 8), spread=0.5,
                        smooth_cells=1.0):
    """(n, 3, nx, nz) relative perturbations in [-amp, amp] of (rho, lambda,
    mu): dipping layer interfaces (2-4 cells thick, dip within 30 degrees)
    plus sparse spikes.  Each event has one amplitude a in [-amp, amp] and
    per-parameter factors in [1-spread, 1+spread] (the contrasts of the three
    parameters are correlated, as in rocks).  Gaussian-smoothed by
    smooth_cells and zero within `margin` cells of the edges (the sponge)."""
    r = np.zeros((n, 3, nx, nz), np.float32)
    xx, zz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    for i in range(n):
        for _ in range(rng.integers(nlayers[0], nlayers[1] + 1)):
            z0 = rng.uniform(margin, nz - margin)
            dip = np.tan(np.radians(rng.uniform(-30, 30)))
            th = rng.uniform(2.0, 4.0)
            mask = np.abs(zz - (z0 + dip * (xx - nx / 2))) < th / 2
            a = rng.uniform(-amp, amp) * rng.uniform(1 - spread, 1 + spread, 3)
            r[i][:, mask] += a[:, None]
        for _ in range(rng.integers(nspikes[0], nspikes[1] + 1)):
            x, z = rng.integers(margin, nx - margin), rng.integers(margin, nz - margin)
            r[i][:, x, z] += rng.uniform(-amp, amp) * rng.uniform(1 - spread, 1 + spread, 3)
        if smooth_cells > 0:
            for c in range(3):
                r[i, c] = smooth(r[i, c], smooth_cells)
    r = np.clip(r, -amp, amp)
    r[:, :, :margin] = 0
    r[:, :, nx - margin:] = 0
    r[:, :, :, :margin] = 0
    r[:, :, :, nz - margin:] = 0
    return r


class Problem:
    """One shot over a background window: Born modelling and migration of
    the recorded components (comp_mask bit c: Vx, Vz, sigmaxx, sigmazz,
    sigmaxz; the single-shot configuration records Vx and Vz)."""

    def __init__(self, rho, lam, mu, dx, dt, nt, xsrc, zsrc, zrec, fp, abc, nsource=250, comp_mask=3):
        self.rho, self.lam, self.mu = (np.ascontiguousarray(a, np.float32) for a in (rho, lam, mu))
        self.nx, self.nz = self.rho.shape
        self.dx, self.dt, self.nt = dx, dt, nt
        self.xsrc, self.zsrc, self.zrec = xsrc, zsrc, zrec
        self.fp, self.abc, self.nsource = fp, abc, nsource
        self.comp_mask = comp_mask
        self.bg = np.stack([self.rho, self.lam, self.mu])

    def _call(self, n, dm=None, data=None, data_in=None, img=None):
        check(load().rtm_born_migrate_c_(self.nz, self.nx, self.nt, self.dx, self.dt, self.xsrc, self.zsrc, self.zrec,
                                         self.fp, self.nsource, self.abc, self.comp_mask, ptr(self.rho), ptr(self.lam),
                                         ptr(self.mu), n, ptr(dm), ptr(data), ptr(data_in), ptr(img), 0))

    def born(self, dm):
        """(n, 3, nx, nz) perturbations -> (n, 5, nx, nt) gathers."""
        dm = np.ascontiguousarray(dm, np.float32)
        data = np.zeros((dm.shape[0], 5, self.nx, self.nt), np.float32)
        self._call(dm.shape[0], dm=dm, data=data)
        return data

    def migrate(self, data):
        data = np.ascontiguousarray(data, np.float32)
        img = np.zeros((data.shape[0], 3, self.nx, self.nz), np.float32)
        self._call(data.shape[0], data_in=data, img=img)
        return img

    def normal(self, dm):
        """Migrated images L^T L dm (n, 3, nx, nz) only."""
        dm = np.ascontiguousarray(dm, np.float32)
        img = np.zeros((dm.shape[0], 3, self.nx, self.nz), np.float32)
        self._call(dm.shape[0], dm=dm, img=img)
        return img

    def born_migrate(self, dm):
        dm = np.ascontiguousarray(dm, np.float32)
        n = dm.shape[0]
        data = np.zeros((n, 5, self.nx, self.nt), np.float32)
        img = np.zeros((n, 3, self.nx, self.nz), np.float32)
        self._call(n, dm=dm, data=data, img=img)
        return data, img

    def lsrtm(self, data, niter):
        """Plain LSRTM of one shot's gathers (5, nx, nt); (dm, resid, seconds)."""
        t0 = time.perf_counter()
        dm, resid = R.lsrtm(self.rho, self.lam, self.mu, data[None], [self.xsrc], [self.zsrc], self.zrec, self.dx,
                            self.dt, self.nt, self.fp, self.abc, niter=niter, nsource=self.nsource,
                            comp_mask=self.comp_mask)
        return dm, resid, time.perf_counter() - t0


def to_nhwc(a):
    return np.ascontiguousarray(np.transpose(a, (0, 2, 3, 1)), np.float32)


def from_nhwc(a):
    return np.ascontiguousarray(np.transpose(a, (0, 3, 1, 2)), np.float32)


class Preconditioner:
    """U-Net on normalised migrated images -> reflectivity.  The estimate is
    kept to the imaging region of the training targets: zero within
    `margin` cells of the edges (the sponge, where the source sits and the
    data are most sensitive to any model change)."""

    def __init__(self, nx, nz, batch=32, seed=0, margin=0, mask_input=True):
        self.net = UNet(nx, nz, batch, seed=seed)
        self.batch = batch
        self.margin = margin
        self.mask_input = mask_input
        self.in_scale = np.ones((3, 1), np.float32)
        self.clip = 0.0
        self.out_scale = np.float32(10.0)  # reflectivity is O(0.1)

    def fit_scales(self, img, mode="depth", clip=20.0):
        """Input normalisation from the training images (n, 3, nx, nz).
        mode "channel": one RMS per channel; "interior": one RMS per channel
        over the imaging region (outside `margin`); "depth": one RMS per
        channel and depth row over the imaging region's columns (a gain that
        compensates the decay of illumination with depth).  clip > 0 clips
        the normalised image to [-clip, clip] (the strong image next to the
        source)."""
        a = np.asarray(img, np.float64)
        m = self.margin
        inner = a[:, :, m:a.shape[2] - m, :] if m else a
        if mode == "channel":
            rms = np.sqrt(np.mean(a ** 2, axis=(0, 2, 3)))[:, None]
        elif mode == "interior":
            rms = np.sqrt(np.mean(inner[:, :, :, m:a.shape[3] - m] ** 2, axis=(0, 2, 3)))[:, None]
        elif mode == "depth":
            rms = np.sqrt(np.mean(inner ** 2, axis=(0, 2)))  # (3, nz)
            rms = np.maximum(rms, 1e-3 * rms.max(axis=1, keepdims=True))
        else:
            raise ValueError(mode)
        self.in_scale = (1.0 / np.maximum(rms, 1e-30)).astype(np.float32)
        self.clip = clip

    def inputs(self, img):
        """Normalised network input; with mask_input, zero outside the
        imaging region (the image next to the source and in the sponge
        carries no information on the targets, which are zero there)."""
        s = self.in_scale
        x = img * s[None, :, None, :]
        if self.clip:
            x = np.clip(x, -self.clip, self.clip)
        if self.mask_input and self.margin:
            m = self.margin
            x = x.copy()
            x[:, :, :m] = 0
            x[:, :, x.shape[2] - m:] = 0
            x[:, :, :, :m] = 0
            x[:, :, :, x.shape[3] - m:] = 0
        return to_nhwc(x)

    def train(self, img, refl, steps, lr=1e-3, seed=0, log_every=0):
        """Adam on random batches of (image, reflectivity) pairs held on the
        device; returns the per-step losses."""
        import torch
        x = torch.from_numpy(self.inputs(img)).cuda()
        y = torch.from_numpy(to_nhwc(refl * self.out_scale)).cuda()
        rng = np.random.default_rng(seed)
        n = x.shape[0]
        losses = []
        for s in range(steps):
            idx = torch.from_numpy(rng.choice(n, size=min(self.batch, n), replace=False)).cuda()
            losses.append(self.net.train_step(x.index_select(0, idx).contiguous(), y.index_select(0, idx).contiguous(),
                                              lr=lr))
            if log_every and s % log_every == 0:
                print("step", s, "loss", losses[-1], flush=True)
        return losses

    def apply(self, img, bg):
        """Migrated images (n, 3, nx, nz) -> model perturbations dm = bg * r."""
        out = []
        for i in range(0, img.shape[0], self.batch):
            out.append(from_nhwc(self.net.forward(self.inputs(img[i:i + self.batch]))))
        r = np.concatenate(out) / self.out_scale
        if self.margin:
            m = self.margin
            r[:, :, :m] = 0
            r[:, :, r.shape[2] - m:] = 0
            r[:, :, :, :m] = 0
            r[:, :, :, r.shape[3] - m:] = 0
        return r * bg[None]


def residual(problem, dm, d):
    """||L dm - d|| / ||d|| per pair."""
    pred = problem.born(dm)
    return np.linalg.norm((pred - d).reshape(len(d), -1), axis=1) / np.linalg.norm(d.reshape(len(d), -1), axis=1)


def scaled_residual(problem, m, d):
    """Born residual of the best scalar multiple of m (per pair)."""
    Lm = problem.born(m).astype(np.float64)
    out = []
    for k in range(len(d)):
        a = float(np.vdot(Lm[k], d[k])) / max(float(np.vdot(Lm[k], Lm[k])), 1e-300)
        out.append(np.linalg.norm(a * Lm[k] - d[k]) / np.linalg.norm(d[k]))
    return np.array(out)
