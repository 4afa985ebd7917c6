"""Seeded synthetic models and surveys with the sizes and value ranges of the
benchmark configurations (no public data is used).

* ``layered_model`` -- three layers Vp 2000/2800/3500 m/s with a 5% Gaussian
  blob, Vs = Vp/1.73, Gardner density rho = 310 Vp^0.25.
* ``smooth_random_model`` -- Vp in [vmin, vmax] from Gaussian-filtered white
  noise with the given correlation length.
* ``uneven_survey`` -- shots at a fixed spacing, each on a subgrid of seeded
  width in [wmin, wmax] centred on the source and clipped to the grid.
* ``dipping_reflectivity`` -- a seeded relative perturbation of a few
  dipping reflectors and point scatterers, the "true model minus background"
  of the survey workloads.
* ``single_shot_models`` -- the plain single-shot RTM case: migration model
  (smoothed three-layer Lame parameters) and the Born perturbation that the
  5% Gaussian blob of the true model adds to it.
"""
import numpy as np


def lame_from_vp(vp, vs_ratio=1.73):
    vs = vp / vs_ratio
    rho = 310.0 * vp ** 0.25
    lam = rho * (vp ** 2 - 2.0 * vs ** 2)
    mu = rho * vs ** 2
    return rho.astype(np.float32), lam.astype(np.float32), mu.astype(np.float32)


def layered_model(nz, nx, seed=0, blob=0.05):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :]
    vp = np.where(z < nz // 3, 2000.0, np.where(z < 2 * nz // 3, 2800.0, 3500.0)) * np.ones((nx, 1))
    if blob:
        xx, zz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
        cx, cz = nx * rng.uniform(0.3, 0.7), nz * rng.uniform(0.4, 0.6)
        vp = vp * (1 + blob * np.exp(-((xx - cx) ** 2 + (zz - cz) ** 2) / (2 * (nz / 10) ** 2)))
    return vp


def smooth_random_model(nz, nx, dx, corr_len=200.0, vmin=1800.0, vmax=4000.0, seed=0):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nx, nz))
    kx = np.fft.fftfreq(nx, d=dx)[:, None]
    kz = np.fft.rfftfreq(nz, d=dx)[None, :]
    filt = np.exp(-2.0 * (np.pi * corr_len) ** 2 * (kx ** 2 + kz ** 2) / 4.0)
    s = np.fft.irfft2(np.fft.rfft2(w) * filt, s=(nx, nz))
    s = (s - s.min()) / (s.max() - s.min())
    return vmin + (vmax - vmin) * s


def uneven_survey(nx, nshots, spacing, wmin, wmax, first=None, seed=0):
    """Returns 1-based (x0, widths, xsrc) arrays."""
    rng = np.random.default_rng(seed)
    span = (nshots - 1) * spacing
    first = (nx - span) // 2 if first is None else first
    xs = first + spacing * np.arange(nshots)
    widths = rng.integers(wmin, wmax + 1, nshots)
    x0 = np.clip(xs - widths // 2, 0, None)
    x0 = np.minimum(x0, nx - widths)
    return (x0 + 1).astype(np.int32), widths.astype(np.int32), (xs + 1).astype(np.int32)


def synthetic_traces(n, seed=0):
    """Seeded float32 trace samples (content does not affect the cost)."""
    rng = np.random.default_rng(seed)
    return (1e-3 * rng.standard_normal(n)).astype(np.float32)


def gaussian_smooth(a, sigma):
    """Gaussian smoothing of a plane (sigma in cells), edges extended by their
    last value so the smoothing does not bend the model at the border."""
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(np.asarray(a, np.float64), sigma, mode="nearest")


def single_shot_models(nz=200, nx=400, seed=0, blob=0.05, smooth_cells=5.0):
    """Migration model and true-model perturbation of the single-shot RTM
    case: three layers Vp 2000/2800/3500 m/s smoothed by a Gaussian of
    `smooth_cells` cells, Vs = Vp/1.73, Gardner density; the true model
    multiplies the smoothed Vp by a seeded Gaussian blob of relative size
    `blob`.  Returns ((rho, lam, mu), (drho, dlam, dmu)) as float32 [nx, nz]
    planes (z fastest), the perturbation being true minus migration model."""
    layers = layered_model(nz, nx, seed=seed, blob=0.0)
    vp0 = gaussian_smooth(layers, smooth_cells)
    vp1 = layered_model(nz, nx, seed=seed, blob=blob) / layers * vp0
    m0 = lame_from_vp(vp0)
    m1 = lame_from_vp(vp1)
    dm = tuple((b.astype(np.float64) - a.astype(np.float64)).astype(np.float32) for a, b in zip(m0, m1))
    return m0, dm


def dipping_reflectivity(nz, nx, seed=0, n_layers=6, n_points=20, amp=0.05, top=20, bottom=None):
    """Relative perturbation [nx, nz]: `n_layers` dipping reflectors (one
    cell thick, slopes within +-15 degrees, amplitudes within +-amp) and
    `n_points` point scatterers, all between rows `top` and `bottom`
    (default: 5 rows above the bottom of the grid)."""
    rng = np.random.default_rng(seed)
    bottom = nz - 5 if bottom is None else min(bottom, nz - 5)
    r = np.zeros((nx, nz))
    x = np.arange(nx)
    for _ in range(n_layers):
        z0 = rng.uniform(top, bottom)
        slope = np.tan(np.radians(rng.uniform(-15.0, 15.0)))
        z = np.round(z0 + slope * (x - nx / 2)).astype(int)
        ok = (z >= top) & (z < bottom)
        r[x[ok], z[ok]] += rng.uniform(-amp, amp)
    for _ in range(n_points):
        r[rng.integers(5, nx - 5), rng.integers(top, bottom)] += rng.uniform(-amp, amp)
    return r
