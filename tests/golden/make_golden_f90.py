"""Golden vectors from an execution of the reference's Fortran RTM path.

The reference's modules (2d_rtm_restart/Src_working/rtm-mod-adj.f90 and the
modules it uses, with its C recursion rtmlib-modC.c) are translated to C by
oracle/f90c.py and driven like its main program (oracle/ref90_driver.c).
This script runs them on seeded inputs and commits inputs and outputs, so
that the oracle (tests/test_oracle.py) and the GPU (tests/test_gpu_config1.py,
tests/test_gpu_elastic2d.py) are checked against the reference on machines
without the reference tree.  Needs the reference tree; run once here:

    python tests/golden/make_golden_f90.py

ref90_small.npz -- per case "name/key": geometry, a perturbed layered model,
  a Born perturbation, the reference's five Born gathers for it, and the
  reference's RTM images of those gathers.
ref90_config1.npz -- the plain single-shot RTM case at full size: 400 x 200
  cells, dx = dz = 10 m, dt = 1 ms, nt = 2000, 40-cell sponge, 15 Hz Ricker
  at (x, z) = (2000 m, 50 m) = 1-based grid indices (201, 6), 400 receivers
  at z = 50 m (row 6), three-layer smoothed migration model with the 5%
  Gaussian-blob perturbation of the true model as the Born model.  Stored:
  the inputs; SHA-256 digests of the reference's five Born gathers; the
  reference's images of the Vx, Vz gathers (stress traces zeroed) and their
  digests; the same images and the relative L2 errors of the gathers and
  images computed by the float64 oracle (the reference's algorithm in
  double precision).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402

F = np.float32

# (name, nz, nx, nt, abc, zsrc, xsrc, zrec): an odd-sized grid, and one that
# crosses the GPU kernels' 128-row strips and several column tiles
SMALL = [("odd", 37, 45, 260, 8, 12, 23, 12), ("tiles", 150, 140, 260, 20, 22, 70, 22)]
DX, DT, FP = 10.0, 1e-3, 15.0


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, F).tobytes()).hexdigest()


def small_model(nz, nx, seed):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :]
    vp = np.where(z < nz // 3, 2000.0, np.where(z < 2 * nz // 3, 2800.0, 3500.0)) * np.ones((nx, 1))
    vp = vp * (1 + 0.02 * rng.standard_normal((nx, nz)))
    vs = vp / 1.73
    rho = (310.0 * vp ** 0.25).astype(F)
    lam = (rho * (vp ** 2 - 2 * vs ** 2)).astype(F)
    mu = (rho * vs ** 2).astype(F)
    dm = [(0.05 * rng.standard_normal((nx, nz)) * m).astype(F) for m in (rho, lam, mu)]
    return (rho, lam, mu), dm


def make_small():
    out = {}
    for name, nz, nx, nt, abc, zsrc, xsrc, zrec in SMALL:
        (rho, lam, mu), dm = small_model(nz, nx, seed=nz * 7 + nx)
        zero_d = [np.zeros((nx, nt), F)] * 5
        born = O.ref90_rtm(False, rho, lam, mu, dm, zero_d, DX, DT, nt, zsrc, xsrc, zrec, FP, abc)["D"]
        img = O.ref90_rtm(True, rho, lam, mu, [np.zeros((nx, nz), F)] * 3, born, DX, DT, nt, zsrc, xsrc, zrec,
                          FP, abc)["dm"]
        for tag, val in (("geom", np.array([nz, nx, nt, abc, zsrc, xsrc, zrec], np.int32)),
                         ("phys", np.array([DX, DT, FP], F)), ("rho", rho), ("lam", lam), ("mu", mu),
                         ("dm", np.stack(dm)), ("born", np.stack(born)), ("gathers", np.stack(born)),
                         ("image", np.stack(img))):
            if tag == "gathers":
                continue
            out["%s/%s" % (name, tag)] = val
        print(name, "born max", [float(np.abs(b).max()) for b in born], "image max",
              [float(np.abs(i).max()) for i in img])
    np.savez_compressed(os.path.join(HERE, "ref90_small.npz"), **out)


def rel(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a.astype(np.float64) - b) / n) if n > 0 else float(np.linalg.norm(a))


def make_config1():
    from elastic_gb300 import synth
    (rho, lam, mu), dm = synth.single_shot_models(nz=200, nx=400, seed=0)
    nx, nz = rho.shape
    nt, abc, zsrc, xsrc, zrec = 2000, 40, 6, 201, 6
    zero_d = [np.zeros((nx, nt), F)] * 5
    born = O.ref90_rtm(False, rho, lam, mu, dm, zero_d, DX, DT, nt, zsrc, xsrc, zrec, FP, abc)["D"]
    gathers = [born[0], born[1]] + [np.zeros((nx, nt), F)] * 3
    img = O.ref90_rtm(True, rho, lam, mu, [np.zeros((nx, nz), F)] * 3, gathers, DX, DT, nt, zsrc, xsrc, zrec,
                      FP, abc)["dm"]
    f8 = lambda L: [np.asarray(x, np.float64) for x in L]
    _, born8 = O.rtm_op2(False, *f8([rho, lam, mu]), f8(dm), f8(zero_d), DX, DT, nt, zsrc, xsrc, zrec, FP, abc, 250)
    img8, _ = O.rtm_op2(True, *f8([rho, lam, mu]), f8([np.zeros((nx, nz))] * 3), f8(gathers), DX, DT, nt, zsrc,
                        xsrc, zrec, FP, abc, 250)
    err_born = [rel(born[k], born8[k]) for k in range(5)]
    err_img = [rel(img[k], img8[k]) for k in range(3)]
    print("config1 Born rel. L2 vs float64:", err_born)
    print("config1 image rel. L2 vs float64:", err_img)
    np.savez_compressed(
        os.path.join(HERE, "ref90_config1.npz"),
        geom=np.array([nz, nx, nt, abc, zsrc, xsrc, zrec], np.int32), phys=np.array([DX, DT, FP], F),
        rho=rho, lam=lam, mu=mu, dm=np.stack(dm), born_sha256=np.array([digest(b) for b in born]),
        image=np.stack(img), image_sha256=np.array([digest(i) for i in img]), image_f64=np.stack(img8),
        born_err_f64=np.array(err_born), image_err_f64=np.array(err_img),
        born_norm=np.array([float(np.linalg.norm(b.astype(np.float64))) for b in born]))


if __name__ == "__main__":
    O.build(ref=True)
    make_small()
    if "--small-only" not in sys.argv:
        make_config1()
