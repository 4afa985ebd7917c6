"""Golden vectors from an execution of the reference's PML Born modelling.

The reference's program 2d_rtm_restart/working_Src/born.f90 (born-mod.f90
with bornlib-mod.f90, pml-mod.f90, source-mod.f90, seis-mod-born.f90,
snap-mod-born.f90) is translated to C by oracle/f90c.py --set pml and
driven like its main program (oracle/refpml_driver.c).  This script runs it
on seeded models and commits inputs and outputs, so that the oracle
(tests/test_pml_oracle.py) and the GPU (tests/test_gpu_pml.py) are checked
against the reference on machines without the reference tree.  Needs the
reference tree; run once here:

    python tests/golden/make_golden_pml.py

refpml_small.npz -- per case "name/key": the parameters, the six model
  planes, the reference's six receiver lines and six snapshot cubes (small
  cases), or their SHA-256 digests (the multi-block case).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

F = np.float32

# (name, nz, nx, abc, zsource, xsource, zrec, nsnap, Ttime, fpeak, free_surface, lame, full outputs)
CASES = [
    ("odd", 37, 61, 8, 12, 30, 10, 4, 0.1, 60.0, False, False, True),
    ("surface", 48, 40, 10, 8, 21, 6, 3, 0.1, 60.0, True, False, True),
    ("lame", 40, 50, 6, 15, 24, 9, 3, 0.1, 60.0, False, True, True),
    ("noabc", 33, 45, 0, 16, 20, 12, 2, 0.08, 60.0, False, False, True),
    ("blocks", 150, 140, 20, 30, 70, 25, 3, 0.15, 40.0, False, False, False),
]
DX = 10.0


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, F).tobytes()).hexdigest()


def model(nz, nx, seed, lame):
    """Three layers with 2 % noise; perturbations of +-5 % with both signs,
    so that the set-up's dl, dmi < 1e-2 cut-off applies to some cells."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :]
    vp = (np.where(z < nz // 3, 2000.0, np.where(z < 2 * nz // 3, 2500.0, 3000.0)) * np.ones((nx, 1))
          * (1 + 0.02 * rng.standard_normal((nx, nz)))).astype(F)
    vs = (vp / 1.73).astype(F)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(F)
    dvp = (0.05 * vp * rng.standard_normal((nx, nz))).astype(F)
    dvs = (0.05 * vs * rng.standard_normal((nx, nz))).astype(F)
    drho = (0.05 * rho * rng.standard_normal((nx, nz))).astype(F)
    if lame:
        lam = (rho * (vp * vp - 2 * vs * vs)).astype(F)
        mu = (rho * vs * vs).astype(F)
        dlam = (0.05 * lam * rng.standard_normal((nx, nz))).astype(F)
        dmu = (0.05 * mu * rng.standard_normal((nx, nz))).astype(F)
        return lam, mu, rho, dlam, dmu, drho
    return vp, vs, rho, dvp, dvs, drho


def run_case(case):
    name, nz, nx, abc, zs, xs, zrec, nsnap, Tt, fp, fs, lame, full = case
    m = model(nz, nx, nz * 7 + nx, lame)
    P = O.pml_params(nz, nx, DX, Tt, fp=fp)
    seis, snap = O.refpml_born(*m, DX, P["dt"], P["nt"], xs, zs, P["nsource"], fp, nsnap, P["nseis"], abc, zrec,
                               fs, lame)
    return m, P, seis, snap


def main():
    O.build(ref=True)
    out = {}
    for case in CASES:
        name, nz, nx, abc, zs, xs, zrec, nsnap, Tt, fp, fs, lame, full = case
        m, P, seis, snap = run_case(case)
        out[name + "/geom"] = np.array([nz, nx, P["nt"], xs, zs, P["nsource"], nsnap, P["nseis"], abc, zrec, int(fs),
                                        int(lame)], np.int32)
        out[name + "/phys"] = np.array([DX, P["dt"], fp], F)
        out[name + "/model"] = np.stack(m)
        if full:
            out[name + "/seis"] = np.stack(seis)
            out[name + "/snap"] = np.stack(snap)
        out[name + "/seis_sha256"] = np.array([digest(a) for a in seis])
        out[name + "/snap_sha256"] = np.array([digest(a) for a in snap])
        print(name, "nt", P["nt"], "seis max", ["%.3g" % float(np.abs(a).max()) for a in seis])
    np.savez_compressed(os.path.join(HERE, "refpml_small.npz"), **out)


if __name__ == "__main__":
    main()
