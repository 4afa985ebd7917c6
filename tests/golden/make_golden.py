"""Generate golden vectors for the adjoint recursion from the reference itself.

Runs the reference's own rtm_op3_c_ (2d_rtm_restart/Src_working/rtmlib-modC.c,
compiled CPU-only by oracle/Makefile into oracle/_ref/librefc.so) on seeded
inputs and stores inputs and outputs in rtm_op3_c_ref.npz.  A second
fixture, rtm_op3_c_sizes.npz, covers odd sizes, several GPU tiles and a slice
of the single-shot grid (400 x 200): its inputs come from detgen.field
(reproducible on every platform), so it stores only salts and the SHA-256
digest of the reference's output.  Needs the reference tree; run once here,
the fixtures are committed.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402


def make(seed=20151203, nz=16, nx=16, nt=59):
    rng = np.random.default_rng(seed)
    # physically scaled coefficients (dt/dx * lambda etc. ~ O(1e-1)) and a
    # sparse receiver-like input: random levels, as the C receives them
    coefs = [(0.05 + 0.05 * rng.random((nx, nz))).astype(np.float32) for _ in range(5)]
    H = [(rng.standard_normal((nt, nx, nz))).astype(np.float32) for _ in range(5)]
    Hin = [h.copy() for h in H]
    O.ref_rtm_op3_c(H, coefs)
    return coefs, Hin, H


# (nz, nx, nt): odd, one 128-row strip plus a partial one across several
# column tiles, and the single-shot grid over a short window (the
# reference C divides by nt/59 in its progress output: nt >= 59)
SIZES = [(37, 45, 64), (160, 128, 60), (200, 400, 60)]


def sizes_inputs(nz, nx, nt):
    import detgen
    salt = nz * 1000003 + nx * 1009 + nt
    coefs = [detgen.field((nx, nz), salt + k, 0.05, 0.1) for k in range(5)]
    H = [detgen.field((nt, nx, nz), salt + 10 + k) for k in range(5)]
    return coefs, H


def make_sizes():
    import detgen
    out = {}
    for nz, nx, nt in SIZES:
        coefs, H = sizes_inputs(nz, nx, nt)
        O.ref_rtm_op3_c(H, coefs)
        out["%dx%dx%d" % (nz, nx, nt)] = np.array(detgen.digest(H))
    np.savez(os.path.join(HERE, "rtm_op3_c_sizes.npz"), **out)
    print("wrote rtm_op3_c_sizes.npz", sorted(out))


if __name__ == "__main__":
    O.build(ref=True)
    sys.path.insert(0, HERE)
    make_sizes()
    coefs, Hin, Hout = make()
    np.savez_compressed(os.path.join(HERE, "rtm_op3_c_ref.npz"), coefs=np.stack(coefs), hin=np.stack(Hin),
                        hout=np.stack(Hout))
    print("wrote rtm_op3_c_ref.npz", np.stack(Hout).shape, float(np.abs(np.stack(Hout)).max()))
