"""Generate golden vectors for the adjoint recursion from the reference itself.

Runs the reference's own rtm_op3_c_ (2d_rtm_restart/Src_working/rtmlib-modC.c,
compiled CPU-only by oracle/Makefile into oracle/_ref/librefc.so) on seeded
inputs and stores inputs and outputs in rtm_op3_c_ref.npz.  Needs the
reference tree; run once here, the fixture is committed.

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


if __name__ == "__main__":
    O.build(ref=True)
    coefs, Hin, Hout = make()
    np.savez_compressed(os.path.join(HERE, "rtm_op3_c_ref.npz"), coefs=np.stack(coefs), hin=np.stack(Hin),
                        hout=np.stack(Hout))
    print("wrote rtm_op3_c_ref.npz", np.stack(Hout).shape, float(np.abs(np.stack(Hout)).max()))
