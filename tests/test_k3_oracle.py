"""The oracle's 3D elastic step against the reference's own test of its 3D
elastic kernel (kernel_3d_test/rtmlib-modC.c): the reference's main --
seeded random 200^3 fields, the GPU hand-off, its CPU step, func_check at
1e-13 on all nine fields -- compiled unchanged with the hand-off served by
the oracle (oracle/k3_shim.c).  A planted one-ulp mistake in the oracle's
output must be reported."""
import os

import pytest

import oracle as O

pytestmark = pytest.mark.skipif(
    not (os.path.exists(O.K3_CHECK) or (O.ref_root() and os.path.isdir(os.path.join(O.ref_root(), "kernel_3d_test")))),
    reason="reference tree not present")


def _binary():
    if not os.path.exists(O.K3_CHECK):
        O.build(ref=True)
    return O.K3_CHECK


def test_reference_check_passes_with_oracle_step():
    err = _binary() and O.k3_reference_check()
    print(err[-600:])
    assert err.count("Check Okay") == 9


def test_reference_check_reports_planted_mistake():
    err = _binary() and O.k3_reference_check(plant=True)
    assert err.count("Check Okay") == 8
