"""Nonlinear elastic modelling (the reference's elastic.x time loop with
receivers at zrec) on the fused forward kernel, two rolling levels per
field: the gathers equal the rows zrec of the oracle's full forward history
bit for bit (exact arithmetic), for both kernel generations."""
import numpy as np
import pytest

import oracle as O
from elastic_gb300 import rtm as R
from elastic_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("version", [1, 2])
@pytest.mark.parametrize("nz,nx,nt,abc,zrec", [(60, 80, 120, 12, 6), (45, 37, 60, 20, 9)])
def test_nonlinear_modelling_matches_oracle_rows(version, nz, nx, nt, abc, zrec):
    R.set_kernel_version(version)
    try:
        vp = synth.smooth_random_model(nz, nx, 10.0, 80.0, 1800.0, 3200.0, seed=nz)
        rho, lam, mu = synth.lame_from_vp(vp)
        dx, dt, fp, ns, xsrc, zsrc = np.float32(10.0), np.float32(1e-3), np.float32(30.0), 40, nx // 2, 7
        coefs = list(O.coefficients(rho, lam, mu, dx, dt))
        src = O.source_op2(nt, dt, fp, ns)
        H = O.forward(coefs, nt, dt, zsrc, xsrc, src, abc, O.abc_init(abc))
        D = R.model(rho, lam, mu, 10.0, 1e-3, nt, xsrc, zsrc, zrec, 30.0, abc, ns)
        for c in range(5):
            np.testing.assert_array_equal(D[c], np.ascontiguousarray(H[c][:, :, zrec - 1].T))
        assert np.abs(D[0]).max() > 0
    finally:
        R.set_kernel_version(0)
