"""GPU split-field PML Born modelling (pml_born_c_, pml_born_dev) against
the reference's execution and the oracle: bit-exact receiver lines and
snapshots on the committed reference fixtures (tests/golden/
refpml_small.npz), on further sizes against the oracle (which is pinned to
the reference by tests/test_pml_oracle.py), and an exact size-independent
property on the 2000 x 800 survey grid."""
import os
import sys

import numpy as np
import pytest

import oracle as O
from elastic_gb300 import pml

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden_pml as G  # noqa: E402
from test_pml_oracle import (CASES, EDGE_CASES, GOLD, case_args, check_against_fixture, edge_case_args,  # noqa: E402
                             same_bits)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_fixtures(gold, name):
    m, kw = case_args(gold, name)
    seis, snap = pml.born(*m, **kw)
    check_against_fixture(gold, name, seis, snap)
    assert pml.launches() >= 2 * kw["nt"]


@pytest.fixture(params=list(pml.KERNELS))
def kernel(request):
    pml.set_kernel(request.param)
    yield request.param
    pml.set_kernel()


@pytest.mark.parametrize("nz,nx,abc,fs,lame,seed", [
    (29, 30, 12, False, False, 1),    # left and right PML columns overlap
    (26, 52, 11, True, False, 2),     # top and bottom PML rows overlap
    (11, 11, 0, False, False, 3),     # smallest grid
    (130, 97, 16, False, True, 4),    # ragged against the 32 x 8 blocks
    (257, 66, 30, True, False, 5),
])
def test_gpu_matches_oracle(nz, nx, abc, fs, lame, seed, kernel):
    m = G.model(nz, nx, seed, lame)
    P = O.pml_params(nz, nx, 10.0, 0.08, fp=60.0)
    kw = dict(dx=10.0, dt=P["dt"], nt=P["nt"], xsource=max(1, nx // 2), zsource=min(12, nz - 3),
              nsource=P["nsource"], fp=60.0, nsnap=3, nseis=P["nseis"], abc=abc, zrec=min(8, nz), free_surface=fs,
              lame=lame)
    os_, oc = O.pml_born(*m, **kw)
    gs, gc = pml.born(*m, **kw)
    for k in range(6):
        assert same_bits(gs[k], os_[k]), ("seis", O.PML_SEIS[k])
        assert same_bits(gc[k], oc[k]), ("snap", O.PML_SEIS[k])


@pytest.mark.parametrize("case", EDGE_CASES, ids=lambda c: "%dx%d_abc%d_seed%d" % (c[0], c[1], c[2], c[5]))
def test_gpu_edge_cases_match_oracle(case):
    """The edge cases the oracle is held to against the reference (widest
    PML, sources outside the operators' ranges and inside the PML,
    receivers on the second and the last row), GPU against the oracle."""
    m, kw = edge_case_args(*case)
    os_, oc = O.pml_born(*m, **kw)
    gs, gc = pml.born(*m, **kw)
    for k in range(6):
        assert same_bits(gs[k], os_[k]) and same_bits(gc[k], oc[k]), O.PML_SEIS[k]


def test_device_entry_matches_host_entry(gold):
    import torch
    m, kw = case_args(gold, "odd")
    hs, hc = pml.born(*m, **kw)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in m]
    nx, nz = m[0].shape
    seis = [torch.full((nx - 2 * kw["abc"], kw["nseis"]), 7.0, device="cuda") for _ in range(6)]
    snap = [torch.full((kw["nsnap"], nx, nz), 7.0, device="cuda") for _ in range(6)]
    args = {k: v for k, v in kw.items() if k not in ("nsnap", "nseis")}
    pml.born_dev(dev, seis, snap, **args)
    torch.cuda.synchronize()
    for k in range(6):
        assert same_bits(seis[k].cpu().numpy(), hs[k]) and same_bits(snap[k].cpu().numpy(), hc[k])


def test_tile_wait_limit_reports_status_4(gold):
    """The staged-tile form's bounded wait: a flag that nothing sets makes
    its first launch give up after about a second; the call returns status
    4, and the next call (hook off) gives the reference's bits again."""
    from elastic_gb300._lib import RtmError
    m, kw = case_args(gold, "noabc")
    pml.set_kernel("tile-prefetch")
    try:
        pml.set_test_stall(True)
        with pytest.raises(RtmError, match="status 4"):
            pml.born(*m, **kw)
        pml.set_test_stall(False)
        seis, snap = pml.born(*m, **kw)
        check_against_fixture(gold, "noabc", seis, snap)
    finally:
        pml.set_test_stall(False)
        pml.set_kernel()


def survey_grid_case(seed=11):
    """2000 x 800 cells (the survey grid), two layers, 60-cell PML."""
    nz, nx = 800, 2000
    rng = np.random.default_rng(seed)
    vp = np.full((nx, nz), 2500.0, np.float32)
    vp[:, nz // 2:] = 3200.0
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    dvp = (0.1 * vp).astype(np.float32)
    dvs = (0.1 * vs).astype(np.float32)
    drho = (rho * rng.uniform(0.01, 0.05, (nx, nz))).astype(np.float32)
    P = pml.params(10.0, 0.05, fp=40.0)
    kw = dict(dx=10.0, dt=P["dt"], nt=P["nt"], xsource=nx // 2, zsource=70, nsource=P["nsource"], fp=40.0,
              nsnap=2, nseis=P["nseis"], abc=60, zrec=70)
    return [vp, vs, rho, dvp, dvs, drho], kw


def test_survey_grid_matches_oracle():
    """The whole grid of the survey at its full size, the first 70 levels
    (receiver lines from level 57 on), bit for bit against the oracle."""
    m, kw = survey_grid_case()
    gs, gc = pml.born(*m, **kw)
    os_, oc = O.pml_born(*m, **kw)
    for k in range(6):
        assert np.abs(gs[k]).max() > 0
        assert same_bits(gs[k], os_[k]) and same_bits(gc[k], oc[k]), O.PML_SEIS[k]


def test_scattered_field_is_linear_on_survey_grid():
    """Doubling the density perturbation (every Born coefficient scales with
    it exactly; magnitudes far from the set-up's 1e-2 cut-off) leaves the
    background bit-identical and doubles the scattered lines and snapshots
    (to 1e-6 relative: only subnormal values at the numerical wave front
    can round differently)."""
    m, kw = survey_grid_case()
    s1, c1 = pml.born(*m, **kw)
    m2 = list(m[:5]) + [(2 * m[5]).astype(np.float32)]
    s2, c2 = pml.born(*m2, **kw)
    for k in range(3):
        assert same_bits(s1[k], s2[k]) and same_bits(c1[k], c2[k]), O.PML_SEIS[k]
    for k in range(3, 6):
        for a, b in ((s1[k], s2[k]), (c1[k], c2[k])):
            a64 = 2 * a.astype(np.float64)
            err = np.linalg.norm(b - a64) / np.linalg.norm(a64)
            print(O.PML_SEIS[k], "relative deviation from 2x:", err)
            assert err <= 1e-6
