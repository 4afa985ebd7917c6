"""The oracle's split-field PML Born modelling (oracle/pml2d.c) against the
reference's own program, 2d_rtm_restart/working_Src/born.f90, executed here
through its Fortran modules translated to C (oracle/f90c.py --set pml):
bit-exact on every receiver line and snapshot, through the committed
fixtures (tests/golden/refpml_small.npz) and, where the reference tree is
present, on further cases run directly."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
import sys
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from elastic_gb300 import pml

GOLD = os.path.join(os.path.dirname(__file__), "golden", "refpml_small.npz")
CASES = ("odd", "surface", "lame", "noabc", "blocks")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def case_args(g, name):
    nz, nx, nt, xs, zs, nsource, nsnap, nseis, abc, zrec, fs, lame = (int(v) for v in g[name + "/geom"])
    dx, dt, fp = (float(v) for v in g[name + "/phys"])
    return list(g[name + "/model"]), dict(dx=dx, dt=dt, nt=nt, xsource=xs, zsource=zs, nsource=nsource, fp=fp,
                                          nsnap=nsnap, nseis=nseis, abc=abc, zrec=zrec, free_surface=bool(fs),
                                          lame=bool(lame))


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def check_against_fixture(g, name, seis, snap):
    assert [digest(a) for a in seis] == list(g[name + "/seis_sha256"])
    assert [digest(a) for a in snap] == list(g[name + "/snap_sha256"])
    if name + "/seis" in g:
        for k in range(6):
            assert same_bits(seis[k], g[name + "/seis"][k]), (name, O.PML_SEIS[k])
            assert same_bits(snap[k], g[name + "/snap"][k]), (name, O.PML_SEIS[k])


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixtures(gold, name):
    m, kw = case_args(gold, name)
    seis, snap = O.pml_born(*m, **kw)
    check_against_fixture(gold, name, seis, snap)
    # the case records something in every line
    assert all(np.abs(s).max() > 0 for s in seis)


def test_planted_ulp_is_seen(gold, monkeypatch):
    m, kw = case_args(gold, "odd")
    monkeypatch.setenv("ORA_PML_PLANT", "1")
    seis, snap = O.pml_born(*m, **kw)
    assert [digest(a) for a in seis[:3] + snap[:3]] == list(gold["odd/seis_sha256"][:3]) + list(
        gold["odd/snap_sha256"][:3]), "the background does not see the scattered field"
    assert any(not same_bits(seis[k], gold["odd/seis"][k]) or not same_bits(snap[k], gold["odd/snap"][k])
               for k in range(3, 6))


def test_main_program_parameters():
    """pml.params (the product's helper) and the oracle's restatement of the
    main program's derived sizes agree."""
    for dx, Tt, fp in ((10.0, 0.1, 60.0), (10.0, 1.0, 25.0), (5.0, 0.5, 15.0), (12.5, 2.0, 20.0)):
        assert pml.params(dx, Tt, fp=fp) == O.pml_params(0, 0, dx, Tt, fp=fp)


needs_ref = pytest.mark.skipif(not O.refpml_available(), reason="reference tree not present")


# (nz, nx, abc, free surface, lame, seed, source (z, x) or None, zrec)
EDGE_CASES = [
    (29, 30, 12, False, False, 1, None, 8),   # left and right PML columns overlap (14..17)
    (26, 52, 11, True, False, 2, None, 8),    # top and bottom PML rows overlap
    (41, 39, 1, False, True, 3, None, 8),
    (64, 33, 5, True, True, 4, None, 8),
    (30, 30, 14, False, False, 5, None, 8),   # widest PML: both axes overlap, nx - 2 abc = 2
    (36, 40, 8, False, False, 6, (3, 3), 2),  # source outside every operator's range, receivers at row 2
    (36, 40, 8, True, False, 7, (9, 8), 36),  # source inside the top-left PML, receivers at the last row
]


def edge_case_args(nz, nx, abc, fs, lame, seed, src, zrec):
    import make_golden_pml as G
    m = G.model(nz, nx, seed, lame)
    P = O.pml_params(nz, nx, 10.0, 0.08, fp=60.0)
    zs, xs = src if src else (min(12, nz - 6), nx // 2)
    kw = dict(dx=10.0, dt=P["dt"], nt=P["nt"], xsource=xs, zsource=zs, nsource=P["nsource"], fp=60.0, nsnap=3,
              nseis=P["nseis"], abc=abc, zrec=zrec, free_surface=fs, lame=lame)
    return m, kw


@needs_ref
@pytest.mark.parametrize("case", EDGE_CASES, ids=lambda c: "%dx%d_abc%d" % c[:3] + ("_fs" if c[3] else "") +
                         ("_lame" if c[4] else "") + ("_src%d,%d" % c[6] if c[6] else "") + "_zrec%d" % c[7])
def test_oracle_matches_translated_reference(case):
    m, kw = edge_case_args(*case)
    rs, rc = O.refpml_born(*m, **kw)
    os_, oc = O.pml_born(*m, **kw)
    for k in range(6):
        assert same_bits(rs[k], os_[k]) and same_bits(rc[k], oc[k]), O.PML_SEIS[k]


@needs_ref
@pytest.mark.parametrize("fs", [False, True])
def test_pml_tables_match_reference_module_state(fs):
    """The oracle's PML tables equal pml_mod's pml0_xl .. pml1_zb as the
    reference leaves them after a run."""
    import make_golden_pml as G
    m = G.model(30, 34, 9, False)
    P = O.pml_params(30, 34, 10.0, 0.01, fp=60.0)
    abc = 7
    O.refpml_born(*m, 10.0, P["dt"], P["nt"], 17, 12, P["nsource"], 60.0, 1, P["nseis"], abc, 8, free_surface=fs)
    mine = O.pml_tables(m[0], 10.0, P["dt"], abc, free_surface=fs)
    for name, t in zip(O.PML_TABLES, mine):
        assert same_bits(O.refpml_get("pml_mod." + name, t.shape), t), name
