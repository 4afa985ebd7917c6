"""CPU tests of the C-ABI library: it loads without a GPU, exports every
symbol that include/elastic_rtm.h declares, its host-side tables equal the
oracle's bit for bit, and argument checks fail before any device work."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
from elastic_gb300 import _lib
from elastic_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", txt)
    return sorted(set(n for n in names if n not in ("if", "for", "while", "return", "sizeof")))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        B.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    so = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing
    # and the Python binding covers all of them
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_host_tables_match_oracle(lib):
    from elastic_gb300 import rtm as R
    for abc in (0, 1, 12, 40):
        np.testing.assert_array_equal(R.abc_init(abc), O.abc_init(abc))
    for nt, dt, fp, ns in [(2000, 1e-3, 15.0, 250), (300, 5e-4, 25.0, 40), (10, 1e-3, 15.0, 5)]:
        np.testing.assert_array_equal(R.source_op2(nt, dt, fp, ns),
                                      O.source_op2(nt, np.float32(dt), np.float32(fp), ns))


def test_argument_checks_before_device_work(lib):
    z = np.zeros(16, np.float32)
    p = _lib.ptr(z)
    st = lib.rtm_op_c_(1, 5, 5, 10, 10.0, 1e-3, 1, 1, 1, 15.0, 250, 40, *[p] * 11, 0, 0)
    assert st == 1 and b"too small" in lib.rtm_last_error()
    assert lib.rtm_abc_c_(-1, p) == 1
    assert lib.rtm_source_c_(0, 1e-3, 15.0, 250, p) == 1
    # batch-engine switches reject bad handles and modes before any device use
    assert lib.rtm_batch_set_march(None, 1) == 1
    assert lib.rtm_batch_set_tma(None, 1) == 1
    assert lib.rtm_batch_set_stages(None, 1, 1, 256, 256) == 1
    assert lib.rtm_batch_set_checkpoint(None, 4) == 1
    # PML Born modelling: geometry checked before any device work
    P6 = (ctypes.c_void_p * 6)(*[p] * 6)
    for bad in [dict(nz=8), dict(nsnap=0), dict(abc=40), dict(zrec=1), dict(xsource=0)]:
        g = dict(nz=40, nx=40, nt=10, xsource=20, zsource=10, nsource=20, nsnap=2, nseis=5, abc=5, zrec=8)
        g.update(bad)
        st = lib.pml_born_c_(g["nz"], g["nx"], g["nt"], 10.0, 1e-3, g["xsource"], g["zsource"], g["nsource"], 25.0,
                             g["nsnap"], g["nseis"], g["abc"], g["zrec"], 0, 0, *[p] * 6, P6, P6)
        assert st == 1, bad
