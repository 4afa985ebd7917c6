"""SEP history-file I/O: headers in the reference's layout (program line,
tab-indented key=value pairs, `sets next: in=...`, xdr_float data), round
trips, axis order and the override rule."""
import os

import numpy as np
import pytest

from elastic_gb300 import sep

HEADER = """

Bin/rtm.x:   someone@somehost   Fri Aug 14 13:19:41 2015
\t\tn1=3
\t\to1=0
\t\td1=4
\t\tn2=2
\t\to2=10
\t\td2=5
\t\tsets next: in="{binp}"
\t\tdata_format="xdr_float"
"""


def test_read_reference_style_header(tmp_path):
    binp = tmp_path / "m.H@"
    vals = np.arange(6, dtype=np.float32) * 1.5
    vals.astype(">f4").tofile(binp)  # big-endian, axis 1 (n1=3) fastest
    hp = tmp_path / "m.H"
    hp.write_text(HEADER.format(binp=binp))
    a, h = sep.read(str(hp))
    assert a.shape == (2, 3)
    np.testing.assert_array_equal(a, vals.reshape(2, 3))
    assert sep.axes(h) == [(3, 0.0, 4.0), (2, 10.0, 5.0)]


def test_later_entries_override_and_relative_binary(tmp_path):
    vals = np.array([1, 2, 3, 4], np.float32)
    vals.astype("=f4").tofile(tmp_path / "x.bin")
    (tmp_path / "x.H").write_text('prog: a\n\t\tn1=2 n2=2 in=old.bin\n\t\tn1=4 n2=1\n\t\tin="x.bin" '
                                  'data_format="native_float"\n')
    a, h = sep.read(str(tmp_path / "x.H"))
    assert a.shape == (4,)
    np.testing.assert_array_equal(a, vals)


def test_round_trip_gathers_and_images(tmp_path):
    rng = np.random.default_rng(0)
    g = [rng.standard_normal((7, 11)).astype(np.float32) for _ in range(5)]  # (nx, nt)
    paths = sep.write_gathers(str(tmp_path / "shot1-"), g, dt=1e-3, dx=10.0)
    for p, x in zip(paths, g):
        y, h = sep.read(p)
        np.testing.assert_array_equal(y, x)
        assert h["n1"] == "11" and h["n2"] == "7" and float(h["d1"]) == 1e-3 and h["data_format"] == "xdr_float"
        assert os.path.getsize(p + "@") == x.size * 4
        # the binary is big-endian
        np.testing.assert_array_equal(np.fromfile(p + "@", ">f4").reshape(x.shape), x)
    im = [rng.standard_normal((7, 5)).astype(np.float32) for _ in range(3)]
    for p, x, name in zip(sep.write_images(str(tmp_path / "img-"), im, dz=10.0, dx=10.0), im, ("drho", "dlambda", "dmu")):
        assert p.endswith(name + ".H")
        np.testing.assert_array_equal(sep.read(p)[0], x)


def test_bad_headers(tmp_path):
    (tmp_path / "a.H").write_text("\t\tn1=4\n")
    with pytest.raises(ValueError):
        sep.read(str(tmp_path / "a.H"))
    np.zeros(2, ">f4").tofile(tmp_path / "b.bin")
    (tmp_path / "b.H").write_text('\t\tn1=4 in="b.bin"\n')
    with pytest.raises(ValueError):
        sep.read(str(tmp_path / "b.H"))
    (tmp_path / "c.H").write_text('\t\tn1=2 in="b.bin" data_format="xdr_int"\n')
    with pytest.raises(ValueError):
        sep.read(str(tmp_path / "c.H"))


GOLD_SEP = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sep")


@pytest.mark.parametrize("name,axes", [
    ("lambda-layer.H", [(300, 0.0, 4.0), (300, 0.0, 4.0)]),
    ("dlambda-layer.H", [(300, 0.0, 4.0), (300, 0.0, 4.0)]),
    ("seis-Vx-layer.H", [(3535, 0.0, 0.000565685), (300, 0.0, 4.0)]),
    ("filter.H", [(45, 0.0, 1.0)]),
])
def test_reference_headers_parse(name, axes):
    """The reference's own history headers (2d_rtm_restart/Dat, copied by
    tests/golden/sep/copy_headers.py): axes, binary name and format."""
    h = sep.read_header(os.path.join(GOLD_SEP, name))
    assert sep.axes(h) == axes
    assert h["data_format"] == "xdr_float"
    assert h["in"].startswith("/data/") and h["in"].endswith(("@", "@ewzD0r"))


def test_reference_headers_agree_with_the_reference_code():
    """filter.H has abc+5 = 45 samples for abc = 40 (W/abc-mod.f90:42-56) and
    the gathers' time step is rtm.f90's dt = 0.4*dx/(sqrt(2)*2000) for the
    model's dx = 4 m, in single precision (W/rtm.f90:60)."""
    f = sep.axes(sep.read_header(os.path.join(GOLD_SEP, "filter.H")))[0][0]
    assert f == 40 + 5
    ax = sep.axes(sep.read_header(os.path.join(GOLD_SEP, "seis-Vx-layer.H")))
    dt = np.float32(0.4) * np.float32(4.0) / (np.sqrt(np.float32(2.0)) * np.float32(2000.0))
    assert abs(ax[0][2] - float(dt)) < 5e-10
    assert ax[1][2] == sep.axes(sep.read_header(os.path.join(GOLD_SEP, "lambda-layer.H")))[1][2]


def test_reference_header_reads_a_local_binary(tmp_path):
    """A reference header whose binary is re-pointed by an appended in= (the
    later entry wins, as SEPlib reads it) reads xdr_float data in Fortran
    axis order."""
    text = open(os.path.join(GOLD_SEP, "filter.H")).read()
    vals = (np.arange(45, dtype=np.float32) / 45).astype(">f4")
    vals.tofile(tmp_path / "filter.H@")
    (tmp_path / "filter.H").write_text(text + '\n\t\tin="filter.H@"\n')
    a, _ = sep.read(str(tmp_path / "filter.H"))
    np.testing.assert_array_equal(a, vals.astype(np.float32))
