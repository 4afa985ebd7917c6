"""SEP history files (.H header + binary) for the reference's models,
gathers and images.

The reference reads its models and writes its gathers and images through
SEPlib (v7, not vendored; `W/seis-mod-rtm.f90:21-142` for the outputs).
A history file is text: a program/user/date line per program that touched
the data, then `key=value` pairs (several per line allowed); a later value
overrides an earlier one.  `in="path"` names the binary, `data_format`
selects its encoding ("xdr_float" = big-endian IEEE float32, "native_float"
= host order), and n1..nN / o1..oN / d1..dN give the axes, axis 1 fastest
(Fortran order).  Arrays here are C-ordered with axis 1 last, as the rest of
the package uses them: a (nz, nx) Fortran model is a (nx, nz) array.
"""
import datetime
import getpass
import os
import re
import socket

import numpy as np

_PAIR = re.compile(r'([A-Za-z_][\w.]*)=("[^"]*"|\'[^\']*\'|\S+)')


def read_header(path):
    """All key=value pairs of a history file (the last occurrence wins),
    values unquoted strings."""
    with open(path, "r", errors="replace") as f:
        text = f.read()
    out = {}
    for k, v in _PAIR.findall(text):
        if len(v) >= 2 and v[0] == v[-1] and v[0] in "\"'":
            v = v[1:-1]
        out[k] = v
    return out


def axes(header):
    """[(n, o, d), ...] for axes 1..N (trailing axes of length 1 dropped,
    at least one axis kept)."""
    ax = []
    i = 1
    while f"n{i}" in header:
        ax.append((int(header[f"n{i}"]), float(header.get(f"o{i}", 0.0)), float(header.get(f"d{i}", 1.0))))
        i += 1
    while len(ax) > 1 and ax[-1][0] == 1:
        ax.pop()
    if not ax:
        raise ValueError("history file has no n1")
    return ax


def _dtype(header):
    fmt = header.get("data_format", "xdr_float")
    esize = int(header.get("esize", 4))
    if esize != 4:
        raise ValueError(f"esize={esize} is not supported (float32 data only)")
    if fmt == "xdr_float":
        return np.dtype(">f4")
    if fmt == "native_float":
        return np.dtype("=f4")
    raise ValueError(f"data_format={fmt!r} is not supported")


def read(path):
    """(array float32, header): the binary named by `in=` (relative paths
    taken from the header's directory), shaped (nN, ..., n1)."""
    h = read_header(path)
    if "in" not in h:
        raise ValueError(f"{path}: no in= entry")
    binp = h["in"]
    if not os.path.isabs(binp):
        binp = os.path.join(os.path.dirname(os.path.abspath(path)), binp)
    ax = axes(h)
    count = int(np.prod([n for n, _, _ in ax]))
    data = np.fromfile(binp, dtype=_dtype(h), count=count)
    if data.size != count:
        raise ValueError(f"{binp}: {data.size} values, header asks for {count}")
    return data.astype(np.float32).reshape([n for n, _, _ in reversed(ax)]), h


def write(path, array, o=None, d=None, labels=None, data_format="xdr_float", program="elastic_gb300", extra=None):
    """Write array (C order, axis 1 last) as path (header) + path + "@"
    (binary).  o, d: per-axis origins and samplings in axis-1-first order."""
    a = np.asarray(array, np.float32)
    shape = list(reversed(a.shape)) or [1]
    o = list(o) if o is not None else [0.0] * len(shape)
    d = list(d) if d is not None else [1.0] * len(shape)
    binp = os.path.abspath(path) + "@"
    dt = np.dtype(">f4") if data_format == "xdr_float" else np.dtype("=f4")
    a.astype(dt).tofile(binp)
    try:
        user = getpass.getuser()
    except Exception:
        user = "unknown"
    lines = ["", "", f"{program}:   {user}@{socket.gethostname()}   {datetime.datetime.now().ctime()}"]
    for i, n in enumerate(shape, start=1):
        lines.append(f"\t\tn{i}={n}")
        lines.append(f"\t\to{i}={o[i - 1]:g}")
        lines.append(f"\t\td{i}={d[i - 1]:g}")
        if labels and i <= len(labels) and labels[i - 1]:
            lines.append(f'\t\tlabel{i}="{labels[i - 1]}"')
    for k, v in (extra or {}).items():
        lines.append(f"\t\t{k}={v}")
    lines.append(f'\t\tsets next: in="{binp}"')
    lines.append(f'\t\tesize=4')
    lines.append(f'\t\tdata_format="{data_format}"')
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def write_gathers(prefix, gathers, dt, dx, names=("Vx_rec", "Vz_rec", "sigmaxx_rec", "sigmazz_rec", "sigmaxz_rec")):
    """The five receiver gathers, each (nx, nt), as the reference's seismo
    writes them (n1=nt, d1=dt, n2=nx, d2=dx, origins 0)."""
    out = []
    for g, name in zip(gathers, names):
        out.append(write(f"{prefix}{name}.H", g, d=(dt, dx)))
    return out


def write_images(prefix, images, dz, dx, lame=True):
    """Images (drho, dlambda, dmu) or (drho, dvp, dvs), each (nx, nz), as the
    reference's img writes them (n1=nz, d1=dz, n2=nx, d2=dx)."""
    names = ("drho", "dlambda", "dmu") if lame else ("drho", "dvp", "dvs")
    return [write(f"{prefix}{n}.H", im, d=(dz, dx)) for im, n in zip(images, names)]
