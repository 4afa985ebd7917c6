"""Deterministic test inputs that every platform reproduces bit for bit.

Values come from the SplitMix64 mixing function of the element index and a
salt, in unsigned 64-bit integer arithmetic, mapped to float32 in [-1, 1)
with a 24-bit mantissa.  Unlike a pseudo-random generator's stream, this
depends on nothing but integer arithmetic, so large golden inputs need not
be stored: a fixture keeps the salt and the digest of the output.
"""
import hashlib

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & M64
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M64
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M64
    return x ^ (x >> np.uint64(31))


def field(shape, salt, scale=1.0, offset=0.0):
    """float32 array of `shape` with values offset + scale * u, u in [-1, 1)."""
    n = int(np.prod(shape))
    with np.errstate(over="ignore"):
        idx = np.arange(n, dtype=np.uint64) + (np.uint64(salt) << np.uint64(40))
        h = splitmix64(idx) >> np.uint64(40)  # 24 bits
    u = h.astype(np.float64) / float(1 << 23) - 1.0
    return (offset + scale * u).astype(np.float32).reshape(shape)


def digest(arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()
