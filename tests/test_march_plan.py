"""CPU tests of the marching kernels' host logic (csrc/batch.cu march_plan,
csrc/march2d.cuh): the work plan covers every (shot, strip, chunk) unit once
in equal pieces with vertically adjacent strips aligned, and the kernels'
staging schedules -- modelled here step for step -- never overwrite a ring
column, slot or landing buffer that a chunk still reads, under any
interleaving of the warps."""
import os
import random

import numpy as np
import pytest

from elastic_gb300 import _lib
from elastic_gb300 import build as B

MC, MRING, TZ = 8, 32, 128  # chunk columns, ring columns, strip rows (march2d.cuh)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        B.build()
    return _lib.load()


def plan(lib, nxs, nz, ctas):
    nxs = np.asarray(nxs, np.int32)
    cap = 4 * int(sum((w + MC - 1) // MC for w in nxs)) * ((nz + TZ - 1) // TZ) + 16
    runs = np.zeros(4 * cap, np.int32)
    lo = np.zeros(ctas + 1, np.int32)
    n = lib.rtm_debug_march_plan(len(nxs), _lib.ptr(nxs), nz, ctas, _lib.ptr(runs), cap, _lib.ptr(lo))
    assert n >= 0
    return [tuple(int(v) for v in runs[4 * i:4 * i + 4]) for i in range(n)], [int(v) for v in lo]


GEOMS = [([1773, 966, 753, 1018], 800, 152), ([64, 70, 90], 48, 152), ([300, 250, 410], 700, 152),
         ([2000], 2000, 152), ([11], 11, 3), ([500, 37, 1200, 64], 300, 7), ([96] * 6, 129, 1)]


@pytest.mark.parametrize("nxs,nz,ctas", GEOMS)
def test_plan_covers_every_unit_once_in_equal_pieces(lib, nxs, nz, ctas):
    runs, lo = plan(lib, nxs, nz, ctas)
    assert lo[0] == 0 and lo[-1] == len(runs) and all(lo[b] <= lo[b + 1] for b in range(ctas))
    seen = set()
    per_cta = []
    for b in range(ctas):
        count = 0
        for s, y, k0, k1 in runs[lo[b]:lo[b + 1]]:
            assert 0 <= s < len(nxs) and y % TZ == 0 and 0 <= y < nz and 0 <= k0 < k1 <= (nxs[s] + MC - 1) // MC
            for k in range(k0, k1):
                assert (s, y, k) not in seen
                seen.add((s, y, k))
            count += k1 - k0
        per_cta.append(count)
    total = sum(((w + MC - 1) // MC) * ((nz + TZ - 1) // TZ) for w in nxs)
    assert len(seen) == total
    busy = [c for c in per_cta if c]
    assert max(busy) - min(busy) <= 1 or total < ctas


def test_plan_aligns_vertically_adjacent_strips(lib):
    """For the configuration-2 group most chunks have the chunk below them in
    the strip underneath handled by the next CTA within two chunks of the same
    time (both walk their runs left to right from the same column)."""
    nxs, nz, ctas = [1773, 966, 753, 1018], 800, 152
    runs, lo = plan(lib, nxs, nz, ctas)
    when = {}  # (shot, strip row, chunk) -> (cta, position in the CTA's walk)
    for b in range(ctas):
        pos = 0
        for s, y, k0, k1 in runs[lo[b]:lo[b + 1]]:
            for k in range(k0, k1):
                when[(s, y, k)] = (b, pos)
                pos += 1
    near = tot = 0
    for (s, y, k), (b, pos) in when.items():
        below = when.get((s, y + TZ, k))
        if below is None:
            continue
        tot += 1
        near += abs(below[1] - pos) <= 2
    assert near / tot > 0.8, near / tot


def forward_schedule_ok(runs, r0, r1):
    """k_fwd_march: group n (what chunk n of the walk reads first: ring chunk
    k+1, or k-1..k+1 for a run's first chunk, and own/coefficient slot n & 1)
    is issued once chunk n-2 is done (n-1 for a run's first group); chunk n
    reads ring columns 8k-5 .. 8k+12 and slot n & 1."""
    walk = [(r, k) for r in range(r0, r1) for k in range(runs[r][2], runs[r][3])]
    ring, slot = {}, {}

    def issue(n):
        r, k = walk[n]
        first = k == runs[r][2]
        for j in (range(k - 1, k + 2) if first else [k + 1]):
            for c in range(j * MC, j * MC + MC):
                ring[c & (MRING - 1)] = (r, c)
        slot[n & 1] = (r, k)

    nis = 0

    def issue_upto(i):
        nonlocal nis
        while nis < len(walk) and nis <= i + 2:
            r, k = walk[nis]
            if k == runs[r][2] and nis > i + 1:
                break
            issue(nis)
            nis += 1

    issue_upto(-1)
    for i, (r, k) in enumerate(walk):
        assert i < nis
        for c in range(k * MC - 5, k * MC + MC + 5):
            assert ring.get(c & (MRING - 1)) == (r, c)
        assert slot.get(i & 1) == (r, k)
        issue_upto(i)
    return True


@pytest.mark.parametrize("nxs,nz,ctas", GEOMS)
def test_forward_staging_schedule_never_overwrites_live_data(lib, nxs, nz, ctas):
    runs, lo = plan(lib, nxs, nz, ctas)
    for b in range(ctas):
        if lo[b] < lo[b + 1]:
            assert forward_schedule_ok(runs, lo[b], lo[b + 1])


class Bar:
    """An mbarrier phase counter (arrivals per phase, try_wait.parity)."""

    def __init__(self, count):
        self.count, self.pending, self.phase = count, count, 0

    def arrive(self):
        self.pending -= 1
        last = self.pending == 0
        if last:
            self.phase += 1
            self.pending = self.count
        return last

    def done(self, parity):
        return (self.phase & 1) != parity


def adjoint_protocol(runs, r0, r1, seed, warps=16):
    """k_adj_march with its warps interleaved at random: product pass P
    (chunk j) waits landing slot P & 1, writes ring columns of chunk j,
    arrives on pd[P & 1]; the last warp out loads pass P + 2 into the slot;
    chunk k waits for the pass of chunk k+1 and reads ring columns 8k-5 ..
    8k+12; the pass of chunk k+2 waits until chunk k-1 is computed by every
    warp (cd).  Landing loads land at random later times."""
    rnd = random.Random(seed)
    # thread t < 8 * 36 of the pass handles column t // 36 (36 row groups)
    cover = [sorted({t // 36 for t in range(32 * w, 32 * w + 32) if t < MC * 36}) for w in range(warps)]
    writers = [[w for w in range(warps) if col in cover[w]] for col in range(MC)]
    pd, cd = [Bar(warps), Bar(warps)], [Bar(warps), Bar(warps)]
    passes = [(r, runs[r][2] - 1 + pl) for r in range(r0, r1) for pl in range(runs[r][3] - runs[r][2] + 2)]
    landing, ring = {}, {}
    issued, landed = [0], [0]
    pending = []
    named = {"n": 0, "gen": 0}

    def issue():
        if issued[0] < len(passes):
            pending.append(issued[0])
            issued[0] += 1

    issue()
    issue()

    def warp(w):
        P = C = 0
        for r in range(r0, r1):
            k0, n = runs[r][2], runs[r][3] - runs[r][2]
            if r > r0:
                g = named["gen"]
                named["n"] += 1
                if named["n"] == warps:
                    named["n"], named["gen"] = 0, named["gen"] + 1
                while named["gen"] == g:
                    yield
            P0, C0 = P, C

            def products(j):
                nonlocal P
                while landed[0] <= P:
                    yield
                assert landing.get(P & 1) == P
                for col in cover[w]:
                    c = j * MC + col
                    ring[(c & (MRING - 1), w)] = (r, c)
                yield
                assert landing.get(P & 1) == P, "landing slot overwritten while read"
                if pd[P & 1].arrive():
                    issue()
                P += 1

            for pl in range(3):
                yield from products(k0 - 1 + pl)
            for c in range(n):
                Q = P0 + c + 2
                while not pd[Q & 1].done((Q >> 1) & 1):
                    yield
                k = k0 + c
                for _ in range(2):
                    for col in range(k * MC - 5, k * MC + MC + 5):
                        for ww in writers[col % MC]:
                            assert ring.get((col & (MRING - 1), ww)) == (r, col)
                    yield
                cd[C & 1].arrive()
                C += 1
                if c + 3 <= n + 1:
                    if c >= 1:
                        D = C0 + c - 1
                        while not cd[D & 1].done((D >> 1) & 1):
                            yield
                    yield from products(k0 + c + 2)

    gens = [warp(w) for w in range(warps)]
    alive = list(range(warps))
    steps = 0
    while alive:
        steps += 1
        assert steps < 2_000_000, "deadlock"
        if pending and rnd.random() < 0.3:
            p = pending.pop(0)
            landing[p & 1] = p
            landed[0] += 1
        i = rnd.choice(alive)
        try:
            next(gens[i])
        except StopIteration:
            alive.remove(i)
    assert not pending and issued[0] == len(passes)
    return True


@pytest.mark.parametrize("nxs,nz,ctas", GEOMS[1:])
def test_adjoint_protocol_has_no_deadlock_and_no_stale_read(lib, nxs, nz, ctas):
    runs, lo = plan(lib, nxs, nz, ctas)
    tried = 0
    for b in range(ctas):
        if lo[b] < lo[b + 1] and tried < 4:
            assert adjoint_protocol(runs, lo[b], lo[b + 1], seed=b)
            tried += 1


def test_plan_rejects_bad_arguments(lib):
    nxs = np.array([100, 200], np.int32)
    runs = np.zeros(4 * 64, np.int32)
    lo = np.zeros(5, np.int32)
    assert lib.rtm_debug_march_plan(0, _lib.ptr(nxs), 100, 4, _lib.ptr(runs), 64, _lib.ptr(lo)) == -1
    assert lib.rtm_debug_march_plan(2, _lib.ptr(nxs), 100, 0, _lib.ptr(runs), 64, _lib.ptr(lo)) == -1
    # more runs than the output holds
    assert lib.rtm_debug_march_plan(2, _lib.ptr(nxs), 1000, 4, _lib.ptr(runs), 1, _lib.ptr(lo)) == -1
