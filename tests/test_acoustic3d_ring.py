"""CPU model of the 3D slice-ring kernel's copy schedule (k_acoustic3d_t in
elastic_gb300/csrc/acoustic3d.cu), checked before it runs on a GPU.

A CTA marches y over [ya, yb) and reads slices y-5 .. y+5 of p1 from a
13-slot shared-memory ring.  One thread issues slices ya-5 .. ya+6 before the
march and slice y+7 at the top of iteration y (after the CTA barrier), each
into slot (s - (ya-5)) mod 13; every thread waits for slices ya-5 .. ya+4
once and for slice y+5 in iteration y.  The model checks that every slice is
issued before it is waited on, waited on before it is read, never
overwritten while it may still be read, and that every issued slice is
waited on (no copy in flight when the CTA exits)."""
import pytest

NR = 13


def schedule(ya, yb):
    last = yb - 1 + 5
    slot_of = {}
    resident = {}  # slot -> slice
    waited = set()
    log = []

    def issue(s, y):
        k = (s - (ya - 5)) % NR
        if k in resident:
            # the previous occupant must be older than every slice read from
            # now on (iteration y reads y-5 .. y+5)
            assert resident[k] < y - 5, (s, k, resident[k], y)
        resident[k] = s
        slot_of[s] = k
        log.append(("issue", s))

    for s in range(ya - 5, min(ya + 6, last) + 1):
        issue(s, ya)
    for y in range(ya, yb):
        for s in range(ya - 5 if y == ya else y + 5, y + 6):
            assert s in slot_of, ("waited before issue", y, s)
            waited.add(s)
        if y + 7 <= last:
            issue(y + 7, y)
        for s in range(y - 5, y + 6):
            assert s in waited, ("read before wait", y, s)
            assert resident[slot_of[s]] == s, ("overwritten while read", y, s)
    assert set(slot_of) == waited, "a copy would be in flight at exit"
    return log


@pytest.mark.parametrize("ya", [5, 131])
@pytest.mark.parametrize("n", [1, 2, 3, 6, 7, 8, 12, 13, 14, 64, 126, 502])
def test_ring_schedule(ya, n):
    log = schedule(ya, ya + n)
    # exactly the slices ya-5 .. yb+4 are loaded, once each
    assert sorted(s for _, s in log) == list(range(ya - 5, ya + n + 5))
