"""Multi-GPU replicas on the CPU: two gloo ranks shard a survey's shot
groups, each "migrates" its groups (a CPU stand-in whose image depends on
the group), and the whole-job aggregation and the image stack equal the
single-process results (elastic_gb300/shard.py, as bench.py uses it)."""
import os
import socket

import numpy as np
import pytest

from elastic_gb300.shard import aggregate, shard_groups, stack_images

GROUPS = [(0, 4), (4, 4), (8, 3), (11, 4), (15, 2)]


def fake_migrate(group, nz=6, nx=5):
    s0, n = group
    rng = np.random.default_rng(s0 * 31 + n)
    return rng.standard_normal((3, nx, nz))


def test_shards_cover_every_group_once():
    for world in (1, 2, 3, 8):
        got = sorted(g for r in range(world) for g in shard_groups(GROUPS, r, world))
        assert got == sorted(GROUPS)
    with pytest.raises(ValueError):
        shard_groups(GROUPS, 2, 2)


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_groups(GROUPS, rank, world)
        img = torch.zeros(3, 5, 6, dtype=torch.float64)
        for g in mine:
            img += torch.from_numpy(fake_migrate(g))
        cells = sum(n for _, n in mine) * 1000.0
        times, counts = aggregate([0.5 + rank, 2.0 * rank], [cells, len(mine)])
        stack_images(img)
        out.put((rank, times, counts, img.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_and_stack():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want_img = sum(fake_migrate(g) for g in GROUPS)
    for rank, times, counts, img in res:
        assert times == [1.5, 2.0]                             # maximum over ranks
        assert counts == [sum(n for _, n in GROUPS) * 1000.0, len(GROUPS)]  # sums
        np.testing.assert_allclose(img, want_img, rtol=0, atol=1e-12)


def test_single_process_is_identity():
    import torch
    times, counts = aggregate([1.0, 2.0], [3.0])
    assert times == [1.0, 2.0] and counts == [3.0]
    img = torch.ones(2)
    assert stack_images(img) is img
