"""Shot-group sharding over the ranks of one node (one process per GPU).

The shots of a survey are independent (each migrates against its own
traces on its own subgrid), so a multi-GPU run is replicas: rank r migrates
groups r, r + world, r + 2 world, ... into its own image, with no collective
on the data path.  Two collectives exist, both outside the per-level work:
the whole-job timing (maximum of the ranks' times, sum of their
cell-updates) and, once at the end of a migration, the stack of the ranks'
images (a sum).
"""


def shard_groups(groups, rank, world):
    """The groups rank `rank` of `world` migrates (every world-th)."""
    if not 0 <= rank < world:
        raise ValueError("rank %d outside 0..%d" % (rank, world - 1))
    return list(groups)[rank::world]


def aggregate(times, counts, device="cpu"):
    """Whole-job figures over the initialised process group (or this process
    alone): maximum of each entry of `times`, sum of each entry of
    `counts`.  Returns two lists of floats."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(times), dtype=torch.float64, device=device)
    c = torch.tensor(list(counts), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()


def stack_images(image):
    """Sum of the ranks' images, in place (a torch tensor on the process
    group's device); the image of a single process is returned as is."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(image, op=dist.ReduceOp.SUM)
    return image
