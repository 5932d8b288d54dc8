"""Scene sharding for batched solves on several GPUs (one process per GPU).

Independent scenes are the unit of work: a rank solves its own scenes and no
data crosses ranks during the solve; only the timing and the per-scene
results are combined at the end.  Scenes go to ranks by longest-processing-
time first on their contact counts (largest scene first, to the least-loaded
rank, ties to the lower rank), which is deterministic on every rank.
"""
from __future__ import annotations

import numpy as np


def shard_scenes(sizes, rank: int, world: int) -> list[int]:
    """Indices of the scenes rank `rank` of `world` solves, in input order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    sizes = np.asarray(sizes, dtype=np.int64)
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load = [0] * world
    owner = np.empty(len(sizes), dtype=np.int64)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += int(sizes[k])
    return [k for k in range(len(sizes)) if owner[k] == rank]


def combine(contact_sweeps: float, seconds: float, world: int):
    """Whole-job contact-sweeps and the slowest rank's time, over the
    default process group when world > 1."""
    if world <= 1:
        return contact_sweeps, seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([contact_sweeps, seconds], dtype=torch.float64)
    a = t[:1].clone()
    b = t[1:].clone()
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    dist.all_reduce(b, op=dist.ReduceOp.MAX)
    return float(a.item()), float(b.item())
