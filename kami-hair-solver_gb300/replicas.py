"""Replica runs across ranks (one process per GPU).

Every rank solves the same workload independently: strands are independent
in assembly and in the block solve, but the line search couples every
strand of a scene through global scalars (energy, slope, CCD bound), so a
scene is not split across GPUs and the data path has no collective.  The
only exchange is this aggregation at the end of a timed region: the whole
job's throughput is the total substeps of all ranks divided by the slowest
rank's time, and the state checksums show that the replicas computed the
same trajectory.
"""
from __future__ import annotations

import numpy as np


def state_checksum(q: np.ndarray) -> float:
    """Order-sensitive checksum of a state array (sum of index-weighted
    entries), equal on two ranks only if their states are equal."""
    flat = np.ascontiguousarray(q, dtype=np.float64).ravel()
    return float(np.dot(flat, 1.0 + np.arange(flat.size, dtype=np.float64) * 1e-7))


def aggregate(substeps: int, seconds: float, checksum: float, dist=None, device: str = "cpu") -> dict:
    """Whole-job substeps/s over ranks: SUM of substeps / MAX of seconds;
    gathers every rank's checksum.  ``dist`` is torch.distributed (or None
    for one process); ``device`` is where the reduction tensors live ("cuda"
    for NCCL, "cpu" for gloo)."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return {"world": 1, "substeps": int(substeps), "max_seconds": float(seconds),
                "value": substeps / seconds if seconds > 0 else None, "checksums": [checksum]}
    import torch

    world = dist.get_world_size()
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    s = torch.tensor([float(substeps)], dtype=torch.float64, device=device)
    c = torch.tensor([float(checksum)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    gathered = [torch.zeros_like(c) for _ in range(world)]
    dist.all_gather(gathered, c)
    max_s, total = float(t.item()), int(round(s.item()))
    return {"world": world, "substeps": total, "max_seconds": max_s, "value": total / max_s if max_s > 0 else None,
            "checksums": [float(g.item()) for g in gathered]}
