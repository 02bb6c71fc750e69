"""
Sharding observation points across GPUs (one process per GPU).

Every point's sum over prisms is independent, so N ranks split the points
into contiguous shards and compute them with no data-path collective; the
only communication is gathering the shards (or a scalar timing reduction in
the benchmark).  This is the multi-GPU form of harmonica's ``prange`` over
points (``src/harmonica/_forward/prisms/gravity.py:524``).
"""

import numpy as np


def shard_bounds(n, rank, world):
    """[lo, hi) of rank's contiguous shard of n points (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gather_shards(local, n, world, group=None):
    """All-gather variable-size 1-D float64 shards into the full array (torch.distributed)."""
    import torch
    import torch.distributed as dist

    sizes = [shard_bounds(n, r, world)[1] - shard_bounds(n, r, world)[0] for r in range(world)]
    width = max(sizes) if sizes else 0
    buf = torch.zeros(width, dtype=torch.float64, device=local.device)
    buf[: local.numel()] = local
    out = [torch.zeros(width, dtype=torch.float64, device=local.device) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    return torch.cat([o[:s] for o, s in zip(out, sizes)])


def forward_sharded(coordinates, compute, rank, world, group=None):
    """
    Run ``compute(shard_coordinates) -> np.ndarray`` on this rank's shard and
    return the gathered full result on every rank, with the broadcast shape
    of the coordinates.  The coordinates are broadcast against each other
    first (a scalar height with arrays of eastings and northings, as the
    forward models accept).  With an NCCL group the shards are gathered on
    this rank's current CUDA device.
    """
    import torch
    import torch.distributed as dist

    coords = np.broadcast_arrays(*(np.asarray(c, dtype=np.float64) for c in coordinates[:3]))
    shape = coords[0].shape
    n = coords[0].size
    lo, hi = shard_bounds(n, rank, world)
    part = compute(tuple(np.ascontiguousarray(c.ravel()[lo:hi]) for c in coords))
    local = torch.from_numpy(np.ascontiguousarray(np.ravel(part), dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        local = local.to(torch.device("cuda", torch.cuda.current_device()))
    return gather_shards(local, n, world, group).cpu().numpy().reshape(shape)
