"""Query sharding across ranks (one process per GPU).

Every query is independent (the reference evaluates them in one
igl::parallel_for), so N ranks each evaluate a contiguous slice of Q against
their own replica of the tree / expansion and the results are gathered once.
There is no collective on the data path; the only exchange is the final
all-gather of W (a host-side concatenation in rank order).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's contiguous slice of n items (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def evaluate_sharded(evaluate, Q, group=None):
    """Evaluate `evaluate(Q_slice) -> W_slice` on this rank's slice of Q and
    all-gather the slices (torch.distributed, any backend) into the full W,
    identical on every rank.  Without an initialised process group this is a
    plain call."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return np.asarray(evaluate(Q))
    import torch
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    n = Q.shape[0]
    b, e = shard_bounds(n, rank, world)
    local = np.ascontiguousarray(np.asarray(evaluate(Q[b:e])), dtype=np.float64)
    sizes = [shard_bounds(n, r, world)[1] - shard_bounds(n, r, world)[0] for r in range(world)]
    mx = max(sizes)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    buf = torch.zeros(mx, dtype=torch.float64, device=dev)
    buf[: local.shape[0]] = torch.from_numpy(local).to(dev)
    out = [torch.empty(mx, dtype=torch.float64, device=dev) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    return np.concatenate([o[:s].cpu().numpy() for o, s in zip(out, sizes)])
