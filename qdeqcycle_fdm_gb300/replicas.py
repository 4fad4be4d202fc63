"""Independent replicas on several GPUs of one node.

One earthquake-cycle instance does not shard without a halo exchange on
every smoothing sweep, so N GPUs run N independent replicas (one process per
GPU) and the data path has no collective.  The only communication is at the
end: the whole-job throughput is the work all ranks did divided by the
slowest rank's time (weak scaling), which needs one sum and one max.
"""
from __future__ import annotations

import os


def env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str, timeout_s: float | None = None):
    """Join the process group when launched with more than one rank.

    timeout_s bounds every collective: a rank that left or hangs makes the
    others' next collective raise after that long instead of waiting for the
    library's default (minutes)."""
    rank, world, local = env()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            kw = {}
            if timeout_s is not None:
                import datetime
                kw["timeout"] = datetime.timedelta(seconds=timeout_s)
            dist.init_process_group(backend, **kw)
    return rank, world, local


def aggregate(units: float, seconds: float, device=None):
    """(total units over all ranks, max seconds over ranks, throughput).

    With one rank this is (units, seconds, units / seconds)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units, seconds, units / seconds if seconds > 0 else 0.0
    u = torch.tensor([units], dtype=torch.float64, device=device)
    s = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    tu, ts = float(u.item()), float(s.item())
    return tu, ts, tu / ts if ts > 0 else 0.0


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
