"""Multi-GPU runs are replicas: the path shards by image, pass and request, with no
exchange on the data path (each render's film stays on its own device).  The only
cross-rank step is the benchmark's bookkeeping: a barrier around the timed region and
the whole-job figure (units of all ranks over the slowest rank's time)."""
from __future__ import annotations


def aggregate(local_ms: float, local_units: float):
    """(max time over ranks in ms, units summed over ranks); identity without a process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(local_ms), float(local_units)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
