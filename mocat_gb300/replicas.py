"""Several GPUs, one process each: the particle-system step does not shard in
this build, so every rank runs its own filters (its own key, or its own share
of a batch of series / posteriors) with no collective on the data path.  The
job-level throughput is all ranks' work divided by the slowest rank's time.

Works with any torch.distributed backend (nccl on GPUs, gloo on CPU)."""
import numpy as np
import torch
import torch.distributed as dist


def replica_key(seed, rank):
    """PRNGKey-layout key {0, seed + rank} of one replica."""
    return np.array([0, int(seed) + int(rank)], dtype=np.uint32)


def split_batch(B, rank, world):
    """[start, stop) of the items (series, posteriors) rank owns: contiguous,
    sizes differing by at most one, all B covered once."""
    q, r = divmod(int(B), int(world))
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def aggregate(units, seconds):
    """(value, max_seconds, total_units): value = total units over all ranks / the
    largest per-rank time.  Without an initialised process group: this rank alone."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(units) / float(seconds), float(seconds), float(units)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u) / float(t), float(t), float(u)
