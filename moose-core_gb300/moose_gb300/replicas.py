"""Several GPUs: cells are independent (no inter-cell synapses), so every
GPU runs its own batch and nothing is exchanged while stepping.

* ``replicas`` (what bench.py measures): every rank steps the same workload;
  the job's throughput is the sum over ranks, timed from a common barrier to
  the slowest rank.
* ``partition_cells``: a population split over ranks, balanced by
  compartment count (longest first), for a user who wants one population
  spread over several GPUs.

Only host-side collectives are used (a barrier and one max-reduction of the
elapsed time), through torch.distributed with NCCL on GPUs or gloo on CPUs.
"""
import heapq

import numpy as np


def partition_cells(sizes, world):
    """Cell indices of each rank: every cell once, ranks' compartment totals
    balanced (LPT: cells by decreasing size to the least-loaded rank)."""
    sizes = np.asarray(sizes)
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in np.argsort(-sizes, kind="stable"):
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(p) for p in parts]


def max_over_ranks(x, device="cpu"):
    """Max of a float over all ranks (x itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(device=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        if device is not None and dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device])
        else:
            dist.barrier()


def job_throughput(units_per_rank, elapsed_s, world):
    """Units all ranks processed per second, timed to the slowest rank."""
    return world * units_per_rank / elapsed_s
