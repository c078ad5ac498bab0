"""The several-GPU host path on CPUs: two gloo ranks time the same work,
agree on the slowest rank's time, and the cell partition covers every cell
once with balanced compartment totals."""
import os
import socket

import numpy as np
import torch.multiprocessing as tmp

from moose_gb300 import models
from moose_gb300.replicas import job_throughput, partition_cells


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from moose_gb300.replicas import barrier, max_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier()
    local = 1.0 + rank          # the slower rank takes 2.0 s
    out[rank] = max_over_ranks(local)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = tmp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == 2.0
    assert job_throughput(100.0, out[0], 2) == 100.0


def test_partition_covers_every_cell_once_and_balances():
    sizes, _, _ = models.population_sizes(3, 1, 4096)
    for world in (1, 2, 4, 8):
        parts = partition_cells(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(4096))
        loads = [int(np.asarray(sizes)[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= int(np.max(sizes))
