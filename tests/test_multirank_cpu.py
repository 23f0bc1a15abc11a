"""The multi-GPU path of the ensemble (instances sharded over ranks, no data-path
collective; only the timing and unit reductions of the benchmark) with world_size 2 on the
gloo backend, on CPU."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from jaxabm_gb300 import ensemble
    spec = ensemble.rank_spec(64, rank)
    seeds = torch.tensor(spec["seed"], dtype=torch.int64)
    gathered = [torch.zeros_like(seeds) for _ in range(world)]
    dist.all_gather(gathered, seeds)
    units = torch.tensor([float(spec["n"].sum() * 365)], dtype=torch.float64)
    ms = torch.tensor([100.0 + rank], dtype=torch.float64)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((torch.cat(gathered).numpy(), float(units.item()), float(ms.item()),
                 spec["n"].copy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    seeds, units, ms, n0 = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert len(np.unique(seeds)) == len(seeds) == 128  # disjoint members
    # both ranks run the same sizes (weak scaling), so the sum is twice one rank's units
    assert units == pytest.approx(2 * n0.sum() * 365)
    assert ms == 101.0  # the slowest rank defines the step time
