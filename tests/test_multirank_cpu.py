"""The multi-GPU path of the ensemble (the 4,096 members partitioned across ranks, balanced
by agents, no data-path collective; only the timing and unit reductions of the benchmark)
with world_size 2 on the gloo backend, on CPU.  Unmeasured on hardware: every GPU call of
this build has one GPU."""

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
    spec = ensemble.rank_spec(4096, rank, world)
    seeds = torch.full((4096,), -1, dtype=torch.int64)
    seeds[:len(spec["seed"])] = torch.tensor(spec["seed"], dtype=torch.int64)
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
    # the union of the ranks' members is every member exactly once
    seeds = seeds[seeds >= 0]
    assert len(seeds) == 4096 and np.array_equal(np.sort(seeds), np.arange(4096))
    from jaxabm_gb300 import ensemble
    full = ensemble.ensemble_spec(4096)
    assert units == pytest.approx(full["n"].sum() * 365)  # all ranks together: the whole job
    assert abs(n0.sum() - full["n"].sum() / 2) < full["n"].max()  # balanced by agents
    assert ms == 101.0  # the slowest rank defines the step time


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_members_once(world):
    from jaxabm_gb300 import ensemble
    spec = ensemble.ensemble_spec(4096)
    parts = ensemble.partition_members(spec["n"], world)
    allm = np.concatenate(parts)
    assert np.array_equal(np.sort(allm), np.arange(4096))
    loads = np.array([spec["n"][p].sum() for p in parts])
    assert loads.max() - loads.min() <= spec["n"].max()
    for r in range(world):
        rs = ensemble.rank_spec(4096, r, world)
        assert np.array_equal(rs["member"], parts[r])
        assert np.array_equal(rs["seed"], parts[r])
