"""Replicas over ranks (mysph_gb300/replicas.py) with world size 2 on the
gloo backend: sharding of independent systems, the max-over-ranks job
time, gathered results, and an ensemble advanced shard-wise on the CPU
oracle equal to the same ensemble advanced serially."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mysph_gb300 import replicas as R


def test_shard_partitions():
    items = list(range(11))
    parts = [R.shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items
    assert all(len(p) in (3, 4) for p in parts)
    with pytest.raises(ValueError):
        R.shard(items, 3, 3)
    w = [9.0, 1.0, 5.0, 5.0, 2.0, 8.0]
    by = R.shard_by_work(w, 2)
    assert sorted(sum(by, [])) == list(range(6))
    loads = [sum(w[k] for k in p) for p in by]
    assert abs(loads[0] - loads[1]) <= 2.0
    assert R.job_throughput([100, 300], [2.0, 4.0]) == 100.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from mysph_gb300 import cases
        from oracle.oracle import Oracle
        assert R.max_over_ranks(1.5 + rank) == 1.5 + world - 1
        assert R.sum_over_ranks(1.0) == float(world)
        specs = cases.ensemble_specs(count=5, seed=3, n_lo=200, n_hi=600)
        mine = R.shard(list(range(len(specs))), rank, world)
        res = {}
        for k in mine:
            m = cases.ensemble_member(specs[k])
            o = Oracle(m)
            o.advance(3)
            res[k] = o.field("X")[: m.n_real].copy()
        got = R.gather(res)
        if rank == 0:
            merged = {}
            for part in got:
                assert not set(part) & set(merged)
                merged.update(part)
            out.put({k: v.tolist() for k, v in merged.items()})
    finally:
        dist.destroy_process_group()


def test_gloo_world_of_two_ensemble_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from mysph_gb300 import cases
    from oracle.oracle import Oracle
    specs = cases.ensemble_specs(count=5, seed=3, n_lo=200, n_hi=600)
    assert sorted(merged) == list(range(5))
    for k, sp in enumerate(specs):
        m = cases.ensemble_member(sp)
        o = Oracle(m)
        o.advance(3)
        assert np.array_equal(np.array(merged[k]), o.field("X")[: m.n_real])
