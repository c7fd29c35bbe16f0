"""Multi-rank bench plumbing on CPU: gloo, world size 2, 127.0.0.1.

Events shard across ranks with no data-path collective (weak scaling: each
rank owns a disjoint seed block); the only collectives are a barrier and the
max / sum reductions of the step time and event counts.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import bench
    r = bench.Ranks()
    seeds = bench.shard_seeds(1000, 50, r.rank)
    r.barrier()
    mx = r.max(float(rank + 1) * 10.0)
    total = r.sum(float(len(seeds)))
    out[rank] = (seeds.start, seeds.stop, mx, total)
    r.close()


def test_two_rank_sharding_and_reductions():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    a, b = out[0], out[1]
    assert (a[0], a[1]) == (1000, 1050) and (b[0], b[1]) == (1050, 1100)   # disjoint blocks
    assert a[2] == b[2] == 20.0                                            # max over ranks
    assert a[3] == b[3] == 100.0                                           # events over ranks


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "1")
    r = bench.Ranks()

    class A:
        pass
    args = A()
    r.rank = 1
    assert bench.reference_arm(args, r) is None
