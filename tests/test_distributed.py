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


def _bench(*argv, env_extra=None):
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(root, "bench.py"), *argv], capture_output=True, text=True,
                          timeout=300, cwd=root, env=env)


def test_gpus_flag_starts_that_many_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself: the
    printed n_gpus equals the world size, and the ranks own disjoint seed
    blocks on devices 0 and 1."""
    import json
    r = _bench("--gpus", "2", "--plan", "--events", "30")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == d["world_size"] == 2
    ranks = sorted(d["ranks"], key=lambda x: x["rank"])
    assert [x["device"] for x in ranks] == [0, 1]
    assert ranks[0]["seeds"] == [1000, 1030] and ranks[1]["seeds"] == [1030, 1060]


def test_gpus_flag_must_match_the_launcher():
    r = _bench("--gpus", "2", "--plan", env_extra={"WORLD_SIZE": "3", "RANK": "0", "LOCAL_RANK": "0"})
    assert r.returncode != 0 and "WORLD_SIZE=3" in r.stderr
    r = _bench("--plan", "--events", "10")
    assert r.returncode == 0 and '"world_size": 1' in r.stdout
