"""The N > 1 path of bench.py on CPU: world_size-2 gloo process groups
(127.0.0.1). Ranks are replicas (one spot, or one shard of the batched
spots, per GPU) with no exchange in the data path; the only collective is
the max over ranks of the timed region."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "cuda-poker-solver_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from pps import workloads as wl
    slowest = bench.max_over_ranks(10.0 * (rank + 1), dist)
    spots = wl.batched(10, seed=606)
    mine = [s.name for s in bench.shard(spots, rank, world)]
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, mine))


def test_two_rank_timing_and_sharding():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict((r, (t, m)) for r, t, m in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # Every rank sees the slowest rank's time.
    assert out[0][0] == out[1][0] == 20.0
    # Shards are disjoint and cover every spot once.
    names = out[0][1] + out[1][1]
    assert sorted(names) == sorted("batch_%03d" % k for k in range(10))
    assert not set(out[0][1]) & set(out[1][1])
