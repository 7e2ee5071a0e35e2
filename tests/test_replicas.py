"""The N>1 bench path is N independent replicas (the sector's apply does not
shard without an all-gather per matvec): timing is the MAX over ranks and the
value aggregates all ranks' bytes.  Exercised with gloo, world_size 2, on CPU."""
import os
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = bench.dist_env()
    m = bench.max_over_ranks(10.0 + rank, dist)
    v = bench.replica_throughput(1e9, 5, w, m)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, m, v))


def test_replicas_take_max_time_and_aggregate_bytes():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 500)
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 11.0 for o in out)                       # slowest rank's time
    assert all(abs(o[3] - 2 * 1e9 * 5 / 11e-3 / 1e9) < 1e-6 for o in out)


def test_single_process_defaults():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.replica_throughput(2e9, 10, 1, 1000.0) == pytest.approx(20.0)
