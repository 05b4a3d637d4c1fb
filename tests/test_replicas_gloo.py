"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks (replicas, no data-path collective) agree on the
slowest rank's time, and the whole-job throughput counts every rank's views."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 2.0 + rank          # rank 1 is the slow replica
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    q.put((rank, ms, bench.replicas_throughput(world, ms)))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [3.0, 3.0]
    assert res[0][2] == pytest.approx(2 * 1000.0 / 3.0)
