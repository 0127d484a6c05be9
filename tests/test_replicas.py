"""The multi-GPU form of the benchmark: independent replicas, no data exchange.

bench.py --gpus N runs one full closest-hit batch per rank and reports the
whole-job throughput from the slowest rank's time.  That host logic is checked
here with two gloo ranks on the CPU (no GPU, no collective on the data path).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(times[rank], dist, "cpu")
    out.put((rank, slowest, bench.replica_throughput(1000, world, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.5, 0.8]
    port = 29000 + os.getpid() % 2000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, value in res:
        assert slowest == 0.8
        assert value == pytest.approx(2 * 1000 / 0.8 / 1e6)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25
    assert bench.replica_throughput(16_777_216, 1, 0.01678) == pytest.approx(16_777_216 / 0.01678 / 1e6)
