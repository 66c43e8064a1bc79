"""The multi-rank path of the benchmark on CPU: two gloo ranks (127.0.0.1)
run its process-group setup, barrier, max-over-ranks timing, per-rank
particle seeds and whole-job weak-scaling rate.  The E-step shards over
particles with no exchange, so the only collectives are the barrier around
the timed region and the max of the ranks' times."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK="0",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.init_dist()
    assert (r, w, local) == (rank, world, 0)
    bench.barrier(w)
    # ranks finish their steps at different times; the slowest sets the job's time
    ms = bench.reduce_max(w, 10.0 + 5.0 * rank)
    rate = bench.job_rate(64 * 3, ms, w)
    out.put((rank, ms, rate, bench.rank_seed(1001, r)))
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_single_rank_helpers_need_no_process_group():
    import bench
    assert bench.reduce_max(1, 3.5) == 3.5
    bench.barrier(1)
    assert bench.rank_seed(1001, 0) == 1001
    assert bench.job_rate(128 * 150, 2000.0, 1) == pytest.approx(9600.0)


def test_two_gloo_ranks_aggregate_weak_scaling():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    (_, ms0, v0, s0), (_, ms1, v1, s1) = res
    assert ms0 == ms1 == 15.0                      # max over ranks, on every rank
    assert v0 == v1 == pytest.approx(64 * 3 * 2 / 0.015)
    assert s0 != s1                                # each rank has its own particles
