"""The N > 1 path of bench.py on the CPU: two gloo ranks on 127.0.0.1.

The batched solve does not shard across GPUs (independent matrices, no
exchange step), so N ranks run N replicas; the only cross-rank logic is the
timing and the aggregate: a barrier around the timed region, the units every
rank completed summed, the slowest rank's time, and rank 0 alone printing.
The reference arm runs on rank 0 only; the other ranks exit without work."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, results):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo")     # gloo even where CUDA is present; dist_setup reuses it
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and pg is not None
    # the same group again (bench.run_reference calls dist_setup after run setup)
    assert bench.dist_setup()[3] is pg
    bench.barrier(pg)
    # rank r completed 100 * (r + 1) solves in 10 * (r + 1) ms
    rate, slowest = bench.aggregate_rate(pg, 100 * (rank + 1), 10.0 * (rank + 1), None)
    bench.barrier(pg)

    class _NoWork:
        def cpu_sample(self, *a, **k):
            raise AssertionError("a rank other than 0 ran the reference sample")

    class _Args:
        steps, warmup, gpus = 1, 0, world

    rc = bench.run_reference(_Args(), _NoWork()) if rank != 0 else 0
    results[rank] = (rate, slowest, rc)
    pg.destroy_process_group()


def test_two_rank_aggregate_and_reference_arm():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        results = mgr.dict()
        mp.start_processes(_rank, args=(world, port, results), nprocs=world, join=True,
                           start_method="spawn")
        got = dict(results)
    assert set(got) == {0, 1}
    for rank in range(world):
        rate, slowest, rc = got[rank]
        assert slowest == pytest.approx(20.0)
        assert rate == pytest.approx((100 + 200) / 0.020)
        assert rc == 0
