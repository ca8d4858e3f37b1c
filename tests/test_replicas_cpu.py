"""The multi-replica path of bench.py on the CPU: world_size-2 gloo ranks agree on the slowest
replica's time and the whole-job GLUPS (replicas only: the step shards nothing, so no data
crosses ranks)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = bench.dist_env()
    slowest = bench.max_over_ranks(dist, times[rank], "cpu")
    out[rank] = (w, r, slowest, bench.replica_glups(w, 1 << 20, 100, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_replica():
    world, port = 2, _free_port()
    times = [0.25, 0.40]
    with mp.get_context("spawn").Manager() as m:  # no fork of this (threaded) process
        out = m.dict()
        mp.spawn(_rank, args=(world, port, times, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        w, r, slowest, glups = res[rank]
        assert (w, r) == (world, rank)
        assert slowest == pytest.approx(0.40)
        assert glups == pytest.approx(2 * (1 << 20) * 100 / 0.40 / 1e9)


def test_single_process_has_no_collective():
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    assert bench.max_over_ranks(None, 1.5, "cpu") == 1.5
    assert bench.replica_glups(1, 1000, 10, 0.5) == pytest.approx(2e-5)
