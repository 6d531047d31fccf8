"""The N > 1 path of bench.py on CPU (gloo, world size 2): every rank runs a
replica of the workload, the job time is the slowest rank's (all-reduce MAX)
and the reported rate is the whole job's (the path shards by shot; one GPU per
call here, so the ranks are replicas and no data-path collective exists)."""
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


def _worker(rank, world, port, out):
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = 1.0 + rank  # rank 1 is slower
        tmax = bench.max_over_ranks(t, dist, torch.device("cpu"))
        out[rank] = (tmax, bench.whole_job_rate(100.0, 3, world, tmax))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this (threaded) process
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0
    assert res[0][1] == res[1][1] == pytest.approx(100.0 * 3 * 2 / 2.0)


def test_single_rank_is_identity():
    import bench

    assert bench.max_over_ranks(1.5) == 1.5
    assert bench.whole_job_rate(10.0, 2, 1, 4.0) == 5.0
