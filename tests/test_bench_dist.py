"""Multi-rank aggregation of bench.py on CPU (gloo, world_size 2): each rank's
timed region is reduced to the slowest rank's time and the whole-job throughput
counts every rank's queries (weak scaling, replicas)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        local_ms = 100.0 + 50.0 * rank          # rank 1 is the slower one
        total = bench.max_over_ranks(local_ms, ws)
        out[rank] = (total, bench.job_qps(total, ws, 10_000, 4))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_qps_gloo():
    ws = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    # 2 ranks x 10k queries x 4 steps over 0.15 s
    assert res[0][1] == pytest.approx(2 * 10_000 * 4 / 0.15)


def test_single_rank_is_identity():
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_qps(1000.0, 1, 10_000, 10) == pytest.approx(100_000.0)
