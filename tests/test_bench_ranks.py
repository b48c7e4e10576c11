"""
The multi-rank host logic of bench.py on CPU: ranks are replicas of the
workload (each GPU renders the whole configuration), the job time is the
slowest rank's, the value counts every rank's pixel-iterations, and the
reference arm runs on rank 0 only.  Two gloo ranks on 127.0.0.1.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        secs = bench.job_seconds(1.0 + rank, dist, "cpu")
        out[rank] = (secs, bench.job_value(1e9, 10, world, secs))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_slowest_rank_on_every_rank():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0
    assert res[0][1] == res[1][1] == pytest.approx(1e9 * 10 * 2 / 2.0)


def test_single_rank_needs_no_process_group():
    assert bench.job_seconds(3.5) == 3.5
    assert bench.job_value(2e9, 5, 1, 2.0) == pytest.approx(5e9)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""
