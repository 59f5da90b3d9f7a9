"""The bench's N > 1 host logic on CPU with two gloo ranks: the job time is the slowest
rank's, the job rate counts every rank's units, and the reference arm runs on rank 0 only.
(The path has no data exchange: stencils are independent and every rank is a replica.)"""
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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        out[rank] = (ms, bench.job_rate(1000, world, ms))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    assert out[0] == out[1]
    ms, rate = out[0]
    assert ms == 15.0  # the slowest rank's time
    assert rate == pytest.approx(2 * 1000 / 15e-3)


def test_reference_arm_rank_nonzero_does_nothing(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    # rank 1 returns before any work: its arguments are not even read
    assert bench.run_reference(None, bench.CONFIGS["lap3d_4M"], 1000) is None
    assert capsys.readouterr().out == ""
