"""bench.py's replica path on two CPU ranks (gloo): the job's step time is the
slowest rank's, the job rate counts every replica's bytes, and the CPU reference
arm runs on rank 0 only."""
import socket

import pytest
import torch
import torch.distributed as tdist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    tdist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                             world_size=world)
    try:
        # each replica times its own steps; the job time is the maximum
        ms = [2.5, 4.0][rank]
        tdist.barrier()
        got = bench.max_over_ranks(ms, torch.device("cpu"))
        rate = bench.job_rate(world, 1_000_000_000, got)
        # rank 1 of the reference arm returns without work or output
        ran = None
        if rank == 1:
            bench.run_reference(None, rank)
            ran = "skipped"
        q.put((rank, got, rate, ran))
    finally:
        tdist.destroy_process_group()


def test_max_over_ranks_and_job_rate_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate, ran in out:
        assert got == 4.0                      # slowest replica
        assert rate == pytest.approx(2 * 1.0 / 4.0e-3)  # 2 replicas x 1 GB / 4 ms
    assert out[1][3] == "skipped"


def test_single_process_helpers():
    assert bench.max_over_ranks(3.25, torch.device("cpu")) == 3.25
    assert bench.job_rate(1, 2_000_000_000, 1.0) == pytest.approx(2000.0)
