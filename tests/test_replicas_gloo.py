"""The multi-GPU path of bench.py on CPU: independent replicas, one process per GPU,
no data-path collective.  Two gloo ranks check the timing reduction (each rank's
timed milliseconds -> the slowest rank's, the whole-job rate = ranks x steps in that
time), and the reference arm does no work on ranks other than 0."""
import argparse
import os
import socket

import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, ms, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        slowest = bench.max_over_ranks(ms[rank])
        q.put((rank, slowest, bench.whole_job_rate(world, 5, slowest)))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_whole_job_rate():
    world, ms = 2, [120.0, 150.0]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, ms, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in range(world))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert [g[0] for g in got] == [0, 1]
    for _, slowest, rate in got:
        assert slowest == 150.0
        assert abs(rate - world * 5 / 0.150) < 1e-9


def test_single_process_keeps_its_own_time():
    assert bench.max_over_ranks(87.5) == 87.5
    assert abs(bench.whole_job_rate(1, 4, 500.0) - 8.0) < 1e-12


def test_reference_arm_runs_on_rank_0_only(capsys):
    args = argparse.Namespace(config=1, steps=1, warmup=0, out=".")
    assert bench.run_reference(args, 1, 2) is None
    assert capsys.readouterr().out == ""
