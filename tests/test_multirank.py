"""The multi-GPU host path of bench.py on CPU: world size 2 over gloo (replicas, no data-path
collective; the job is timed by its slowest rank and counts every rank's units)."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, ms_by_rank, out):
    sys.path.insert(0, HERE)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_info()
        ms = bench.reduce_max(ms_by_rank[rank], w)
        value = bench.job_throughput(1000.0, w, ms)
        out.put((r, w, local, ms, value))
    finally:
        dist.destroy_process_group()


def test_two_rank_reduction_over_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ms_by_rank = [3.0, 5.0]
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, ms_by_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, local, ms, value) in enumerate(results):
        assert (rank, w, local) == (r, 2, r)
        assert ms == 5.0                                  # slowest rank
        assert value == pytest.approx(2 * 1000.0 / 5e-3)  # both ranks' units


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, HERE)
    import bench
    assert bench.reduce_max(4.0, 1) == 4.0
    assert bench.job_throughput(10.0, 1, 2.0) == pytest.approx(5000.0)


def test_reference_arm_other_ranks_do_no_work(capsys, monkeypatch):
    sys.path.insert(0, HERE)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.run_reference(type("A", (), {"case": "config2", "cpu_pulses": 8, "warmup": 0, "steps": 1})())
    assert capsys.readouterr().out == ""
