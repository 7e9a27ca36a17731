"""The N > 1 path of bench.py on the CPU (gloo, world size 2): the timing is
the slowest rank's (a MAX all-reduce), the value the whole job's throughput
over all replicas, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")  # rank 1 is the slow one
    value = bench.replica_throughput(world, 3, 1000, ms)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, value))


def test_max_over_ranks_and_replica_throughput_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in res:
        assert ms == 15.0  # every rank reports the slowest rank's time
        assert value == pytest.approx(2 * 3 * 1000 / 0.015)  # all replicas' work over that time


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(7.5) == 7.5
    assert bench.replica_throughput(1, 2, 10, 1000.0) == pytest.approx(20.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = types.SimpleNamespace(steps=1, warmup=0, gpus=2)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""  # no work and no line from rank 1
