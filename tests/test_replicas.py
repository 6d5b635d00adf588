"""bench.py's multi-GPU mode runs independent replicas (the path has no data
exchange between GPUs): the job's step time is the slowest rank's and the
throughput counts every rank's particles.  Checked with two gloo ranks on CPU;
the reference arm does no work on ranks other than 0."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    out.put((rank, ms, bench.job_throughput(1000, world, ms)))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 1000 / 0.015) < 1e-6 for r in res)


def test_reference_arm_other_ranks_do_nothing(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    assert bench.run_reference(bench.parse()) == 0
