"""The multi-GPU form is replicas only (independent solves, no data-path collective): each rank runs
its own solve and the job's time is the slowest rank's. Checked here with two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [120.0, 150.0][rank]
    ms = bench.max_over_ranks(local_ms, world, "cpu")
    value = bench.whole_job_rate(1000, 10, world, ms)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, value))


def test_two_replicas_take_the_slowest_rank_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in results:
        assert ms == 150.0
        assert value == pytest.approx(1000 * 3 * 10 * 2 / 0.150 / 1e6)


def test_reference_arm_only_rank0_reports(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 1, 1, 2

    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
