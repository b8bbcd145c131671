"""Multi-rank logic of bench.py on CPU: two gloo ranks (replicas) agree on
the slowest rank's time, the whole-job rate counts every rank's work, and
under torchrun only rank 0 of the reference arm works and prints."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    local_ms = 10.0 + 5.0 * rank            # rank 1 is the slower replica
    total = bench.max_over_ranks(local_ms, ws, "cpu")
    rate = bench.whole_job_rate(1000, 4, ws, total)
    q.put((rank, total, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_slowest_time_and_whole_job_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for _rank, total, rate in got:
        assert total == 15.0                 # the slowest rank's time
        assert rate == pytest.approx(1000 * 4 * 2 / 15e-3)


def test_single_rank_helpers_need_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.whole_job_rate(10, 2, 1, 20.0) == pytest.approx(1000.0)


def test_reference_arm_rank_1_exits_without_work():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], env=env, cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
