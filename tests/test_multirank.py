"""The multi-rank form of bench.py on CPU, with gloo and two ranks: the path does not shard across GPUs beyond
replicas (one per rank, no data-path collective), so what needs testing is the job's clock and the whole-job value:
every rank gets the slowest rank's time, the value counts every rank's cells, and the reference arm's ranks past 0
do no work and print nothing."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ms = 100.0 + 17.0 * rank  # each replica's own time
    dist.barrier()
    job_ms = bench.max_over_ranks(ms, "cpu")
    value = bench.whole_job_cells_per_s(world, 8, 16200, 50, job_ms)
    out.put((rank, job_ms, value))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value_with_gloo():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 100.0 + 17.0 * (world - 1)
    for rank, job_ms, value in got:
        assert job_ms == slowest
        assert value == pytest.approx(world * 8 * 16200 * 50 / (slowest / 1e3))


def test_single_process_time_is_its_own():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(12.5, "cpu") == 12.5


def test_reference_arm_ranks_past_zero_do_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
