"""bench.py with N > 1 processes: the path has no exchange step, so N GPUs run
N replicas of the workload, and the job time is the slowest replica's (the
maximum over ranks); the reference arm runs on rank 0 alone.  The rank logic
runs here as world_size-2 gloo process groups on the CPU."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, values, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.max_over_ranks(values[rank], "cpu")))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("values", [(0.25, 0.5), (3.0, 1.0)])
def test_job_time_is_the_slowest_replica(values):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: max(values), 1: max(values)}


def test_one_process_keeps_its_own_time():
    assert bench.max_over_ranks(0.125, "cpu") == 0.125


def test_reference_arm_runs_on_rank_zero_only():
    # rank 1 of 2 (as torchrun starts it): no work, no line, exit 0
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
