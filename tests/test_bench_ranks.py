"""The replicas-only multi-GPU path of bench.py on CPU: world_size-2 gloo
ranks report the max-over-ranks time and the whole-job rate, and the
reference arm's non-zero ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r pretends its K steps took 100 (r + 1) ms
        q.put((rank, bench.job_rate(100.0 * (rank + 1), world, 500, dist, "cpu")))
    finally:
        dist.destroy_process_group()


def test_job_rate_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms, val = res[r]
        assert ms == 200.0                      # the slower rank's time
        assert abs(val - 2 * 500 / 0.2) < 1e-9  # all ranks' units / max time


def test_job_rate_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.job_rate(250.0, 1, 100) == (250.0, 400.0)


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
