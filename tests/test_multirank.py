"""The replica path of bench.py at world size 2 on the CPU (gloo): the job's
time is the slowest rank's, throughput counts every rank's particles, and the
reference arm's non-zero ranks exit without work."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 10.0 * (rank + 1)  # rank 1 is the slowest
    slowest = bench.max_over_ranks(local_ms)
    value = bench.job_throughput(1_048_576, 100, world, slowest)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, value))


def test_replica_throughput_gloo():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, slowest, value in res:
        assert slowest == 20.0
        assert value == pytest.approx(2 * 1_048_576 * 100 / 0.020)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, env=env,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
