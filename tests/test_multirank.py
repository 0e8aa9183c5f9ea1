"""The multi-GPU paths of bench.py on the CPU (gloo, world size 2): replicas
(the job's time is the slowest rank's, throughput counts every rank's
particles), the ensemble split by scenes (every rank derives the same
disjoint, complete, balanced plan), and the reference arm's non-zero ranks
exiting without work."""
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


def _ensemble_sizes(seed=42, scenes=256):
    import numpy as np
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(4096), np.log(65536), scenes)).astype(int)
    return [max(512, (int(v) + 256) // 512 * 512) for v in n]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_shard_scenes(world):
    sys.path.insert(0, ROOT)
    import bench
    sizes = _ensemble_sizes()
    plans = [bench.shard_scenes(sizes, world, r) for r in range(world)]
    flat = sorted(k for p in plans for k in p)
    assert flat == list(range(len(sizes)))  # complete and disjoint
    assert all(p == sorted(p) for p in plans)
    loads = [sum(sizes[k] for k in p) for p in plans]
    assert max(loads) - min(loads) <= max(sizes)
    if world == 1:
        assert plans[0] == list(range(len(sizes)))


def _ensemble_worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    sizes = _ensemble_sizes()
    mine = bench.shard_scenes(sizes, world, rank)
    plans = [None] * world
    dist.all_gather_object(plans, mine)
    slowest = bench.max_over_ranks(5.0 + rank)
    value = bench.ensemble_throughput(sum(sizes), 500, slowest)
    bench.barrier()
    dist.destroy_process_group()
    q.put((rank, plans, slowest, value))


def test_ensemble_split_gloo():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ensemble_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    total = sum(_ensemble_sizes())
    assert res[0][1] == res[1][1]  # the same plan on both ranks
    assert sorted(res[0][1][0] + res[0][1][1]) == list(range(256))
    for rank, plans, slowest, value in res:
        assert slowest == 6.0
        assert value == pytest.approx(total * 500 / 0.006)
