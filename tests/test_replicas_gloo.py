"""CPU: the multi-GPU path is replicas only (every rank renders its own frame,
no collective on the data path); the bench combines the ranks' timings (max)
and rays (sum).  Two gloo ranks on 127.0.0.1 exercise that combination and
the reference arm's rank-0-only output."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    secs, rays = bench.combine_replicas(dist, 1.0 + rank, 1000 * (rank + 1), "cpu")
    q.put((rank, secs, rays))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_replicas_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, secs, rays in got:
        assert secs == 2.0 and rays == 3000.0   # slowest rank's time, all ranks' rays


def test_reference_arm_prints_on_rank_zero_only(tmp_path):
    """torchrun-style launch of `bench.py --impl reference` with two CPU ranks
    and a tiny sample: rank 0 prints one JSON line, rank 1 exits 0 silently."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--width", "48",
           "--height", "32", "--spp", "2", "--level", "1", "--cpu-seconds", "0.2"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
