"""The N > 1 harness of bench.py on CPU with the gloo backend, world size 2:
the replica barrier and max-over-ranks timing helpers, and a whole
`--impl reference` run under torchrun (rank 0 prints the one JSON line, the
other rank exits without work)."""

import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    world, r, local = bench.dist_setup()
    got = bench.allreduce_max(1.5 * (rank + 1), world)
    bench.barrier(world)
    q.put((r, world, local, got))
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert results == [(0, 2, 0, 3.0), (1, 2, 1, 3.0)]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_world_size_two():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "3",
           "--workload", "dna16x1000_hky"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=550)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
