"""The bench's multi-rank path on the CPU (world size 2, gloo).

Under torchrun every rank runs its own replica of the case (no data-path
collective: the path does not shard); the only exchanges are a barrier and the
max of the ranks' times, which max_over_ranks takes over the process group.
The reference arm runs on rank 0 alone; the other ranks exit 0 without work.
"""
import json
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


def _rank_main(rank, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        q.put((rank, bench.max_over_ranks(1.5 + rank, dist), bench.max_over_ranks(7.0 - rank, dist)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2.5, 7.0), (1, 2.5, 7.0)]


def test_max_over_ranks_without_a_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None) == 3.25


def test_reference_arm_under_torchrun_world_size_2():
    """rank 0 prints the reference arm's one JSON line; rank 1 exits 0 without work"""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--preset", "naca0012_0p2m"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
