"""bench.py's multi-rank path on the CPU (gloo, world size 2): the max-over-ranks reduction and barrier
that time the replicas, and the reference arm under torchrun, where rank 0 alone runs and prints one JSON
line and the other rank exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    ws, r, _ = bench.dist_init()
    bench.barrier(ws)
    v = bench.allreduce_max(ws, float(rank + 1) * 1.5)
    bench.barrier(ws)
    out[rank] = (ws, r, v)
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(port, out), nprocs=2, join=True)
    assert sorted(out.keys()) == [0, 1]
    for rank in (0, 1):
        ws, r, v = out[rank]
        assert ws == 2 and r == rank and v == 3.0


def test_reference_arm_two_ranks_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--size", "16"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["cpu_baseline"]["kind"] == "port"
