"""The bench's N > 1 path on the CPU (gloo, world size 2, 127.0.0.1).

The served and batched solves shard as independent replicas -- no data-path
collective -- so what N > 1 needs is the harness: the barrier, the maximum of
the timed region over ranks, and the reference arm, which runs on rank 0 only
and lets the other ranks exit without work.
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


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    class A:
        impl = "reference"  # gloo on the CPU

    ws, r, local, pg = bench.dist_setup(A())
    bench.barrier(pg)
    m = bench.max_over_ranks(pg, 1.5 + rank)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"ws": ws, "rank": r, "max": m}, f)
    pg.destroy_process_group()


def test_barrier_and_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(port, str(tmp_path)), nprocs=2, join=True)
    for rank in (0, 1):
        d = json.load(open(tmp_path / ("rank%d.json" % rank)))
        assert d == {"ws": 2, "rank": rank, "max": 2.5}


def test_reference_arm_runs_on_rank_0_only():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 times
    the CPU oracle and prints one JSON line, rank 1 exits 0 without output."""
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
