"""Multi-rank paths of bench.py on CPU: two gloo ranks over 127.0.0.1.

The GPU data path shards by walks with no collective; the only cross-rank steps are the
timing and pair-count reductions (max of the elapsed times, sum of the pairs) and the
reference arm, which rank 0 alone runs and prints.
"""
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


def _reductions(rank, ws, port):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    r, w, local, dist = bench.dist_setup()
    assert (r, w, local) == (rank, ws, rank) and dist is not None
    # per-rank elapsed times and pair counts, as the timed region produces them
    assert bench.max_over_ranks(1.5 + rank, dist, "cpu") == 1.5 + (ws - 1)
    assert bench.sum_over_ranks(10.0 * (rank + 1), dist, "cpu") == 10.0 * ws * (ws + 1) / 2
    dist.barrier()
    dist.destroy_process_group()


def test_rank_reductions_two_gloo_ranks():
    mp.spawn(_reductions, args=(2, _free_port()), nprocs=2, join=True)


def test_single_rank_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_setup() == (0, 1, 0, None)
    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.sum_over_ranks(4.0, None, "cpu") == 4.0


def test_reference_arm_prints_once_from_rank_zero(oracle_mod):
    env = dict(os.environ, BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--workload", "tiny", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
