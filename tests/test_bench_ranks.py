"""The benchmark's multi-process host logic on CPU (gloo, two ranks on
127.0.0.1): the path does not shard, so N GPUs run N replicas, timed as the
maximum over ranks and summed by rank 0; the reference arm runs on rank 0
alone and the other ranks exit without output."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CANS_BENCH_GLOO="1")
    sys.path.insert(0, str(ROOT))
    import bench
    ws, r, local = bench.dist_setup()
    bench.barrier(ws)
    out.put((r, ws, bench.max_over_ranks(1.5 + r, ws)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_with_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_zero():
    pytest.importorskip("torch")
    env = dict(os.environ, CANS_BENCH_GLOO="1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
