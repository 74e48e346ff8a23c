"""Multi-process paths on the CPU (gloo): the path shards into independent replicas, so the only
cross-rank steps are the bench's barrier and max-over-ranks timing, and its rank-0-only
reporting. Both are exercised with two ranks."""
import json
import os
import socket
import subprocess
import sys

import pytest

from tests.conftest import ROOT


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(w, 10.0 * r + 1.0)
    bench.barrier(w)
    out.put((r, w, m))
    import torch.distributed as td

    td.destroy_process_group()


def test_barrier_and_max_over_ranks_with_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 11.0), (1, 2, 11.0)]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_zero():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--instances-log2", "10", "--rays-log2", "14"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
