"""The bench's multi-rank logic on CPU (gloo, world size 2): replicas time
their own work, the job's time is the maximum over ranks, and only rank 0
runs and prints the reference arm."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, os.environ["SFFT_ROOT"])
import bench
ws, rank, local = bench.dist_init()
bench.barrier(ws)
t = bench.max_over_ranks(ws, 1.5 + rank)
called = []
bench.cpu_reference_throughput = lambda *a, **kw: called.append(1) or (1.0, "port", 1, [1.0])
class A: gpus = ws; steps = 1; warmup = 0; batch = 1; pool = 1
bench.reference_arm(A(), ws, rank)
print(json.dumps({"rank": rank, "ws": ws, "max": t, "reference_ran": bool(called)}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_max_and_rank0_reference():
    pytest.importorskip("torch")
    port = _port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), SFFT_BENCH_BACKEND="gloo", SFFT_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=240) for p in procs]
    import json
    lines = []
    for (out, err), p in zip(outs, procs):
        assert p.returncode == 0, err
        lines.extend(json.loads(l) for l in out.splitlines() if l.startswith('{"rank"'))
    ref_lines = [l for (out, _) in outs for l in out.splitlines() if '"impl": "reference"' in l]
    by_rank = {l["rank"]: l for l in lines}
    assert set(by_rank) == {0, 1}
    assert all(l["max"] == 2.5 and l["ws"] == 2 for l in lines)      # the slowest rank's time
    assert by_rank[0]["reference_ran"] and not by_rank[1]["reference_ran"]
    assert len(ref_lines) == 1                                        # one JSON line, from rank 0
