"""The multi-rank path of bench.py on CPU (gloo, world size 2): ranks rendezvous on
127.0.0.1, the timed value is the maximum over ranks, and the reference arm under
torchrun prints one line from rank 0 while the other rank exits without work.
Replicas only: no collective exists on the data path."""
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


_RANK = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import bench
ws, rank, local, dist = bench.dist_setup(None)
assert ws == 2 and dist is not None
bench.barrier(dist)
m = bench.max_over_ranks(dist, float(rank + 1) * 0.5)
print("MAX", rank, m, flush=True)
dist.destroy_process_group()
"""


def test_ranks_rendezvous_and_take_the_max():
    port = str(_free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=port, WORLD_SIZE="2", RANK=str(r),
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    vals = sorted(float(line.split()[2]) for o, _ in outs for line in o.splitlines() if line.startswith("MAX"))
    assert vals == [1.0, 1.0]


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch.distributed.run")
    port = str(_free_port())
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", port, os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--cpu-n", "12",
           "--cpu-seconds", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
