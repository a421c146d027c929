"""The multi-process path of bench.py on the CPU (gloo, world size 2): the
rank helper's barrier and max over ranks, and a whole torchrun launch of the
reference arm, where rank 0 alone measures and prints one line. Every rank of
a GPU run is a replica (no data-path collective), so these cover all the
host-side logic of N > 1."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_CHILD = r"""
import os, sys
sys.path.insert(0, os.environ["ROOT"])
import bench
r = bench.Ranks()
r.barrier()
m = r.max(float(r.rank + 1) * 1.5)
print(f"rank {r.rank} world {r.world} max {m}", flush=True)
r.close()
"""


def test_rank_helper_max_over_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    port = _port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    lines = sorted(o.strip() for o, _ in outs)
    assert lines == ["rank 0 world 2 max 3.0", "rank 1 world 2 max 3.0"]


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch.distributed.run")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port()), "bench.py", "--impl", "reference",
           "--config", "1", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                                   # rank 0 alone reports
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "unavailable" in d["reference_cuda"] or d["reference_cuda"]["value"] > 0
