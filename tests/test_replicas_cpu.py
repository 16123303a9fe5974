"""Multi-process path of bench.py on CPU (gloo, world size 2).

The engine runs one LP per GPU; more GPUs run replicas of the workload
(weak scaling) whose timing is the maximum over ranks. These tests run that
host logic with two gloo ranks: the max-over-ranks reduction, and the
reference arm under torchrun, where rank 0 alone measures and prints one
JSON line and the other rank exits cleanly.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import os, sys
sys.path.insert(0, os.environ["IGX_ROOT"])
import torch.distributed as td
import bench
td.init_process_group("gloo")
rank = int(os.environ["RANK"])
v = bench.barrier_max(1.5 + rank, 2)
bench.barrier(2)
with open(os.path.join(os.environ["IGX_OUT"], "rank%d.txt" % rank), "w") as f:
    f.write("max %r" % v)
td.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout, out_dir=""):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    env = dict(os.environ, IGX_ROOT=ROOT, IGX_OUT=str(out_dir), OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=timeout)


def test_barrier_max_over_two_gloo_ranks(tmp_path):
    script = tmp_path / "probe.py"
    script.write_text(PROBE)
    r = torchrun([str(script)], timeout=300, out_dir=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    for rank in (0, 1):
        assert (tmp_path / f"rank{rank}.txt").read_text() == "max 2.5"


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("numpy")
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                  "--warmup", "1", "--scale", "0.01", "--cpu-iters", "4"], timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["scaling"] == "weak"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
