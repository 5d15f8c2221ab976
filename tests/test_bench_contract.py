"""bench.py's reference arm on the CPU: the JSON line it prints (the keys the
bench contract fixes, with the reference arm's own: impl, a cpu_baseline
describing the run, an e2e of no copies), at one process and under torchrun
with two gloo ranks, where rank 0 alone prints.  The GPU arm's line is
checked on the GPU (its timing needs the device)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"}


def json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def check_line(d, n_gpus):
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["n_gpus"] == n_gpus and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["unit"] == "residue-steps/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "C4" and d["config"]["residues"] == 14918
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same metric as the GPU arm's line
    sys.path.insert(0, ROOT)
    import bench
    assert d["metric"] == bench.METRIC


ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.5"]


def test_reference_arm_one_process(built):
    out = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = json_lines(out.stdout)
    assert len(lines) == 1
    check_line(lines[0], 1)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks(built):
    """Launched as the driver launches N > 1: rank 0 prints the line, rank 1
    exits 0 without work."""
    pytest.importorskip("torch.distributed")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--gpus", "2"] + ARGS
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = json_lines(out.stdout)
    assert len(lines) == 1
    check_line(lines[0], 2)
