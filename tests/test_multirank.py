"""The multi-process (torchrun) paths of bench.py on CPU with 2 gloo ranks:
every rank runs its own replica, rank 0 alone prints one JSON line, and the
timing is the maximum over ranks."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--graphs", "12", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=280, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0


WORKER = r"""
import os, sys, json
sys.path.insert(0, %r)
import bench
rank, world, _ = bench.dist_info()
d = bench.Dist(world)
d.barrier()
local_ms = 10.0 + 5.0 * rank
m = d.max(local_ms)
d.barrier()
if rank == 0:
    print(json.dumps({"max_ms": m, "value": world * 100 * 1000.0 / m}))
"""


def test_dist_helper_takes_the_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "worker.py"
    script.write_text(WORKER % ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=200)
    assert r.returncode == 0, r.stderr[-2000:]
    rec = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert rec["max_ms"] == 15.0
    assert abs(rec["value"] - 2 * 100 * 1000.0 / 15.0) < 1e-9


def test_reference_arm_json_line_carries_the_contract_keys():
    """One process: the reference arm's line has the keys of the bench
    contract, its cpu_baseline describes this run, and its e2e moves no
    bytes (the work runs on the host)."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--graphs", "12", "--steps", "2",
           "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=280, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    rec = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in rec, k
    assert rec["impl"] == "reference" and rec["steps"] == 2 and rec["warmup"] == 3 and rec["n_gpus"] == 1
    assert rec["higher_is_better"] is True and rec["value"] > 0 and rec["ms_per_step"] > 0
    import bench
    assert rec["config"] == bench.common_config(12)          # the same config as the GPU arm's line
    assert rec["reference"]["odp_gb300_mapped"] is False
    cb = rec["cpu_baseline"]
    assert cb["value"] == rec["value"] and cb["unit"] == rec["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    e = rec["e2e"]
    assert e["value"] == rec["value"] and e["unit"] == rec["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_each_rank_is_pinned_to_its_local_gpu(monkeypatch):
    """Under torchrun the GPU arm narrows CUDA_VISIBLE_DEVICES to the rank's
    local device (the n-th of the visible ones) before CUDA starts."""
    import bench
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    assert bench.pin_local_gpu(1) == 5 and os.environ["CUDA_VISIBLE_DEVICES"] == "5"
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    assert bench.pin_local_gpu(2) == 2 and os.environ["CUDA_VISIBLE_DEVICES"] == "2"
