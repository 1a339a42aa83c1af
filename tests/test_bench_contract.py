"""bench.py's reference arm on the host (no GPU): one JSON line with the contract's keys.

`bench.py --impl reference` times the reference's own step (oracle/_ref, built from its
sources) on bounded samples of the workload, on the host cores; it needs no GPU, so its
output line is checked here.
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    from oracle import ref_runner

    if not ref_runner.available():
        pytest.skip("reference build not available")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["unit"] == "particle-updates/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "colliding_blocks_1m"
    # the line names the sample it ran, not the full scene it was drawn from
    assert d["config"]["source_particles"] == 1048576
    assert d["config"]["particles"] % 4096 == 0 and d["config"]["particles"] < 1048576
    fit = d["extrapolated_1m"]
    assert fit["kind"] == "extrapolated" and len(fit["measured"]) >= 3 and 0 < fit["value"] < d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    """Under torchrun with two ranks, rank 0 alone runs the reference arm and prints its
    line; the other rank exits 0 without work."""
    import socket

    from oracle import ref_runner

    if not ref_runner.available():
        pytest.skip("reference build not available")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                          "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


@pytest.mark.gpu
def test_gpu_arm_prints_one_contract_line():
    """The default arm on a GB300: one JSON line with the contract's keys, the roofline of
    the dominant kernel and of every phase, the end-to-end figure with its copies counted,
    and the number of this library's launches in the timed region."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--steps", "3", "--warmup", "3",
                          "--no-cpu-baseline", "--no-autotune", "--no-batched", "--no-adjoint", "--no-surface",
                          "--no-render"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config", "roofline", "e2e", "gpu_launches", "clocks"):
        assert key in d, key
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["value"] > 0
    assert d["config"]["workload"] == "colliding_blocks_1m" and d["config"]["particles"] == 1048576
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    assert r["kernel"] in r["kernels"]
    for k in ("lambda", "deltap", "neighbors", "xsph", "vorticity"):
        assert 0 < r["kernels"][k]["frac"] < 1.5, (k, r["kernels"][k])
    assert r["kernels"]["deltap"]["per"] == "launch" and r["kernels"]["deltap"]["launches_per_step"] == 4
    e = d["e2e"]
    assert e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 1048576 * 24
    assert 0 < e["value"] < d["value"]
    assert d["gpu_launches"] == 3 * 20  # kernels a step with statistics on, over the timed steps
