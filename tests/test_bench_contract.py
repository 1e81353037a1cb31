"""The benchmark's JSON line: the keys and value types every run must print.

The reference arm runs on the CPU (the oracle restatement over the host cores); the
GPU arm is run with its optional legs switched off."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE = {"metric": str, "value": float, "unit": str, "n_gpus": int, "steps": int, "warmup": int,
        "ms_per_step": float, "higher_is_better": bool, "scaling": str, "dtype": str,
        "data": str, "config": dict, "cpu_baseline": dict, "e2e": dict}


def _run(args, timeout):
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT,
                       capture_output=True, text=True, timeout=timeout, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def _check_base(d):
    for k, t in BASE.items():
        assert k in d, k
        assert isinstance(d[k], t) or (t is float and isinstance(d[k], int)), (k, d[k])
    assert "workload" in d["config"]
    assert d["vs_baseline"] is None
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in d["e2e"], k
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in d["cpu_baseline"], k


def test_reference_arm_json():
    d = _run(["--impl", "reference", "--steps", "1", "--warmup", "0", "--size", "16"],
             timeout=600)
    _check_base(d)
    assert d["impl"] == "reference" and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["value"] > 0
    assert d["unit"] == "solves/s" and d["dtype"] == "f64"
    assert d["config"]["cells_per_side"] == 16 and d["config"]["rtol"] == 1e-10


@pytest.mark.gpu
def test_gpu_arm_json(cuda):
    d = _run(["--steps", "2", "--warmup", "3", "--batched", "0", "--serving", "0",
              "--newton", "0", "--size", "32", "--fp64-solves", "1", "--cpu-iterations", "1"],
             timeout=900)
    _check_base(d)
    assert d["unit"] == "solves/s" and d["converged"] and d["rel_res"] <= 1e-10
    assert d["fp64_solve"]["converged"] and d["fp64_solve"]["rel_res"] <= 1e-10
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and 0 < rf["frac"] < 1.5
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    assert d["gpu_launches"] > 0 and "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
