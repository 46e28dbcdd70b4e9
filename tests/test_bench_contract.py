"""bench.py prints one JSON line with the fields its consumers read: the
reference arm (the reference's CPU implementation, runs without a GPU) and
the GB300 arm (GPU)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e"}


def _run(args, timeout):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run(["--impl", "reference", "--steps", "1", "--warmup", "3"], 600)
    assert BASE_KEYS <= set(d) and d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1 and d["warmup"] >= 3
    assert d["config"]["workload"] == "rayleigh_taylor_512x1536_fp64"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_loads_no_gpu_library():
    """The reference arm parses its .ini with the oracle's readInifile and
    steps the oracle: no library of the GPU path enters its process."""
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3'];"
            "bench.main(); maps = open('/proc/self/maps').read();"
            "print('LOADED_GB300' if 'libfv3d_gb300' in maps else 'CLEAN')")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().splitlines()[-1] == "CLEAN", r.stdout[-2000:]


@pytest.mark.gpu
def test_gb300_arm_line():
    d = _run(["--steps", "3", "--warmup", "3", "--no-variants"], 900)
    assert BASE_KEYS <= set(d) and d.get("impl", "gb300") != "reference"
    assert d["value"] > 0 and d["unit"] == "Mcell-updates/s" and d["dtype"] == "f64"
    rl = d["roofline"]
    assert rl["bound"] == "hbm" and rl["unit"] == "GB/s" and 0 < rl["frac"] == pytest.approx(rl["achieved"] / rl["peak"])
    assert rl["traffic"] > 0 and 0 < rl["fp64_pipe"]["frac"] <= 1.2
    assert d["e2e"]["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] == 3 * d["steps"]
    assert d["cpu_baseline"]["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert max(d["rel_l1_vs_oracle_one_step"].values()) == 0.0
