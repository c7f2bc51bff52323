"""GPU tests of bench.py's output contract: every workload, run small, prints one JSON line with
the keys the measurement contract asks for (the headline line: metric, value, unit, timing,
config, roofline, cpu_baseline, e2e, gpu_launches, clocks; the reference arm's line: impl,
cpu_baseline and e2e of its own run)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench(*args, timeout=600):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert lines, r.stdout[-2000:]
    return json.loads(lines[-1])


def test_headline_line_keeps_the_contract():
    d = bench("--n", "65536", "--steps", "2", "--warmup", "3")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and "workload" in d["config"]
    r = d["roofline"]
    assert r["bound"] and r["unit"] == "TFLOP/s" and r["peak"] > 0 and 0 < r["frac"] < 1.5
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9 and "traffic" in r
    assert r["executed"]["over_credited"] >= 1.0
    c = d["cpu_baseline"]
    assert c["value"] > 0 and c["kind"] in ("port", "reference") and c["cores"] >= 1 and c["sample"]
    assert c["single_core"]["value"] > 0
    e = d["e2e"]
    assert e["value"] > 0 and e["unit"] == d["unit"] and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert set(d["clocks"]) >= {"sm_mhz", "sm_max_mhz", "reasons"}
    assert d["interactions"]["per_s"] > 0
    cfg = d["configs"]
    assert cfg["forest"]["value"] > 0 and cfg["forest"]["force_error_per_system"]["max_rms"] <= 2e-3
    assert cfg["galaxy"]["value"] > 0 and cfg["galaxy"]["events"] > 0


def test_reference_arm_line():
    d = bench("--impl", "reference", "--n", "16384", "--steps", "1", "--warmup", "1")
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert set(d["per_leaf"]) == {"24", "32"} and d["config"]["leaf_size"] in (24, 32)


@pytest.mark.parametrize("args,keys", [
    (("--workload", "sweep", "--n", "65536", "--steps", "2"), ("rows", "clocks")),
    (("--workload", "galaxy", "--steps", "2"), ("value", "events", "energy_drift", "vs_finest_rung_global_steps")),
    (("--workload", "forest", "--steps", "2", "--warmup", "1"), ("value", "chosen", "force_error_per_system")),
    (("--workload", "adjoint", "--n", "2048", "--steps", "1", "--warmup", "1", "--fd-coords", "2"), ("value", "unit")),
    (("--workload", "scaling", "--sizes", "65536", "--steps", "1", "--warmup", "1"), ("rows",)),
])
def test_workload_lines(args, keys):
    d = bench(*args)
    assert "metric" in d
    for k in keys:
        assert k in d, (args, k)
    if "rows" in d:
        assert d["rows"] and all(r["particle_steps_per_s"] > 0 for r in d["rows"])
