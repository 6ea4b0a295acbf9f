"""bench.py's JSON line on a small plate: the keys and shapes the measurement
contract asks for (the headline metric, the roofline and CPU baseline objects,
the end-to-end leg with its transfer sizes, the clock record, the launch
count), and the serve-only mode on a few requests."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _run(args, timeout=600):
    r = subprocess.run([sys.executable, "bench.py"] + args, cwd=ROOT, capture_output=True, text=True,
                       timeout=timeout)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_bench_line_keys_on_a_small_plate():
    d = _run(["--side", "200", "--steps", "4", "--warmup", "3", "--no-batch", "--no-serve", "--no-accuracy",
              "--scale-side", "0", "--cpu-steps", "1", "--e2e-steps", "3"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "gpu_launches", "clocks", "roofline", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["unit"] == "bond-updates/s" and d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3 and d["value"] > 0
    assert d["gpu_launches"] == 1 + 2 * 4
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and 0 < r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    c = d["cpu_baseline"]
    assert c["value"] > 0 and c["cores"] >= 1 and c["kind"] in ("port", "reference") and c["sample"]
    for e in (d["e2e"], d["mixed"]["e2e"]):
        n = d["config"]["particles"]
        assert e["value"] > 0 and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 48 * n
        assert 0 < e["link"]["bound_ms_per_step"] < e["ms_per_step"]
    dr = d["e2e"]["dropin_api"]
    assert dr["value"] > 0 and dr["h2d_bytes_per_step"] == dr["d2h_bytes_per_step"] == 48 * d["config"]["particles"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert d["bond_assoc"]["device"]["ms_per_step"] > 0 and d["bond_assoc"]["particles"] == 4064


def test_bench_serve_only_reports_sample_counts():
    d = _run(["--serve-only", "--batch-plates", "8", "--batch-steps", "5", "--serve-requests", "6",
              "--serve-fp64-requests", "3"])
    for name, count in (("mixed", 6), ("fp64", 3)):
        m = d["serve"][name]
        assert m["requests"] == m["latency_samples"] == count
        assert 0 < m["p50_latency_s"] <= m["p95_latency_s"] <= m["p99_latency_s"] <= m["max_latency_s"]
        assert m["offered_load_achieved"] is None or m["offered_load_achieved"] > 0
