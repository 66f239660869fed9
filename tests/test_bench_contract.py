"""bench.py's output contract on CPU: the reference arm's JSON line (the CPU
restatement, here timed on a small population) carries every key the runner reads, other
ranks print nothing, and the clock sampler's parser flags throttle reasons."""
import argparse
import contextlib
import io
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def _run_reference(monkeypatch, rank):
    monkeypatch.setattr(bench, "CPU_SAMPLE_N", 200)
    monkeypatch.setattr(bench, "REF_N", 300)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.reference_arm(argparse.Namespace(gpus=1, steps=1, warmup=0), rank)
    return buf.getvalue()


def test_reference_arm_line(monkeypatch):
    lines = [l for l in _run_reference(monkeypatch, 0).splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert "N=300" in cb["sample"] and d["config"]["N"] == 300
    sc = d["single_core"]
    assert sc["cores"] == 1 and sc["value"] > 0 and "N=200" in sc["sample"]
    # derived bandwidth on the GPU roofline's basis: seq-gen/s x 16 B x the row width in words
    W = d["config"]["W_live"]
    assert abs(cb["derived_gbs"] - d["value"] * 16.0 * W / 1e9) <= 1e-9 * cb["derived_gbs"]
    assert sc["derived_gbs"] > 0
    e = d["e2e"]
    assert e == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("large_n")


def test_reference_arm_other_ranks_silent(monkeypatch):
    assert _run_reference(monkeypatch, 1) == ""


def test_clock_parser():
    rows = [
        "0, 1965, 2070, 900.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2032, 2070, 950.4, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1990, 2070, 940.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    c = bench.ClockSampler.parse(rows)
    assert c["samples"] == 3 and c["sm_mhz"] == 1990.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == ["sw_power_cap"]
    c = bench.ClockSampler.parse(["0, 1500, 2070, 1, 0x2, Active, Not Active, Active, Not Active"])
    assert c["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert bench.ClockSampler.parse([])["sm_mhz"] is None


def test_measured_peak_reads_file():
    v, kind = bench.measured_peak()
    assert v > 0 and kind in ("measured", "fallback")
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            assert v == float(json.load(f)["hbm_gbs"]) and kind == "measured"
