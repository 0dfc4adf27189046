"""Host-side checks of bench.py: the reference arm's JSON line (it runs on the
host cores, so it runs here), the roofline arithmetic, and the clock-sample
summary that decides whether a run saw throttling."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "128",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "baseline_cpu" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # without a GPU the reference's own kernels cannot run; the line says why
    assert "reference_gpu" in d


def test_roofline_arithmetic():
    n = 8192
    stats = {"launches": 4, "total_ms": 2.0, "relaxations": 4 * (n - 512) ** 2 * 256.0}
    r = bench.roofline_of(stats, "k", n, 256, 2, 512, 4.0e13, "probe", 6790.0, True, traffic_at_16384=1e9)
    achieved = stats["relaxations"] / 2e-3
    assert r["achieved"] == pytest.approx(achieved) and r["frac"] == pytest.approx(achieved / 4.0e13)
    # tile bytes: each entry read and written once per launch of 256 pivots, 2 bytes per value
    assert r["hbm"]["achieved"] == pytest.approx(stats["relaxations"] * 4 / 256 / 2e-3 / 1e9)
    assert r["bulk_launch"]["algorithmic_bytes"] == 4.0 * (n - 512) ** 2
    assert r["traffic"] == pytest.approx(1e9 * ((n - 512) / (16384 - 512)) ** 2)
    assert bench.roofline_of(None, "k", n, 256, 2, 512, 1.0, "", 1.0, True) is None


def test_clock_summary_flags_throttling():
    s = bench.ClockSampler(0)
    s.lines = [
        "0, 2070, 2070, 400.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2065, 2070, 420.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 1800, 2070, 430.0, 0x8, Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    r = s.summary()
    assert r["samples"] == 3 and r["sm_max_mhz"] == 2070.0 and r["sm_mhz"] == 2065.0 and r["sm_mhz_min"] == 1800.0
    assert r["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert bench.ClockSampler(0).summary()["samples"] == 0


class _FakeRates:
    """Stands in for the library's probe entry points (no GPU here)."""

    def measure_relax_peak(self, stream):
        return 1.9e13, 2.0e13

    def measure_int32_rates(self, stream):
        return {"dpx_addmin": 1.9e13, "imad": 1.9e13, "dpx_min3": 1.9e13, "add": 3.2e13, "min": 1.9e13,
                "dpx_addmin_imad_alternating": 2.8e13, "form_b_relax": 1.75e13, "form_a_relax": 1.91e13,
                "form_b_then_addmin_relax": 2.0e13}


def test_int32_ceiling_model():
    c = bench.int32_ceiling(_FakeRates(), None, None)
    assert c["peak"] == pytest.approx(2.0e13) and c["peak_form"] in ("form_b_then_addmin_relax", "mixed_probe")
    # ALU bound r_alu / ((1 + x) / 2) meets the joint bound r_both / ((3 - x) / 2)
    x = (3 * 1.9 - 2.8) / (1.9 + 2.8)
    assert c["model_addmin_fraction"] == pytest.approx(x, abs=2e-3)
    assert c["model_peak"] == pytest.approx(1.9e13 / ((1 + x) / 2), rel=2e-3)
    assert "per_clock_per_sm" not in c


def test_dijkstra_rows_checker(oracle):
    n = 64
    W = oracle.generate_graph(n, 0.3, 5, 1, 100)
    D = oracle.fw_i32(W)
    rows = {s: D[s].copy() for s in (0, 17, n - 1)}
    r = bench.dijkstra_rows(W, rows, 2)
    assert r["rows_vs_dijkstra"] == "3/3" and r["all_rows_match"] and r["rows"] == [0, 17, n - 1]
    rows[17][3] += 1  # a wrong entry in the result under test is caught
    r = bench.dijkstra_rows(W, rows, 2)
    assert r["rows_vs_dijkstra"] == "2/3" and not r["all_rows_match"]


def test_batched_sample_checker(oracle):
    rng = np.random.default_rng(0)
    sizes = rng.integers(1, 40, 20).astype(np.int32)
    offsets = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)[:-1]])
    packed = np.concatenate([oracle.generate_graph(int(n), 0.5, 100 + g, 1, 9).ravel() for g, n in enumerate(sizes)])
    out = np.concatenate([oracle.fw_i32(packed[o:o + n * n].reshape(n, n)).ravel()
                          for n, o in zip(sizes.tolist(), offsets.tolist())])
    r = bench.batched_sample_check((sizes, offsets, packed, out), 12, 2)
    assert r["batched_graphs_vs_oracle"] == "12/12" and r["batched_all_match"]
    g = int(np.argmax(sizes))  # always sampled (among the 8 largest)
    out[int(offsets[g])] += 1  # a wrong entry in the result under test is caught
    r = bench.batched_sample_check((sizes, offsets, packed, out), 12, 2)
    assert r["batched_graphs_vs_oracle"] == "11/12" and not r["batched_all_match"]
