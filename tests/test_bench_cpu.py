"""bench.py's host-side parts, on the CPU.

The reference arm's JSON line (the oracle port timed on the host cores) at a
small size, the algorithmic-byte formulas the rooflines divide by, and the
clock sampler's window summary and start-up wait.
"""
import json
import os
import subprocess
import sys

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "12",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["warmup"] == 3 and d["steps"] == 1   # at least 3 warm-up steps, whatever is asked
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["cells"] == 12 ** 3 and "workload" in d["config"]
    assert all(i > 0 for i in d["iterations"])


def test_algorithmic_bytes():
    m = {"cells": 10, "stencil_nnz": 100, "boundary_faces": 6, "internal_faces": 27}
    assert bench.stencil_algo_bytes(m) == 10 * (236 + 80) + 4 * 100
    assert bench.stencil_fp64_flops(m) == 2.0 * (15 * 106 + 60 * 10)
    assert bench.pface_algo_bytes(m) == 27 * 136 + 10 * 264
    # CSR SpMV: FP64 12 nnz + 4(N+1) + 16N; FP32 8 nnz + 4(N+1) + 8N
    assert bench.spmv_algo_bytes(100, 700, 8) == 12 * 700 + 4 * 101 + 16 * 100
    assert bench.spmv_algo_bytes(100, 700, 4) == 8 * 700 + 4 * 101 + 8 * 100


def test_pcg_iteration_bytes_two_levels():
    levels = [{"rows": 100, "nnz_A": 700, "nnz_P": 120, "nnz_R": 120, "layout": 2, "value_bytes": 4},
              {"rows": 10, "nnz_A": 60, "nnz_P": 0, "nnz_R": 0, "layout": -1, "value_bytes": 4}]
    n, nc, V = 100, 10, 4
    fine = 4 * (8 * 700 + 4 * 101 + 8 * 100) + 3 * 2 * V * n
    fine += (4 + V) * 120 + 4 * (nc + 1) + V * n + V * nc
    fine += (4 + V) * 120 + 4 * (n + 1) + V * nc + 2 * V * n
    coarse = 8.0 * nc * nc + 2 * V * nc
    outer = (12 * 700 + 4 * 101 + 16 * 100) + 16 * n + 16 * n + 48 * n + V * n
    assert bench.pcg_iteration_bytes(levels) == pytest.approx(fine + coarse + outer, rel=0, abs=0)


def test_clock_summary_window():
    c = bench.ClockSampler(0)
    # rows: time, index, clocks.sm, clocks.max.sm, power, active, hw, hw_thermal, sw_thermal, sw_power_cap
    c.rows = [[0.5, "0", "1500", "2070", "900", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
              [1.1, "0", "2070", "2070", "1100", "0x0", "Not Active", "Not Active", "Not Active", "Active"],
              [1.3, "0", "2060", "2070", "1150", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
              [2.5, "0", "900", "2070", "300", "0x0", "Active", "Not Active", "Not Active", "Not Active"]]
    c.mark(1.0, 2.0)
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2065.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_settle_waits_for_the_rest(monkeypatch):
    now = [100.0]
    slept = []
    monkeypatch.setattr(bench.time, "monotonic", lambda: now[0])
    monkeypatch.setattr(bench.time, "sleep", lambda s: slept.append(s))
    c = bench.ClockSampler(0)
    c.t_start = 99.0          # started 1 s ago
    c.settle(3.0)
    assert slept == [pytest.approx(2.0)]
    slept.clear()
    c.t_start = 90.0          # started long ago: no wait
    c.settle(3.0)
    assert slept == []


def test_workload_config_keys():
    case = bench.bench_case(6)
    cfg = bench.workload_config(6, case.mesh, 1)
    assert cfg["cells"] == 216 and cfg["parallelism"] == "one device"
    assert "workload" in cfg and "faces" in cfg and "nnz" in cfg
