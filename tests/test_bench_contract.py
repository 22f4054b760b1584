"""The bench's JSON contract on the CPU: the reference arm (the oracle port
on the host cores) prints one line with the contract's keys, and the
roofline helper reports the traffic figure with its source."""
import json
import os
import subprocess
import sys

from harness import ROOT


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["warmup"] >= 3 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["unit"] == line["unit"]
    assert "workload" in line["config"]


def test_roofline_reports_traffic_and_source():
    sys.path.insert(0, ROOT)
    import bench
    cells = 32 ** 6
    for key in ("step_fp64", "step_fp64_split", "step_fp32_w2z"):
        prec = "fp32" if "fp32" in key else "fp64"
        rf = bench.roofline(prec, cells, 0.5, key)
        assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and rf["traffic"] > 0
        assert rf["traffic_source"].startswith("profiles/")
        assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-3
    assert [c[0] for c in bench.FP64_CANDIDATES] == ["tma", "split", "fast"]


def test_fp64_roofline_is_bound_by_the_fp64_pipe():
    """the binary64 line reports the binary64-pipe roofline (ops per cell of
    the fast schedule from its source, measured fma rate) with the HBM
    fraction beside it"""
    sys.path.insert(0, ROOT)
    import bench
    n = (32,) * 6
    ops = bench.fp64_ops_per_cell("fast", n)
    # 6 per axis (5 along x: the lanes of a 32-cell row share their
    # differences), face 0 once per 32 cells: v*E(0) on the five clamped
    # axes, a full flux on z with the lower reflection
    assert abs(ops - (1 + 6 * 6 - 1 + (5 * 1 + 4) / 32)) < 1e-12
    assert abs(bench.fp64_ops_per_cell("fast", n, lower_reflection=False) - (1 + 35 + 6 / 32)) < 1e-12
    assert bench.fp64_ops_per_cell("split", n) is None
    assert bench.fp64_ops_per_cell("fast", (8, 1, 1, 1, 1, 8)) == 1 + 2 * (6 + 1 / 8) - 1
    assert abs(bench.fp64_ops_per_cell("fast", (6, 1, 1, 1, 1, 8)) - (1 + 2 * 6 + 1 / 6 + 1 / 8)) < 1e-12
    rf = bench.roofline("fp64", 32 ** 6, 0.1, "step_fp64_split", fp64=(ops, 5e11))
    assert rf["bound"] == "fp64" and rf["unit"] == "G binary64 ops/s"
    assert abs(rf["achieved"] - ops * 32 ** 6 / 0.1 / 1e9) < 0.01
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-3
    assert rf["hbm"]["unit"] == "GB/s" and rf["hbm"]["alg_bytes_per_cell"] == 72
    assert bench.roofline("fp64", 32 ** 6, 0.1, "step_fp64_split", fp64=(None, 5e11))["bound"] == "hbm"
