"""The benchmark's reporting contract on CPU: the algorithmic bytes per
particle-update, the recorded force-kernel figures the bench line carries,
and one JSON line of the reference arm (the oracle timed on the host cores)
on the C0 workload."""

from __future__ import annotations

import json
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_bytes_per_update_formula():
    # 3 (3S + 8d + 16) with S = 8(2d + 1) (FP64) or 8d + 4d + 4 (FP32C).
    assert bench.bytes_per_update(2, "fp64") == 456
    assert bench.bytes_per_update(3, "fp64") == 624
    assert bench.bytes_per_update(2, "fp32c") == 348
    assert bench.bytes_per_update(3, "fp32c") == 480


def test_recorded_force_kernel_figures():
    for dim in (2, 3):
        c = bench.forces_ceiling(dim, "fp32c")
        assert c["unit"] == "SM issue slots" and 0.0 < c["pct_busy"] <= 100.0
        assert (ROOT / c["source"]).exists()
        assert bench.forces_traffic(dim, "fp32c", 1000) > 0.0
        assert "recorded" in bench.forces_traffic_source(dim, "fp32c")
    assert bench.forces_ceiling(2, "fp64")["unit"] == "FP64 pipe"
    assert bench.forces_ceiling(3, "fp64") is None


def test_compute_roofline_fields():
    c = bench.forces_compute(2, 1000, 48_000, 0.01, {"sm_mhz": 2070.0})
    assert c["pairs_per_fluid_particle"] == 48.0
    assert c["pair_flops_per_launch"] == 48_000 * bench.FLOPS_PER_PAIR[2]
    peak = 152 * 128 * 2 * 2070e6
    assert abs(c["fp32_frac"] - c["pair_flops_per_launch"] / 1e-5 / peak) < 1e-12


def test_bench_defaults_to_the_3d_dam_break():
    name, _ = bench.make_config("c4")
    assert "3D dam break" in name and "16,000,000 fluid" in name
    assert bench.err_config("c4") == "c4q" and bench.err_config("c1") == "c1"


@pytest.mark.timeout(600)
def test_reference_arm_json_line_on_c0():
    res = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", "c0",
         "--steps", "2", "--warmup", "3"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0.0 and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 3
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    # C0 is timed on the workload itself, with the warm-up steps untimed.
    assert "the workload itself (12800 fluid)" in line["cpu_baseline"]["sample"]
    assert "3 untimed + 2 timed" in line["cpu_baseline"]["sample"]
    assert line["config"]["workload"] == bench.make_config("c0")[0]
    assert line["config"]["fluid_particles"] == 12800
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT,
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
