"""CPU tests of the bench's own bookkeeping: the clock record that decides
whether a run is kept (throttle reasons, median clock), the algorithmic byte
counts, and the reference arm's JSON line on a small sample."""
import json
import os
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def clocks_from(lines):
    c = bench.Clocks(0)
    c.lines = lines
    return c.summary()


def test_clock_summary_median_max_and_no_reason():
    lines = ["2070, 2070, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "2055, 2070, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "2070, 2070, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"]
    s = clocks_from(lines)
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3}


def test_clock_summary_reports_throttle_reasons():
    lines = ["1800, 2070, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "1500, 2070, 0x0000000000000048, Not Active, Active, Not Active, Not Active",
             "garbage line",
             "[N/A], 2070, 0x0, Not Active, Not Active, Not Active, Not Active"]
    s = clocks_from(lines)
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert s["samples"] == 2 and s["sm_mhz"] == 1650.0


def test_clock_summary_without_samples():
    assert clocks_from([]) == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_algorithmic_bytes():
    # scan reads and writes 8 B per Int64 element, fold reads 4 B per Float32,
    # permute reads 4 B per index and reads + writes the 2^16 Int32 bins,
    # stencil reads and writes 4 B per Float32 cell
    assert bench.BYTES == {"scan": 16 << 28, "fold": 4 << 28, "permute": (4 << 28) + 8 * (1 << 16),
                           "stencil": 8 * 8192 * 8192}
    assert bench.cpu_bytes(1, 8192) == bench.BYTES
    assert bench.cpu_bytes(4, 4096)["stencil"] == bench.BYTES["stencil"] // 4
    assert bench.whole_job_gbs(1, 10 ** 9, 1.0) == pytest.approx(1000.0)


def test_reference_arm_json_line():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--cpu-scale", "256"], env=env, capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert set(line["per_skeleton_gbs"]) == {"scan", "fold", "permute", "stencil"}
