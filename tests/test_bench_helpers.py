"""Host-side helpers of bench.py: the roofline traffic figure read from the
committed raster-stage profile, and the parsing of nvidia-smi clock samples
taken during the timed region."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_traffic_line_is_the_sum_of_its_kernels():
    with open(bench.TRAFFIC_FILE) as f:
        line = next(ln for ln in f if ln.startswith("raster stage DRAM bytes per launch:"))
    total = int(line.split(":")[1].split()[0].replace(",", ""))
    parts = [int(x.replace(",", "")) for x in re.findall(r"(?:\(|\+ )\w+ ([\d,]+)", line)]
    assert len(parts) == 5, line
    assert sum(parts) == total
    assert bench.traffic_from_profiles() == total


def _row(uuid, sm, mx, active="0x0", hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return ", ".join([uuid, str(sm), str(mx), "500.0", active, hw, hwt, swt, cap])


def test_clock_samples_median_and_reasons():
    lines = [_row("GPU-a", 2070, 2070), _row("GPU-a", 2055, 2070, cap="Active"),
             _row("GPU-a", 2070, 2070), _row("GPU-b", 1000, 2070, hwt="Active")]
    r = bench.parse_clock_samples(lines, "GPU-a")
    assert r == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    # without a uuid every GPU's lines count
    r = bench.parse_clock_samples(lines)
    assert r["samples"] == 4 and r["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_samples_skip_malformed_lines():
    lines = ["", "garbage", _row("GPU-a", "[N/A]", 2070), _row("GPU-a", 1980, 2070)]
    r = bench.parse_clock_samples(lines, "GPU-a")
    assert r["samples"] == 1 and r["sm_mhz"] == 1980.0
    assert bench.parse_clock_samples(["x, y"], "GPU-a") is None
