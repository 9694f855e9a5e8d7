"""Host-side pieces of bench.py that decide whether a run is valid, on
canned input (no GPU): the clock sampler's reading of nvidia-smi's CSV lines
(median SM clock under load, the maximum clock, the throttle reasons seen)."""
from __future__ import annotations

import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402

IDLE = "0, 2070, 2070, 812.40, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"


def sampler(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s.summary()


def test_clean_run_has_no_reasons():
    r = sampler([IDLE, IDLE.replace("2070, 2070", "2055, 2070")])
    assert r["reasons"] == [] and r["samples"] == 2
    assert r["sm_max_mhz"] == 2070.0 and r["sm_mhz"] == (2070.0 + 2055.0) / 2


def test_power_cap_and_thermal_reasons_are_reported():
    cap = "0, 1980, 2070, 1399.00, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    hot = "0, 1500, 2070, 900.00, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    r = sampler([IDLE, cap, hot])
    assert r["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert r["sm_mhz"] == 1980.0 and r["samples"] == 3


def test_malformed_and_unavailable_lines_are_skipped():
    r = sampler(["", "garbage", "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]", IDLE])
    assert r["samples"] == 1 and r["sm_mhz"] == 2070.0


def test_no_samples():
    r = sampler([])
    assert r == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
