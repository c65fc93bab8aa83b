"""bench.py's clock record: only samples inside the timed region count, throttle reasons are collected."""

from __future__ import annotations

import datetime
import sys
import time
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import bench  # noqa: E402


def _ts(t):
    return datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]


def test_clock_samples_are_windowed():
    now = time.time()
    lines = [f"{_ts(now - 1)}, 0, 1500, 2070, 300, 0x0, Not Active, Not Active, Not Active, Not Active",
             f"{_ts(now + 0.05)}, 0, 2070, 2070, 900, 0x0, Not Active, Not Active, Not Active, Active",
             f"{_ts(now + 0.10)}, 0, 2070, 2070, 950, 0x0, Not Active, Not Active, Not Active, Not Active",
             f"{_ts(now + 5)}, 0, 1000, 2070, 200, 0x0, Not Active, Active, Not Active, Not Active",
             "garbage line"]
    inside = bench.ClockSampler.parse(lines, now, now + 1)
    assert inside == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 2, "samples_in_timed_region": 2,
                      "reasons": ["sw_power_cap"]}
    every = bench.ClockSampler.parse(lines)  # no window: every sample, every reason
    assert every["samples"] == 4 and every["samples_in_timed_region"] == 0
    assert every["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert bench.ClockSampler.parse([]) ["sm_mhz"] is None
