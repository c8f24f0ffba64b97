"""The bench's clock record: nvidia-smi samples are kept by their own timestamps, inside the timed region."""
import datetime
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

LINES = """2026/12/04 17:30:00.100, 0, 1980, 2070, 500.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active
2026/12/04 17:30:00.150, 0, 2070, 2070, 900.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active
2026/12/04 17:30:00.200, 0, 2050, 2070, 910.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active
2026/12/04 17:30:00.250, 0, 1400, 2070, 300.0, 0x0000000000000000, Not Active, Active, Not Active, Not Active
garbage line
"""


def _sampler(t0_ms, t1_ms):
    c = bench.ClockSampler(0)
    c.proc, c.out, c.stopped = object(), LINES, True
    c.t0 = datetime.datetime(2026, 12, 4, 17, 30, 0, t0_ms * 1000)
    c.t1 = datetime.datetime(2026, 12, 4, 17, 30, 0, t1_ms * 1000)
    return c


def test_only_samples_inside_the_timed_region_count():
    s = _sampler(120, 210).summary()
    assert s["samples"] == 2 and s["window"] == "timed region"
    assert s["sm_mhz"] == 2060.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]          # the thermal-slowdown sample lies after the region


def test_short_region_reports_the_bracketing_samples():
    s = _sampler(160, 170).summary()
    assert s["samples"] == 2 and s["window"].startswith("bracketing")
    assert s["sm_mhz"] == 2060.0


def test_throttle_reason_inside_the_region_is_reported():
    s = _sampler(120, 260).summary()
    assert "hw_thermal_slowdown" in s["reasons"] and s["samples"] == 3


def test_no_sampler_gives_no_record():
    c = bench.ClockSampler(0)
    assert c.summary() is None
