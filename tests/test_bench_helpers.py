"""Host-side helpers behind the bench line, on fixed inputs (no GPU): the clock record's summary
and the time-to-error reading of an error curve."""
import math
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _clocks_from(tmp_path, lines):
    c = bench.Clocks(0)
    c.path = str(tmp_path / "clocks.csv")
    Path(c.path).write_text("\n".join(lines) + "\n")
    return c.summary()


def test_clock_summary_takes_the_median_and_every_active_reason(tmp_path):
    row = "0, {sm}, 2070, 900.5, 0x{a:x}, {hw}, {hwt}, {swt}, {cap}"
    lines = [row.format(sm=s, a=0, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active")
             for s in (2070, 2055, 2070, 1995, 2070)]
    lines.append(row.format(sm=1980, a=4, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Active"))
    lines.append("garbage line")
    s = _clocks_from(tmp_path, lines)
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 6  # the upper median
    assert s["reasons"] == ["sw_power_cap"]
    lines.append(row.format(sm=1500, a=8, hw="Active", hwt="Not Active", swt="Active", cap="Not Active"))
    assert _clocks_from(tmp_path, lines)["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]


def test_clock_summary_without_samples_says_so(tmp_path):
    s = _clocks_from(tmp_path, ["nvidia-smi not found"])
    assert s["sm_mhz"] is None and s["reasons"] == ["unavailable"]


def test_time_to_level_is_the_last_crossing_interpolated_in_log_error():
    curve = [(1, 0.1, 10.0), (2, 0.2, 1.0), (4, 0.4, 2.0), (8, 0.8, 0.1)]
    assert bench._time_to(curve, 20.0) == 0.1  # below the level from the start
    # 1.0 is crossed for good between 0.4 s (error 2) and 0.8 s (error 0.1), not at 0.2 s
    want = 0.4 + 0.4 * (math.log(2.0) - math.log(1.0)) / (math.log(2.0) - math.log(0.1))
    assert bench._time_to(curve, 1.0) == pytest.approx(want)
    assert bench._time_to(curve, 0.05) is None  # the curve ends above the level
