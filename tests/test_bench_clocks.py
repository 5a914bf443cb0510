"""bench.py's clock record: which nvidia-smi samples count for the timed
regions, and the throttle reasons read from them (host logic, no GPU)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

# index, clocks.sm, clocks.max.sm, power.draw, reasons.active, hw_slowdown,
# hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
IDLE = "0, 2070, 2070, 300.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
CAPPED = "0, 1905, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
THERMAL = "0, 1500, 2070, 1400.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"


def sampler(lines, windows):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    s.windows = list(windows)
    return s


def test_only_samples_inside_the_windows_count():
    s = sampler([(0.90, THERMAL), (1.00, IDLE), (1.02, CAPPED), (1.50, IDLE), (2.00, THERMAL)],
                [(0.95, 1.03), (1.45, 1.55)])
    r = s.summary()
    assert r["samples"] == 3
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    # the thermal samples lie outside both regions
    assert r["reasons"] == ["sw_power_cap"]
    assert r["regions_ms"] == [80.0, 100.0]


def test_a_short_window_keeps_the_nearest_sample():
    s = sampler([(1.00, IDLE), (1.20, THERMAL)], [(1.17, 1.18)])
    r = s.summary()
    assert r["samples"] == 1
    assert r["reasons"] == ["hw_thermal_slowdown"]
    assert r["sm_mhz"] == 1500.0


def test_no_windows_uses_every_sample_and_no_samples_reports_none():
    r = sampler([(1.0, IDLE), (2.0, CAPPED)], []).summary()
    assert r["samples"] == 2 and r["reasons"] == ["sw_power_cap"]
    r = sampler([], [(1.0, 2.0)]).summary()
    assert r["samples"] == 0 and r["sm_mhz"] is None


def test_malformed_lines_are_skipped():
    s = sampler([(1.0, "0, [N/A], 2070"), (1.1, "garbage"), (1.2, IDLE)], [(0.9, 1.3)])
    r = s.summary()
    assert r["samples"] == 1 and r["sm_mhz"] == 2070.0


def test_samples_are_placed_by_their_own_timestamp():
    """A line that reaches the reader late still counts where nvidia-smi
    took it; a line without a readable timestamp falls back to its arrival."""
    import datetime
    s = bench.ClockSampler(0)
    t = datetime.datetime(2026, 12, 4, 13, 0, 0, 250000)
    stamp = t.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    s.add(stamp + ", " + THERMAL, arrival=t.timestamp() + 5.0)
    s.add("not a time, " + IDLE, arrival=t.timestamp() + 6.0)
    assert abs(s.lines[0][0] - t.timestamp()) < 1e-3
    assert s.lines[1][0] == t.timestamp() + 6.0
    s.windows = [(t.timestamp() - 0.1, t.timestamp() + 0.1)]
    r = s.summary()
    assert r["samples"] == 1 and r["reasons"] == ["hw_thermal_slowdown"]
