"""Host-side pieces of bench.py: the clock-sample summary (throttle reasons) and the
roofline peak lookup."""
import json

import bench


def test_clock_summary_reports_reasons_and_median():
    c = bench.ClockSampler(0)
    c.lines = ["2070, 2070, 900.5, Not Active, Not Active, Not Active, Not Active",
               "2050, 2070, 1100.0, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 1200.0, Not Active, Active, Not Active, Not Active",
               "garbage line"]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_measured_peak_file_or_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peak() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6768.8}))
    assert bench.measured_peak() == (6768.8, "measured")
