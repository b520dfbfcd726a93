"""Host-side parts of bench.py that need no GPU: the clock sampler keeps only the samples taken inside the timed
region (plus the one that closes it) and reports throttle reasons."""
import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fake_smi(tmp_path, reasons_after=None):
    script = tmp_path / "nvidia-smi"
    # one CSV line every 50 ms: index, sm clock (counts up from 1900), max clock, power, active, hw, hw_thermal,
    # sw_thermal, sw_power_cap
    power_cap = "Active" if reasons_after is not None else "Not Active"
    script.write_text("#!/bin/bash\ni=0\nwhile true; do\n"
                      f"  echo \"0, $((1900+i)), 2070, 500.0, 0x0, Not Active, Not Active, Not Active, {power_cap}\"\n"
                      "  i=$((i+1)); sleep 0.05\ndone\n")
    script.chmod(script.stat().st_mode | stat.S_IEXEC)
    return str(tmp_path)


def test_clock_sampler_keeps_the_timed_region(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", _fake_smi(tmp_path) + os.pathsep + os.environ["PATH"])
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench.ClockSampler, "PERIOD_MS", 50)
    c = bench.ClockSampler(0)
    c.start()
    time.sleep(0.2)  # samples before the region are dropped
    c.begin()
    time.sleep(0.3)
    c.end()
    out = c.stop()
    assert out is not None
    assert 3 <= out["samples"] <= 10, out
    assert out["sm_mhz"] > 1902, out  # the first samples (taken before begin()) are not counted
    assert out["sm_max_mhz"] == 2070 and out["reasons"] == []
    assert abs(out["region_s"] - 0.3) < 0.1


def test_clock_sampler_reports_power_cap(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, reasons_after=0) + os.pathsep + os.environ["PATH"])
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench.ClockSampler, "PERIOD_MS", 50)
    c = bench.ClockSampler(0)
    c.start()
    c.begin()
    time.sleep(0.2)
    c.end()
    out = c.stop()
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    sys.path.insert(0, ROOT)
    import bench
    c = bench.ClockSampler(0)
    c.start()
    c.begin()
    c.end()
    assert c.stop() is None
