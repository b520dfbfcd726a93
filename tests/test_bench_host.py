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


def test_tuning_string_maps_to_the_system_calls():
    """--tuning: the first seven fields go to System.set_tuning, the eighth to set_lanes, the ninth to set_lane_split,
    the last two to set_pass_groups; missing trailing fields take their defaults."""
    sys.path.insert(0, ROOT)
    import bench

    class Fake:
        def __init__(self):
            self.calls = []

        def set_tuning(self, *a):
            self.calls.append(("tuning", a))

        def set_lanes(self, k):
            self.calls.append(("lanes", k))

        def set_lane_split(self, k):
            self.calls.append(("split", k))

        def set_pass_groups(self, m, b):
            self.calls.append(("passes", m, b))

    S = Fake()
    bench._apply_tuning(S, "2,8,0,0,1,1,3,32,1562,8,8")
    assert S.calls == [("tuning", (2.0, 8, 0, 0, True, 1, 3)), ("lanes", 32), ("split", 1562), ("passes", 8, 8)]
    S = Fake()
    bench._apply_tuning(S, "4,8,0,0,0")
    assert S.calls == [("tuning", (4.0, 8, 0, 0, False, 1, 0)), ("lanes", 0), ("split", 0), ("passes", 0, 0)]
    # every named workload has a configuration (the sizes the measurements use)
    for name in ("bumpy_screen", "torus_nvt", "ico_nve", "noisy_torus_nvt", "batch64", "mlp_infer"):
        assert bench.workload_config(name)
