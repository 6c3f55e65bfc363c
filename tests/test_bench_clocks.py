"""bench.py's clock record (CPU, no GPU and no driver library): the NVML
sampler keeps only the samples taken inside the timed steps, reports their
median SM clock, and decodes the clock-event reason bits; without NVML and
without nvidia-smi the record says so instead of inventing a clock."""
import threading

import bench


class _FakeLib:
    def nvmlShutdown(self):
        return 0


def _sampler(samples, max_mhz=2070.0):
    s = bench.NvmlClocks.__new__(bench.NvmlClocks)   # no driver library here
    s.lib = _FakeLib()
    s.samples = list(samples)
    s.max_mhz = max_mhz
    s.stop_flag = False
    s.t = threading.Thread(target=lambda: None)
    s.t.start()
    return s


def test_samples_inside_the_timed_steps_only():
    # (time, SM MHz, reason bits); the timed steps run from t = 1.0 to 2.0
    samples = [(0.5, 1000.0, 0x8), (1.1, 2070.0, 0x0), (1.5, 2060.0, 0x4),
               (1.9, 2070.0, 0x0), (2.5, 900.0, 0x40)]
    r = _sampler(samples).stop(1.0, 2.0)
    assert r["samples"] == 3
    assert r["sm_mhz"] == 2070.0
    assert r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]      # the slowdowns lay outside
    assert r["source"] == "nvml"


def test_reason_bits():
    samples = [(1.2, 1500.0, 0x8 | 0x20), (1.4, 1400.0, 0x40)]
    r = _sampler(samples).stop(1.0, 2.0)
    assert r["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_timed_steps_shorter_than_a_sample_period():
    r = _sampler([(0.9, 2070.0, 0), (1.3, 2065.0, 0)]).stop(1.0, 1.01)
    assert r["samples"] == 1 and r["window"].startswith("adjacent")


def test_no_clock_source(monkeypatch):
    def no_process(*a, **k):
        raise FileNotFoundError("nvidia-smi")
    monkeypatch.setattr(bench.subprocess, "Popen", no_process)
    c = bench.ClockSampler(0)          # no CUDA device given: NVML is not tried
    c.start()
    c.mark_begin()
    c.mark_end()
    r = c.stop()
    assert r["sm_mhz"] is None and r["reasons"] == ["nvidia-smi unavailable"]
