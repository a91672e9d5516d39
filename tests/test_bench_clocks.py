"""The bench's clock record on CPU: the sampler's summary from a fake NVML
(read-only queries: SM clock, power, clock-event reasons) and its fallback
when neither NVML nor nvidia-smi answers."""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402


class FakeNvml:
    """Stands in for bench._Nvml: a fixed clock trace and reason bits."""

    max_mhz = 2070.0

    def __init__(self, trace):
        self.trace = list(trace)
        self.k = 0

    def sample(self):
        clk, watts, names = self.trace[min(self.k, len(self.trace) - 1)]
        self.k += 1
        return clk, watts, names


def _sampled(trace, seconds=0.05):
    c = bench.ClockSampler(0, period=0.002)
    c._nvml = FakeNvml(trace)
    with c:
        time.sleep(seconds)
    return c.summary()


def test_summary_from_nvml_samples():
    s = _sampled([(2070.0, 900.0, []), (2070.0, 950.0, ["sw_power_cap"]), (1980.0, 1000.0, [])])
    assert s["source"].startswith("nvml")
    assert s["samples"] >= 3
    assert s["sm_max_mhz"] == 2070.0
    assert s["sm_min_mhz"] == 1980.0
    assert s["sm_mhz"] in (1980.0, 2070.0)
    assert s["reasons"] == ["sw_power_cap"]


def test_throttle_reasons_are_reported():
    s = _sampled([(1500.0, 1400.0, ["hw_slowdown", "sw_thermal_slowdown"])])
    assert s["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1500.0


def test_reason_bits_of_the_nvml_mask():
    # the clock-event reason bits NVML reports and the names the bench gives them
    assert bench._Nvml.REASONS[0x4] == "sw_power_cap"
    assert bench._Nvml.REASONS[0x8] == "hw_slowdown"
    assert bench._Nvml.REASONS[0x20] == "sw_thermal_slowdown"
    assert bench._Nvml.REASONS[0x40] == "hw_thermal_slowdown"


def test_no_clock_source():
    c = bench.ClockSampler(0)
    c._nvml = None
    c.rows = []
    s = c.summary()
    assert s["samples"] == 0 and s["sm_mhz"] is None
