"""Host-side pieces of bench.py that need no GPU: the clock record's
summary (NVML reason bits and nvidia-smi lines), and the timed arm's error
measure."""
import numpy as np
import pytest

import bench


def test_clock_summary_decodes_nvml_reason_bits():
    c = bench.ClockSampler(0)
    # nvmlClocksEventReason bits: 0x1 idle (ignored), 0x4 sw power cap, 0x8 hw slowdown, 0x20 sw thermal,
    # 0x40 hw thermal
    c.samples = [(2070.0, 2070.0, 0x1), (1980.0, 2070.0, 0x4), (2070.0, 2070.0, 0x0)]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3, "source": "nvml"}
    c.samples.append((1500.0, 2070.0, 0x8 | 0x20 | 0x40))
    assert c.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]


def test_clock_summary_reads_nvidia_smi_lines():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "0, 2055, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "garbage"]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    assert s["source"] == "nvidia-smi"


def test_median_error_is_relative_per_particle():
    ref = np.array([[1.0, 0.0], [0.0, 2.0], [3.0, 4.0]])
    got = ref + np.array([[1e-3, 0.0], [0.0, 2e-2], [0.0, 0.0]])
    med, p90, mx = bench.median_error(got, ref)
    assert med == pytest.approx(1e-3, rel=1e-12) and mx == pytest.approx(1e-2, rel=1e-12)
