"""Host-side pieces of bench.py that need no GPU: the clock record's
summary (NVML reason bits and nvidia-smi lines), and the timed arm's error
measure."""
import json

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


def _fake_arm(order, err, ms):
    return {"t_total": ms * 20 / 1e3, "depth": 11, "order": order, "theta": 0.75, "mac": "bmax", "tau": None,
            "err": (err, 3 * err, 50 * err), "graph": True, "launches": 2460,
            "stages": {"sort": 0.25, "build": 0.55, "lists": 0.45, "far": 0.7, "near": 1.3, "l2p": 0.1,
                       "reduce": 0.03},
            "counters": {"p2p_pairs": 2_359_484_542, "m2p": 0, "p2l": 0, "m2l": 14_200_000},
            "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 17, "source": "nvml"},
            "nonempty_nodes": 600_000, "near_pairs": 9_000_000}


def test_headline_line_stays_small_with_every_trial_recorded():
    """The printed line carries the chosen configurations only: hundreds of
    autotuning trials must not grow it past a few KB."""
    import argparse
    trials = [{"mac": "bmax", "depth": 11, "theta": 0.5 + 0.01 * i, "order": 8, "ms": 3.0, "err": 9e-5}
              for i in range(400)]
    calib = {"plain_best": trials[0], "plain_p12": dict(trials[1], order=12), "learned_best": {"depth": 12, "tau": 5e-4},
             "plain_trials": trials, "learned_trials": trials,
             "controller": {"samples": 8_900_000, "systems": 8, "system_n": 1 << 20, "steps": 6000,
                            "orders": [4, 6, 8, 10, 12], "loss_curve": list(range(6000))},
             "reference_order": {"theta": 0.15, "median_err": 9e-5, "ms_per_step": 370.0,
                                 "particles_per_s": 1.1e7, "depth": 10}}
    r = {"head": "plain_best", "calib": calib, "e2e_ms": [5.0, 5.1],
         "arms": {"plain_best": _fake_arm(8, 7.8e-5, 3.1), "plain_p12": _fake_arm(12, 8e-5, 4.0),
                  "learned": dict(_fake_arm(12, 7e-5, 6.1), tau=5e-4)}}
    args = argparse.Namespace(steps=20, warmup=5, leaf_p2p=64)
    w = bench.WORKLOADS["nbody_two_disks_4m"]
    line = bench.headline_line(args, w, r, 1, {"workload": "nbody_two_disks_4m"}, {"hbm_gbs": 6752.1,
                               "sm_max_mhz": 2070.0}, "measured", 152)
    text = json.dumps(line)
    assert len(text) < 6000, len(text)
    assert json.loads(text)["value"] == pytest.approx(4194304 * 20 / (3.1 * 20 / 1e3))
    for k in ("roofline", "e2e", "clocks", "gpu_launches", "step_roofline"):
        assert k in line
    sr = line["step_roofline"]
    assert 0 < sr["achieved"] < 1 and sr["t_stages_ms"] == pytest.approx(3.38)
    # overlapping stages: the step roofline is taken against the measured step, not the stage sum
    assert sr["t_step_ms"] == pytest.approx(3.1) and sr["achieved"] == pytest.approx(sr["t_roof_ms"] / 3.1, rel=1e-3)
    assert "learned_speedup_vs_plain_p12" in line["comparison"]


def test_tuning_and_evaluation_rows_are_disjoint():
    a, b = bench.sample_rows(4194304)
    assert len(a) == len(b) == bench.N_SAMPLES
    assert not set(a.tolist()) & set(b.tolist())
    assert np.all(np.diff(a) > 0) and np.all(np.diff(b) > 0)


def test_m2l_flop_count_matches_the_kernel_formula():
    # order 8: 10 K(8) + 2 sum_k (k+1) K(8-k) = 450 + 990
    assert bench.m2l_flops(8) == 1440
