"""bench.py's host-side pieces on CPU: the algorithmic work per lit
subaperture-frame behind ``roofline.achieved`` (the figures the design
quotes for the 74x74 workload), and the parsing of the nvidia-smi clock
samples that decides whether a run saw throttling."""
import math

import bench


def test_algorithmic_work_of_the_74x74_workload():
    F, B = bench.algorithmic_per_subap()
    p, N, C, m = 10, 20, 20, 10
    want = 6 * p * p + 10 * N * N * math.log2(N) + 3 * C * C + 10 * C * C * math.log2(C) + 6 * C * (C // 2 + 1) \
        + C * C + 3 * m * m
    assert F == want and round(F) == 38395
    assert B == 808.0  # 4 p^2 phase in + 4 m^2 image out + 8 centroid bytes
    # tensor work of one GEMM-DFT pass: 2 (2c^2)(2p^2) + 2 m^2 c^2
    assert bench.tensor_flops_per_subap() == 400000.0


def _sampler(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s.summary()


def test_clock_samples_median_and_throttle_reasons():
    ok = "0, 2070, 2070, 812.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
    cap = "0, 1980, 2070, 1390.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    hot = "0, 1500, 2070, 1100.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    s = _sampler([ok, ok, cap])
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    s = _sampler([ok, hot, hot, "garbage", "0, [N/A], 2070, 1, 0, x, x, x, x"])
    assert s["sm_mhz"] == 1500.0 and s["reasons"] == ["hw_thermal_slowdown"] and s["samples"] == 3
    assert _sampler([]) == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
