"""bench.py's host-side arithmetic (no GPU): the workloads' bag matrices and
algorithmic bytes per step, the ncu traffic lookup, and the clock summary
that decides whether a timed run is kept."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)


def test_workload_bag_matrices():
    # 1,000 boids on 200 x 200: 31 x 31 bags; 1M boids: 973 x 973; 4M boids: 1944 x 1944
    assert bench.bag_count(bench.WORKLOADS["flock1k"]["side"]) == 31 * 31
    assert bench.bag_count(bench.WORKLOADS["flock1m"]["side"]) == 946_729
    assert bench.bag_count(bench.WORKLOADS["clustered4m"]["side"]) == 3_779_136
    assert np.float32(bench.WORKLOADS["flock1m"]["side"]) == np.float32(6476.3447)


def test_algorithmic_bytes_per_step():
    # n * 32 + cells * 8: 41,128,264 B at 1M boids, 164,450,816 B at 4M boids
    assert bench.algorithmic_bytes(1 << 20, 946_729)["step"] == 41_128_264
    assert bench.algorithmic_bytes(1 << 22, 3_779_136)["step"] == 164_450_816
    ab = bench.algorithmic_bytes(1000, 961)
    assert ab["force"] == ab["rebin"] == 1000 * 44 + 961 * 8 and ab["scan"] == 961 * 8


def test_ncu_traffic_comes_from_the_committed_summary():
    t = bench.ncu_traffic("k_flock_force")
    assert isinstance(t, int) and t > 0
    assert bench.ncu_traffic("no_such_kernel") is None


def test_clock_summary():
    c = bench.ClockSampler(0)
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2025, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage",
    ]
    s = c.summary()
    assert s["sm_mhz"] == 2025 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.lines = ["0, 1500, 2070, 700.0, 0x40, Not Active, Active, Not Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_thermal_slowdown"]
    c.lines = []
    assert c.summary()["reasons"] == ["unsampled"]
