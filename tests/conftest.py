"""Shared test setup: marker registration and in-place builds.

Tests marked ``gpu`` need a CUDA device and call the product through the C ABI
(libkrabgpu.so).  Everything else runs on CPU: the oracle against the
reference's own pins, the host-side logic, and the C ABI's loading/exports.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LIB = os.path.join(ROOT, "krabmaga_gb300", "libkrabgpu.so")
ORACLE = os.path.join(ROOT, "oracle", "build", "libkrab_oracle.so")
if not (os.path.exists(LIB) and os.path.exists(ORACLE)):
    import __graft_entry__

    __graft_entry__.build()

# The 1,000-boid flock: a 200x200 torus, bags of d = 10/1.5 in f32, radius 10.
SIDE_1K = 200.0
FLOCK_D = float(np.float32(10.0) / np.float32(1.5))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the kernels)")


@pytest.fixture(scope="session")
def gpu():
    import krabmaga_gb300 as kg

    n = kg.device_count()
    assert n > 0, "GPU test run without a visible CUDA device"
    return 0
