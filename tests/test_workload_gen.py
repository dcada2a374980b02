"""The oracle-side workload generator (oracle/workload_gen.cpp) against the
library's own (kb_gen_uniform / kb_gen_clustered): the same seeded flocks bit
for bit, so that the CPU arms of the benchmark build their inputs without
loading the GPU library.  Host code only: no GPU needed."""
import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle


def _same(a, b):
    for x, y in zip(a, b):
        assert x.dtype == y.dtype
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("n,side,seed,scale", [(1000, 200.0, 42, 1.0), (5000, 447.21, 7, 0.7),
                                               (1, 10.0, 0, 1.0), (0, 10.0, 3, 1.0),
                                               (20000, 6476.3447, 2**40 + 5, 1.0)])
def test_uniform_flocks_equal(n, side, seed, scale):
    _same(oracle.gen_uniform(n, side, side, seed, scale), kg.gen_uniform(n, side, side, seed, scale))


@pytest.mark.parametrize("n,side,k,sigma,asig,seed", [(4096, 12952.0, 256, 40.0, 0.3, 11),
                                                      (3000, 300.0, 7, 25.0, 0.5, 99),
                                                      (100, 50.0, 1, 80.0, 0.0, 1)])
def test_clustered_flocks_equal(n, side, k, sigma, asig, seed):
    _same(oracle.gen_clustered(n, side, side, k, sigma, asig, seed),
          kg.gen_clustered(n, side, side, k, sigma, asig, seed))


def test_full_size_prefix_equal():
    # the first quarter-million boids of the 1M workload (same per-id draws)
    n, side = 1 << 18, float(np.float32(np.sqrt((1 << 20) / 0.025)))
    _same(oracle.gen_uniform(n, side, side, 7), kg.gen_uniform(n, side, side, 7))


def test_bad_arguments_raise():
    with pytest.raises(ValueError):
        oracle.gen_uniform(10, 0.0, 1.0, 1)
    with pytest.raises(ValueError):
        oracle.gen_clustered(10, 1.0, 1.0, 0, 1.0, 0.1, 1)
