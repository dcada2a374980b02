"""The synthetic workloads the benchmark runs (no GPU): the 512-replica
exploration sweep and the Poisson request stream have the sizes, parameter
ranges and offered load of their specification, and are reproducible."""
import numpy as np

import krabmaga_gb300 as kg


def test_sweep_replicas_match_their_specification():
    reps = kg.sweep_replicas(512)
    ns = np.array([r.n for r in reps])
    # N log-uniform in [1024, 65536]: mean (65536 - 1024) / ln 64 = 15,512; about 7.9M in all
    assert ns.min() >= 1024 and ns.max() <= 65536
    assert abs(ns.mean() - 15512) < 0.08 * 15512
    for i, r in enumerate(reps):
        p = r.params
        assert 0.5 <= min(p.cohesion, p.avoidance, p.consistency, p.randomness, p.momentum)
        assert max(p.cohesion, p.avoidance, p.consistency, p.randomness, p.momentum) <= 1.5
        assert 0.3 <= p.jump <= 1.0 and 5.0 <= p.neighbor_radius <= 15.0
        assert np.float32(r.discretization) == np.float32(p.neighbor_radius) / np.float32(1.5)
        assert p.seed == i
        # density 0.025 on a square torus
        assert r.width == r.height and abs(r.n / (r.width * r.height) - 0.025) < 1e-4
    again = kg.sweep_replicas(3)
    assert [(r.n, r.params.jump) for r in again] == [(r.n, r.params.jump) for r in reps[:3]]
    assert all(np.array_equal(a.state[1], b.state[1]) for a, b in zip(again, reps[:3]))


def test_request_stream_matches_its_specification():
    rs = kg.request_stream(200.0, 60.0)
    times = np.array([t for t, _ in rs])
    ns = np.array([r.nboids for _, r in rs], np.float64)
    steps = np.array([r.steps for _, r in rs], np.float64)
    # Poisson 200/s for 60 s: about 12,000 requests, arrivals increasing inside the window
    assert abs(len(rs) - 12000) < 4 * np.sqrt(12000)
    assert np.all(np.diff(times) > 0) and times[0] > 0 and times[-1] < 60.0
    # N log-uniform in [1024, 262144] (mean 47,090); steps uniform in [100, 1000]
    assert ns.min() >= 1024 and ns.max() <= 262144 and abs(ns.mean() - 47090) < 0.05 * 47090
    assert steps.min() >= 100 and steps.max() <= 1000 and abs(steps.mean() - 550) < 10
    # offered load about 5.2e9 boid-updates/s
    assert abs((ns * steps).sum() / 60.0 - 5.2e9) < 0.1 * 5.2e9
    seeds = {r.init_seed for _, r in rs}
    assert len(seeds) == len(rs)
    assert [r.nboids for _, r in kg.request_stream(200.0, 1.0)] == [r.nboids for t, r in rs if t < 1.0]
