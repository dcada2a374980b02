"""Cross-checks of the oracle's transcription (CPU).

The reference cannot run here (no Rust toolchain), and its tests pin bag and
query semantics but not the force arithmetic (bird.rs draws from an unseeded
rng).  So the oracle's Bird::step is checked against a second, independent
transcription (tests/py_restatement.py) on small fields, bit for bit, and
against the committed golden trajectories.
"""
import os

import numpy as np
import pytest

import oracle
import py_restatement as pr
from conftest import FLOCK_D, SIDE_1K

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_two_transcriptions_agree():
    rng = np.random.default_rng(1)
    for _ in range(200):
        ctr = rng.integers(0, 2**32, 4, dtype=np.uint64)
        key = rng.integers(0, 2**32, 2, dtype=np.uint64)
        a = oracle.philox(ctr.astype(np.uint32), key.astype(np.uint32))
        b = pr.philox4x32_10(ctr.tolist(), key.tolist())
        assert list(a) == b


def test_jitter_draws_are_uniform():
    # r1, r2 of the jitter stream behave like U[0,1) across ids and steps
    vals = []
    for step in range(4):
        for i in range(2500):
            o = pr.philox4x32_10([i, step, 0, 0], [42, 0])
            vals.append(float(pr.unit(o[0])))
    v = np.array(vals)
    assert 0.49 < v.mean() < 0.51
    hist, _ = np.histogram(v, bins=10, range=(0, 1))
    assert hist.min() > 850 and hist.max() < 1150


def _random_flock(n, side, seed):
    rng = np.random.default_rng(seed)
    xy = (rng.random((n, 2), dtype=np.float32) * np.float32(side)).astype(np.float32)
    ang = rng.random(n) * 2 * np.pi
    dxy = np.stack([np.cos(ang), np.sin(ang)], 1).astype(np.float32)
    return np.arange(n, dtype=np.uint32), xy, dxy


@pytest.mark.parametrize("kind,side,d,radius,n", [
    (0, 40.0, FLOCK_D, 10.0, 80),     # relaxed query, 3x3 stencil
    (1, 40.0, FLOCK_D, 10.0, 80),     # exact query (check_circle)
    (1, 10.0, 0.5, 10.0, 12),      # the reference test geometry (state.rs:11-14)
    (0, 30.0, 2.0, 5.0, 120),      # dd = 2
])
def test_oracle_matches_python_transcription(kind, side, d, radius, n):
    ids, xy, dxy = _random_flock(n, side, seed=n + kind)
    weights, jump, seed = (1.0, 1.3, 0.7, 1.0, 0.9), 0.7, 1234
    py = pr.PyField(side, side, d)
    for i, p, h in zip(ids, xy, dxy):
        b = (int(i), np.float32(p[0]), np.float32(p[1]), np.float32(h[0]), np.float32(h[1]))
        py.set(b, b[1], b[2])
    py.lazy_update()
    orc = oracle.OracleField(side, side, d, True)
    orc.set_many(ids, xy, dxy)
    orc.lazy_update()
    p = oracle.params(*weights, jump=jump, radius=radius, query_mode=kind, seed=seed)
    for step in range(3):
        pr.flock_step(py, kind, radius, weights, jump, seed, step)
        orc.flock_run(p, step, 1)
        o_ids, o_st, _ = orc.iter(1)
        py_all = [b for bag in py.read for b in bag]
        assert [b[0] for b in py_all] == list(o_ids)
        py_st = np.array([[b[1], b[2], b[3], b[4]] for b in py_all], np.float32)
        assert np.array_equal(py_st.view(np.uint32), o_st.view(np.uint32)), f"step {step}"


@pytest.mark.parametrize("wrap", [False, True])
def test_queries_match_python_transcription(wrap):
    ids, xy, dxy = _random_flock(300, 50.0, seed=9)
    for d in (FLOCK_D, 1.7):
        py = pr.PyField(50.0, 50.0, d, wrap=wrap)
        orc = oracle.OracleField(50.0, 50.0, d, True, cell_wrap=1 if wrap else 0)
        for i, p, h in zip(ids, xy, dxy):
            py.set((int(i), p[0], p[1], h[0], h[1]), p[0], p[1])
        orc.set_many(ids, xy, dxy)
        py.lazy_update()
        orc.lazy_update()
        rng = np.random.default_rng(5)
        for _ in range(60):
            q = (rng.random(2) * 52 - 1).astype(np.float32)
            r = float(rng.choice([0.0, 0.3, 3.0, 10.0, 17.5, 30.0]))
            for kind in (0, 1):
                want = [b[0] for b in py.query(kind, q[0], q[1], r)]
                got, _ = orc.query(kind, float(q[0]), float(q[1]), r)
                assert want == list(got)


def test_true_torus_query_sees_across_the_seam():
    # the reference's toroidal query clamps its cell range (field_2d.rs:495-500)
    # and misses a neighbour one unit away across x = 0; the true-torus option
    # finds it
    ids = np.array([1, 2], np.uint32)
    xy = np.array([[0.5, 25.0], [49.5, 25.0]], np.float32)
    dxy = np.zeros((2, 2), np.float32)
    found = {}
    for wrap in (0, 1):
        orc = oracle.OracleField(50.0, 50.0, 2.0, True, cell_wrap=wrap)
        orc.set_many(ids, xy, dxy)
        orc.lazy_update()
        got, _ = orc.query(0, 0.5, 25.0, 3.0)
        found[wrap] = sorted(int(v) for v in got)
    assert found[0] == [1]
    assert found[1] == [1, 2]


def test_golden_trajectories_reproduce():
    """The committed 1,000-boid fixtures (generated by tests/golden/make_golden.py)."""
    g = np.load(os.path.join(GOLDEN, "flock1k_relax_strict.npz"))
    orc = oracle.OracleField(SIDE_1K, SIDE_1K, FLOCK_D, True)
    orc.set_many(g["ids0"], g["xy0"], g["dxy0"])
    orc.lazy_update()
    p = oracle.params(seed=int(g["seed"]), query_mode=0)
    done = 0
    for step in g["checkpoints"]:
        orc.flock_run(p, done, int(step) - done)
        done = int(step)
        ids, st, _ = orc.iter(1)
        assert np.array_equal(ids, g[f"ids_{step}"])
        assert np.array_equal(st.view(np.uint32), g[f"st_{step}"].view(np.uint32))


def test_threaded_timing_run_equals_the_sequential_steps():
    # the all-cores timing run of the oracle (the agent pass on host threads,
    # insertion in agent order) gives the parity run's state bit for bit
    ids, xy, dxy = _random_flock(2000, 300.0, seed=4)
    p = oracle.params(seed=5, query_mode=0)
    _, f = oracle.simulate_timed_threads(300.0, 300.0, FLOCK_D, p, ids, xy, dxy, 6, 4,
                                         keep_field=True)
    o = oracle.OracleField(300.0, 300.0, FLOCK_D, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    o.flock_run(p, 0, 6)
    a_ids, a_st, _ = f.iter(1)
    b_ids, b_st, _ = o.iter(1)
    assert np.array_equal(a_ids, b_ids) and np.array_equal(a_st.view(np.uint32), b_st.view(np.uint32))


def test_warm_up_steps_are_steps_of_the_same_run():
    # the timed runs' warm-up steps are the run's first steps (untimed): a
    # 2 + 4 step run ends where a 6-step run does, in both timing runs
    ids, xy, dxy = _random_flock(1500, 260.0, seed=9)
    p = oracle.params(seed=3, query_mode=0)
    _, a = oracle.simulate_timed(260.0, 260.0, FLOCK_D, p, ids, xy, dxy, 4, keep_field=True,
                                 warmup=2)
    _, b = oracle.simulate_timed(260.0, 260.0, FLOCK_D, p, ids, xy, dxy, 6, keep_field=True)
    _, c = oracle.simulate_timed_threads(260.0, 260.0, FLOCK_D, p, ids, xy, dxy, 4, 3,
                                         keep_field=True, warmup=2)
    _, e = oracle.simulate_timed_threads(260.0, 260.0, FLOCK_D, p, ids, xy, dxy, 6, 3,
                                         keep_field=True)
    for x, y in ((a, b), (c, e)):
        sx, sy = x.iter(1), y.iter(1)
        assert np.array_equal(sx[0], sy[0]) and np.array_equal(sx[1].view(np.uint32), sy[1].view(np.uint32))
