"""The reference's own Field2D tests, run against the oracle.

Ports tests/engine/field_2d.rs:31-246 (sequential build) and the
tests/explore/simulate.rs:18-38 smoke test.  The Flocker state of the
reference tests is a 10x10 torus with discretization 0.5
(tests/model/flockers/state.rs:11-14), the in-tree Bird query radius is 10
(bird.rs:41) with get_neighbors_within_distance.
"""
import numpy as np

import oracle

W = H = 10.0
D = 0.5
RELAX, EXACT, GET, GET_UNBUF = 0, 1, 2, 3


def flocker_field():
    return oracle.OracleField(W, H, D, True)


def test_field_2d_single_step():
    # field_2d.rs:31-50: 10 random birds, one schedule.step, both queries at
    # (5,5) with r=10 see all 10.
    rng = np.random.default_rng(3)
    f = flocker_field()
    n = 10
    xy = (rng.random((n, 2), dtype=np.float32) * np.float32(W)).astype(np.float32)
    f.set_many(np.arange(n), xy, np.zeros((n, 2), np.float32))
    f.lazy_update()  # schedule.rs:349-351 (step 0 update)
    f.flock_run(oracle.params(query_mode=EXACT, seed=1), 0, 1)
    assert f.nagents == n
    ids, _ = f.query(EXACT, 5.0, 5.0, 10.0)
    assert len(ids) == n
    ids, _ = f.query(RELAX, 5.0, 5.0, 10.0)
    assert len(ids) == n


def test_field_2d_neighbors():
    # field_2d.rs:58-117
    for fly in range(5, 10):
        f = flocker_field()
        f.set(1, 0.0, 0.0)
        f.set(2, 0.0, 0.0)
        f.lazy_update()
        assert f.nagents == 2
        assert len(f.query(EXACT, 5.0, 5.0, 1.0)[0]) == 0
        assert len(f.query(RELAX, 5.0, 5.0, 1.0)[0]) == 0
        b1 = (float(fly), float(fly))
        f.set(1, *b1)
        f.set(2, 0.0, 0.0)
        f.lazy_update()
        ids, _ = f.query(EXACT, *b1, 1.0)
        assert list(ids) == [1]
        ids, _ = f.query(EXACT, 0.0, 0.0, 1.0)
        assert list(ids) == [2]
        ids, _ = f.query(EXACT, 5.0, 5.0, 10.0)
        assert sorted(ids) == [1, 2]
        ids, _ = f.query(RELAX, 5.0, 5.0, 10.0)
        assert sorted(ids) == [1, 2]


def test_field_2d_gets():
    # field_2d.rs:125-178
    f = flocker_field()
    f.set(1, 0.0, 0.0)
    f.set(2, 5.0, 5.0)
    f.set(3, 5.0, 5.0)
    f.lazy_update()
    assert f.nagents == 3
    ids, _ = f.query(GET, 5.0, 5.0)
    assert sorted(ids) == [2, 3]
    assert len(f.query(GET, 10.0, 0.0)[0]) == 0
    assert f.num_at(5.0, 5.0) == 2
    assert f.num_at(0.0, 0.0) == 1
    f.set(4, 0.0, 0.0)
    assert len(f.query(GET_UNBUF, 0.0, 0.0)[0]) == 1
    assert len(f.query(GET, 0.0, 0.0)[0]) == 1
    f.remove(4, 0.0, 0.0)
    assert len(f.query(GET_UNBUF, 0.0, 0.0)[0]) == 0


def test_field_2d_bags():
    # field_2d.rs:186-210
    f = flocker_field()
    assert len(f.empty_bags()) == f.dh * f.dw == 441
    f.set(1, 0.0, 0.0)
    f.set(2, 0.0, 0.0)
    f.set(3, 4.0, 4.0)
    f.lazy_update()
    bags = f.empty_bags()
    assert len(bags) == f.dh * f.dw - 2
    assert not any((b[0] == 0.0 and b[1] == 0.0) or (b[0] == 4.0 and b[1] == 4.0) for b in bags)


def test_field_2d_iter():
    # field_2d.rs:218-246
    f = flocker_field()
    f.set(1, 0.0, 0.0)
    f.set(2, 0.01, 0.01)
    f.set(3, 5.0, 5.0)
    ids, st, cells = f.iter(0)
    assert sorted(ids) == [1, 2, 3]
    for i, c in zip(ids, cells):
        x, y = float(np.float32(c // f.dh) * np.float32(D)), float(np.float32(c % f.dh) * np.float32(D))
        assert i in f.query(GET_UNBUF, x, y)[0]
    f.lazy_update()
    assert len(f.query(GET, 0.0, 0.0)[0]) == 2
    ids, st, cells = f.iter(1)
    for i, c in zip(ids, cells):
        x, y = float(np.float32(c // f.dh) * np.float32(D)), float(np.float32(c % f.dh) * np.float32(D))
        assert i in f.query(GET, x, y)[0]


def test_simulate_old_smoke():
    # tests/explore/simulate.rs:18-38: Flocker::new((200,200), 100), 10 steps
    # through the priority-queue schedule; positive time and steps/s.
    n = 100
    rng = np.random.default_rng(0)
    xy = (rng.random((n, 2), dtype=np.float32) * np.float32(200.0)).astype(np.float32)
    secs, f = oracle.simulate_timed(200.0, 200.0, D, oracle.params(query_mode=EXACT), np.arange(n),
                                    xy, np.zeros((n, 2), np.float32), 10, keep_field=True)
    assert secs > 0 and 10 / secs > 0
    assert len(f.iter(1)[0]) == n


def test_out_of_matrix_location_is_a_panic():
    # field_2d.rs:838-846 indexes bags[(x*dh)+y] unchecked: a negative or
    # too-large index panics in the reference; the oracle reports it.
    f = flocker_field()
    assert f.set(1, -3.0, 0.0) == -1
    assert f.set(2, 10.0, 10.0) == 0   # the x=w, y=h bag exists (dw = max_x+1)
    assert f.set(3, 10.6, 10.6) == -1  # beyond the last bag
