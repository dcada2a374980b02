"""Field2D through the C ABI on the GPU.

The reference's own tests (tests/engine/field_2d.rs:31-246) against the GPU
field, and the field's queries against the oracle on random fields: the
returned lists must equal the oracle's bit for bit, in the same visiting order.
"""
import ctypes as C

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D
from krabmaga_gb300 import Bird, Real2D
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu

W = H = 10.0
D = 0.5


def flocker(n=0):
    return kg.Flocker((W, H), n, discretization=D,
                      params=kg.FlockParams(query_mode=kg.KB_QUERY_EXACT, seed=5))


def test_field_2d_single_step(gpu):
    # field_2d.rs:31-50
    state = flocker(10)
    schedule = kg.Schedule()
    state.init(schedule)
    schedule.step_state(state)
    assert state.field1.nagents == 10
    assert len(state.field1.get_neighbors_within_distance(Real2D(5.0, 5.0), 10.0)) == 10
    assert len(state.field1.get_neighbors_within_relax_distance(Real2D(5.0, 5.0), 10.0)) == 10


@pytest.mark.parametrize("fly", [5, 7, 9])
def test_field_2d_neighbors(gpu, fly):
    # field_2d.rs:58-117
    state = flocker(2)
    f = state.field1
    b1 = Bird(1, Real2D(0.0, 0.0))
    b2 = Bird(2, Real2D(0.0, 0.0))
    f.set_object_location(b1, b1.pos)
    f.set_object_location(b2, b2.pos)
    state.update(0)
    assert f.nagents == 2
    assert len(f.get_neighbors_within_distance(Real2D(5.0, 5.0), 1.0)) == 0
    assert len(f.get_neighbors_within_relax_distance(Real2D(5.0, 5.0), 1.0)) == 0
    b1 = Bird(1, Real2D(float(fly), float(fly)))
    f.set_object_location(b1, b1.pos)
    f.set_object_location(b2, b2.pos)
    state.update(0)
    v = f.get_neighbors_within_distance(b1.pos, 1.0)
    assert len(v) == 1 and b1 in v
    v = f.get_neighbors_within_distance(b2.pos, 1.0)
    assert len(v) == 1 and b2 in v
    v = f.get_neighbors_within_distance(Real2D(5.0, 5.0), 10.0)
    assert len(v) == 2 and b1 in v and b2 in v
    v = f.get_neighbors_within_relax_distance(Real2D(5.0, 5.0), 10.0)
    assert len(v) == 2 and b1 in v and b2 in v


def test_field_2d_gets(gpu):
    # field_2d.rs:125-178
    state = flocker(2)
    f = state.field1
    b1, b2, b3 = Bird(1, Real2D(0.0, 0.0)), Bird(2, Real2D(5.0, 5.0)), Bird(3, Real2D(5.0, 5.0))
    for b in (b1, b2, b3):
        f.set_object_location(b, b.pos)
    state.update(0)
    assert f.nagents == 3
    birds = f.get_objects(Real2D(5.0, 5.0))
    assert len(birds) == 2 and b2 in birds and b3 in birds
    assert len(f.get_objects(Real2D(10.0, 0.0))) == 0
    assert f.num_objects_at_location(Real2D(5.0, 5.0)) == 2
    assert f.num_objects_at_location(Real2D(0.0, 0.0)) == 1
    b4 = Bird(4, Real2D(0.0, 0.0))
    f.set_object_location(b4, b4.pos)
    assert len(f.get_objects_unbuffered(Real2D(0.0, 0.0))) == 1
    assert len(f.get_objects(Real2D(0.0, 0.0))) == 1
    f.remove_object_location(b4, b4.pos)
    assert len(f.get_objects_unbuffered(Real2D(0.0, 0.0))) == 0


def test_field_2d_bags(gpu):
    # field_2d.rs:186-210
    state = flocker(0)
    f = state.field1
    assert len(f.get_empty_bags()) == f.dh * f.dw == 441
    for b in (Bird(1, Real2D(0.0, 0.0)), Bird(2, Real2D(0.0, 0.0)), Bird(3, Real2D(4.0, 4.0))):
        f.set_object_location(b, b.pos)
    state.update(0)
    assert len(f.get_empty_bags()) == f.dh * f.dw - 2
    rb = f.get_random_empty_bag(seed=3)
    assert rb is not None
    assert (rb.x != 0.0 or rb.y != 0.0) and (rb.x != 4.0 or rb.y != 4.0)


def test_field_2d_iter(gpu):
    # field_2d.rs:218-246
    state = flocker(0)
    f = state.field1
    for b in (Bird(1, Real2D(0.0, 0.0)), Bird(2, Real2D(0.01, 0.01)), Bird(3, Real2D(5.0, 5.0))):
        f.set_object_location(b, b.pos)
    seen = []
    f.iter_objects_unbuffered(lambda loc, obj: seen.append(obj in f.get_objects_unbuffered(loc)))
    assert seen == [True, True, True]
    state.update(0)
    assert len(f.get_objects(Real2D(0.0, 0.0))) == 2
    seen = []
    f.iter_objects(lambda loc, obj: seen.append(obj in f.get_objects(loc)))
    assert seen == [True, True, True]


def test_out_of_matrix_location_is_an_error(gpu):
    f = kg.Field2D(W, H, D, True)
    with pytest.raises(kg.KbError) as e:
        f.set_object_location(Bird(1, Real2D(-3.0, 0.0)), Real2D(-3.0, 0.0))
    assert e.value.status == kg._lib.KB_ERR_RANGE
    f.set_object_location(Bird(2, Real2D(10.0, 10.0)), Real2D(10.0, 10.0))  # the x=w bag exists


def _random_fields():
    rng = np.random.default_rng(11)
    for side, d, n, tor in [(50.0, FLOCK_D, 400, True), (50.0, 1.7, 900, True),
                            (30.0, 2.0, 300, False), (10.0, 0.5, 60, True)]:
        ids = rng.permutation(n).astype(np.uint32)
        xy = (rng.random((n, 2), dtype=np.float32) * np.float32(side)).astype(np.float32)
        xy[:5] = 0.0           # seam corner
        xy[5:8] = np.float32(side)  # the x = w / y = h bag
        dxy = rng.standard_normal((n, 2)).astype(np.float32)
        yield side, d, tor, ids, xy, dxy


@pytest.mark.parametrize("case", range(4))
def test_queries_match_oracle(gpu, case):
    side, d, tor, ids, xy, dxy = list(_random_fields())[case]
    g = kg.Field2D(side, side, d, tor)
    g.set_locations(ids, xy, dxy)
    g.lazy_update()
    o = oracle.OracleField(side, side, d, tor)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    # stored order == the oracle's iteration order (insertion order in bags)
    gi, gs = g.get_state()
    oi, os_, _ = o.iter(1)
    assert np.array_equal(gi, oi) and np.array_equal(gs, os_)
    rng = np.random.default_rng(case)
    q = (rng.random((500, 2)) * (side + 2) - 1).astype(np.float32)
    q[:50] = xy[:50]
    for r in (0.0, 0.4, 3.0, 10.0, 0.75 * side):
        for kind in (kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT):
            gc, gl = g.neighbor_lists(kind, r, q)
            oc, ol = o.neighbor_lists(kind, r, q)
            assert np.array_equal(gc, oc), (r, kind)
            assert np.array_equal(gl, ol), (r, kind)
            gc2, gd = g.neighbor_digest(kind, r, q)
            oc2, od = o.neighbor_digest(kind, r, q)
            assert np.array_equal(gc2, oc2) and np.array_equal(gd, od)
    # single-point API, both kinds, with the states
    for k in range(20):
        loc = Real2D(float(q[k, 0]), float(q[k, 1]))
        got = g.get_neighbors_within_distance(loc, 5.0)
        want_ids, want_st = o.query(1, loc.x, loc.y, 5.0)
        assert [b.id for b in got] == list(want_ids)
        assert all(b.pos.x == s[0] and b.last_d.y == s[3] for b, s in zip(got, want_st))
    # empty bags and iteration
    eb = np.array([[b.x, b.y] for b in g.get_empty_bags()], np.float32).reshape(-1, 2)
    assert np.array_equal(eb, o.empty_bags())


def test_write_buffer_semantics_match_oracle(gpu):
    rng = np.random.default_rng(2)
    side, d = 20.0, 1.0
    g = kg.Field2D(side, side, d, True)
    o = oracle.OracleField(side, side, d, True)
    n = 200
    xy = (rng.random((n, 2), dtype=np.float32) * np.float32(side)).astype(np.float32)
    for rnd in range(3):
        for i in range(n):
            loc = xy[(i * 7 + rnd) % n]
            g.set_object_location(Bird(i, Real2D(float(xy[i, 0]), float(xy[i, 1]))),
                                  Real2D(float(loc[0]), float(loc[1])))
            o.set(i, float(xy[i, 0]), float(xy[i, 1]), 0.0, 0.0, float(loc[0]), float(loc[1]))
        for i in range(0, n, 9):
            loc = xy[(i * 7 + rnd) % n]
            g.remove_object_location(Bird(i, Real2D(0.0, 0.0)), Real2D(float(loc[0]), float(loc[1])))
            o.remove(i, float(loc[0]), float(loc[1]))
        for k in range(0, n, 13):
            loc = Real2D(float(xy[k, 0]), float(xy[k, 1]))
            want, _ = o.query(3, loc.x, loc.y)
            assert [b.id for b in g.get_objects_unbuffered(loc)] == list(want)
        g.lazy_update()
        o.lazy_update()
        assert g.nagents == o.nagents
        gi, gs = g.get_state()
        oi, os_, _ = o.iter(1)
        assert np.array_equal(gi, oi) and np.array_equal(gs, os_)


def test_empty_single_and_growing_fields(gpu):
    p = kg.FlockParams(seed=1, arith=kg.KB_ARITH_STRICT)
    pc = p.to_c()
    # no boids at all: steps run and leave nothing
    f = kg.Field2D(50.0, 50.0, FLOCK_D, True)
    f.lazy_update()
    L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(0), C.c_uint32(5))
    ids, st = f.get_state()
    assert len(ids) == 0 and f.nagents == 0
    assert len(f.get_neighbors_within_relax_distance(Real2D(25.0, 25.0), 10.0)) == 0
    # one boid (its only candidate is itself) and a field grown from no
    # capacity to 5,000 boids, against the oracle
    for n in (1, 5000):
        ids0, xy0, dxy0 = kg.gen_uniform(n, 200.0, 200.0, 3, 1.0)
        g = kg.Field2D(200.0, 200.0, FLOCK_D, True, capacity_hint=0)
        g.set_locations(ids0, xy0, dxy0)
        g.lazy_update()
        o = oracle.OracleField(200.0, 200.0, FLOCK_D, True)
        o.set_many(ids0, xy0, dxy0)
        o.lazy_update()
        L.call("kb_flock_step", g.handle, C.byref(pc), C.c_uint64(0), C.c_uint32(12))
        o.flock_run(oracle.params_from(p), 0, 12)
        gi, gs = g.get_state()
        oi, os_, _ = o.iter(1)
        assert np.array_equal(gi, oi) and np.array_equal(gs.view(np.uint32), os_.view(np.uint32))


def test_query_radius_edge_values_match_oracle(gpu):
    # the device's float -> i32 conversion must act as Rust's `as i32`
    # (truncate, saturate, NaN -> 0) in floor(dist / d): a NaN radius gives a
    # one-bag range (dd = 0) in both, a huge one the whole matrix
    side, d = 60.0, 2.5
    rng = np.random.default_rng(8)
    ids = np.arange(500, dtype=np.uint32)
    xy = (rng.random((500, 2)) * side).astype(np.float32)
    dxy = np.zeros((500, 2), np.float32)
    g = kg.Field2D(side, side, d, True)
    g.set_locations(ids, xy, dxy)
    g.lazy_update()
    o = oracle.OracleField(side, side, d, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    q = xy[:40]
    for r in (float("nan"), 1.0e6, 2.5, 2.4999998):
        for kind in (kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT):
            gc, gl = g.neighbor_lists(kind, r, q)
            oc, ol = o.neighbor_lists(kind, r, q)
            assert np.array_equal(gc, oc) and np.array_equal(gl, ol), (r, kind)


def test_bulk_set_rejects_bad_objects_and_keeps_the_write_buffer(gpu):
    f = kg.Field2D(50.0, 50.0, 2.0, True)
    f.set_object_location(Bird(1, Real2D(3.0, 4.0)), Real2D(3.0, 4.0))
    ids = np.arange(10, 20, dtype=np.uint32)
    xy = np.full((10, 2), 10.0, np.float32)
    dxy = np.zeros((10, 2), np.float32)
    xy[6] = (-5.0, 10.0)  # outside the bag matrix: the reference panics
    with pytest.raises(kg.KbError) as e:
        f.set_locations(ids, xy, dxy)
    assert e.value.status == L.KB_ERR_RANGE and "object 6" in str(e.value)
    xy[6] = (10.0, 10.0)
    dxy[3] = (float("nan"), 0.0)
    with pytest.raises(kg.KbError) as e:
        f.set_locations(ids, xy, dxy)
    assert e.value.status == L.KB_ERR_ARG
    # the refused batches left nothing behind; a good one follows the earlier write
    dxy[3] = (0.0, 0.0)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    got, st = f.get_state()
    assert list(got) == [1] + list(range(10, 20))
    assert f.nagents == 11


def test_lookups_by_object_read_and_write_buffers(gpu):
    # the parallel build's get / get_location (read buffer) and get_unbuffered /
    # get_location_unbuffered (write buffer): the stored copy or None
    f = kg.Field2D(10.0, 10.0, 0.5, True)
    a, b = Bird(1, Real2D(1.0, 2.0), Real2D(0.5, 0.0)), Bird(2, Real2D(7.0, 3.0))
    f.set_object_location(a, a.pos)
    f.set_object_location(b, b.pos)
    assert f.get(a) is None and f.get_location_unbuffered(a) == Real2D(1.0, 2.0)
    f.lazy_update()
    assert f.get_location(a) == Real2D(1.0, 2.0) and f.get(b) == b
    assert f.get(a).last_d == Real2D(0.5, 0.0)
    assert f.get_unbuffered(a) is None and f.get(Bird(9, Real2D(0.0, 0.0))) is None
    moved = Bird(1, Real2D(4.0, 4.0))
    f.set_object_location(moved, moved.pos)
    assert f.get_location_unbuffered(a) == Real2D(4.0, 4.0)
    assert f.get_location(a) == Real2D(1.0, 2.0)  # the read buffer until lazy_update
    f.lazy_update()
    assert f.get_location(a) == Real2D(4.0, 4.0) and f.get(b) is None
    # many at once, after steps of a flock: equal to the stored states
    ids, xy, dxy = kg.gen_uniform(3000, 300.0, 300.0, 5, 1.0)
    g = kg.Field2D(300.0, 300.0, float(np.float32(10.0) / np.float32(1.5)), True)
    g.set_locations(ids, xy, dxy)
    g.lazy_update()
    L.call("kb_flock_step", g.handle, C.byref(kg.FlockParams(seed=2).to_c()), C.c_uint64(0),
           C.c_uint32(5))
    sid, sst = g.get_state()
    q = np.concatenate([sid[::7], [70000, 70001]]).astype(np.uint32)
    found, st = g.get_locations(q)
    assert found[:-2].all() and not found[-2:].any()
    order = {int(i): k for k, i in enumerate(sid)}
    want = sst[[order[int(i)] for i in q[:-2]]]
    assert np.array_equal(st[:-2].view(np.uint32), want.view(np.uint32))


def test_handles_close_as_context_managers(gpu):
    with kg.Field2D(W, H, D, True) as f:
        f.set_locations(np.array([4], np.uint32), np.array([[1.0, 2.0]], np.float32),
                        np.zeros((1, 2), np.float32))
        f.lazy_update()
        ids, _ = f.get_state()
        assert ids.tolist() == [4]
    assert f.handle is None
    f.close()  # closing twice is harmless
