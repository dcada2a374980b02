"""Birds joining and leaving the schedule, on the GPU, against a per-bird
restatement of Schedule::step over the CPU oracle (strict arithmetic: the
read buffers agree bit for bit after every phase)."""
import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D
from schedule_restatement import BirdQueue

pytestmark = pytest.mark.gpu

N0 = 300
SIDE = float(np.sqrt(N0 / 0.025))


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def new_birds(ids, seed):
    rng = np.random.default_rng(seed)
    xy = (rng.random((len(ids), 2)) * SIDE).astype(np.float32)
    dxy = (rng.standard_normal((len(ids), 2)) * 0.5).astype(np.float32)
    return np.asarray(ids, np.uint32), xy, dxy


def pair(seed=8):
    p = kg.FlockParams(seed=seed, arith=kg.KB_ARITH_STRICT)
    ids, xy, dxy = kg.gen_uniform(N0, SIDE, SIDE, 5, 1.0)
    g = kg.Flocker((SIDE, SIDE), N0, discretization=FLOCK_D, params=p, init_state=(ids, xy, dxy))
    s = kg.Schedule()
    g.init(s)
    r = BirdQueue(SIDE, SIDE, FLOCK_D, oracle.params_from(p))
    r.init(ids, xy, dxy)
    return g, s, r


def check(g, s, r, what):
    ids, st = g.field1.get_state()
    rids, rst = r.state()
    assert s.step == r.step and s.time == r.time, what
    assert np.array_equal(ids, rids) and same_bits(st, rst), what


def test_birds_join_wait_and_leave_like_the_reference_schedule(gpu):
    g, s, r = pair()
    g.run_steps(s, 3)
    r.run(3)
    check(g, s, r, "plain steps")

    a = new_birds(range(300, 350), 1)      # schedule_repeating at time 5
    b = new_birds(range(350, 370), 2)      # schedule_once at time 4
    g.schedule_birds(*a, 5.0)
    r.schedule(*a, 5.0)
    g.schedule_birds(*b, 4.0, repeating=False)
    r.schedule(*b, 4.0, repeating=False)
    g.run_steps(s, 3)                      # times 3 (plain), 4 (+ once), 5 (+ joiners)
    r.run(3)
    check(g, s, r, "joiners")
    assert g.queued_birds() == N0 + 50

    assert g.dequeue_birds(np.arange(0, 30)) == 30
    assert r.dequeue(np.arange(0, 30)) == 30
    g.run_steps(s, 2)
    r.run(2)
    check(g, s, r, "dequeued")
    assert g.field1.num_objects() == N0 + 20

    # birds at a time between two steps of the field: the field's birds wait
    c = new_birds(range(400, 420), 3)
    e = new_birds(range(420, 430), 4)
    g.schedule_birds(*c, 7.5, the_ordering=1)
    r.schedule(*c, 7.5, the_ordering=1)
    g.schedule_birds(*e, 7.5, the_ordering=0)
    r.schedule(*e, 7.5, the_ordering=0)
    for k in range(3):                     # times 7.5, 8, 8.5
        g.run_steps(s, 1)
        r.run(1)
        check(g, s, r, f"half-time step {k}")

    # dequeue waiting and stepping birds, and ids that are not queued
    drop = np.concatenate([np.arange(40, 60), np.arange(405, 410), [9999, 5]])
    assert g.dequeue_birds(drop) == r.dequeue(drop)
    g.run_steps(s, 4)
    r.run(4)
    check(g, s, r, "after the second dequeue")
    assert g.queued_birds() == len(r.q)


def test_every_bird_leaves_then_a_group_arrives(gpu):
    g, s, r = pair(seed=3)
    g.run_steps(s, 2)
    r.run(2)
    a = new_birds(range(1000, 1040), 9)
    g.schedule_birds(*a, 6.0)
    r.schedule(*a, 6.0)
    assert g.dequeue_birds(np.arange(N0)) == N0
    r.dequeue(np.arange(N0))
    # no bird steps before time 6: the next step jumps there (the field
    # empties at the first lazy_update, since nothing is written)
    g.run_steps(s, 3)
    r.run(3)
    check(g, s, r, "jump to the group's time")
    assert g.field1.num_objects() == 40
    assert g.dequeue_birds(a[0]) == 40
    r.dequeue(a[0])
    g.run_steps(s, 2)                      # nothing queued: empty steps
    r.run(2)
    check(g, s, r, "empty queue")
    assert g.field1.num_objects() == 0 and g.queued_birds() == 0


def test_flock_compute_agents_matches_oracle(gpu):
    # the device primitive alone: caller-held agents after a full agent pass
    p = kg.FlockParams(seed=2, arith=kg.KB_ARITH_STRICT)
    ids, xy, dxy = kg.gen_uniform(N0, SIDE, SIDE, 7, 1.0)
    f = kg.Field2D(SIDE, SIDE, FLOCK_D, True)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    o = oracle.OracleField(SIDE, SIDE, FLOCK_D, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    # agents anywhere, one of them with the id of a field bird (it skips that
    # bird as itself, bird.rs:50), one far outside the field
    aid = np.array([5000, 5001, 17, 5003], np.uint32)
    ast = np.array([[10, 10, 0.3, 0.1], [SIDE - 1, 2, -0.2, 0.5], [50, 60, 0, 0],
                    [-40, SIDE + 30, 0.1, 0.1]], np.float32)
    f.flock_compute(p, 4)
    o.flock_compute(oracle.params_from(p), 4)
    f.flock_compute_agents(p, 4, aid, ast)
    o.flock_compute_agents(oracle.params_from(p), 4, aid, ast)
    assert f.remove_ids([17, 123456]) == 2 and o.remove_ids([17, 123456]) == 2
    f.lazy_update()
    o.lazy_update()
    gi, gs = f.get_state()
    oi, os_, _ = o.iter(1)
    assert len(gi) == N0 + 2          # both birds with id 17 removed
    assert np.array_equal(gi, oi) and same_bits(gs, os_)
    with pytest.raises(kg.KbError):
        f.flock_compute_agents(p, 5, aid[:1], np.array([[np.nan, 0, 0, 0]], np.float32))
