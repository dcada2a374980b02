"""The schedule bookkeeping on the CPU.

* ``Schedule`` with host-side agents follows schedule.rs:283-413 (priority
  order, time jumps, repeating / once, is_stopped, dequeue).
* The per-bird restatement of Schedule::step over the oracle equals the
  oracle's plain flock run when no bird joins or leaves.
* ``Flocker``'s grouped bird schedule, driven over an oracle-backed field,
  equals the per-bird restatement bit for bit (strict arithmetic) while birds
  join, wait and leave.  The GPU tests run the same scenario on the device.
"""
import numpy as np

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D
from schedule_restatement import BirdQueue

N0 = 300
SIDE = float(np.sqrt(N0 / 0.025))


class Recorder(kg.State):
    def __init__(self):
        self.log = []

    def init(self, schedule):
        pass


class Tick(kg.Agent):
    def __init__(self, name, stop_after=None):
        self.name, self.stop_after, self.n = name, stop_after, 0

    def step(self, state):
        self.n += 1
        state.log.append(self.name)

    def is_stopped(self, state):
        return self.stop_after is not None and self.n >= self.stop_after


def test_schedule_pops_by_time_then_ordering():
    st, s = Recorder(), kg.Schedule()
    assert s.schedule_repeating(Tick("a"), 0.0, 1)
    assert s.schedule_repeating(Tick("b"), 0.0, 0)
    assert s.schedule_repeating(Tick("c", stop_after=2), 1.0, 0)
    s.schedule_once(kg.AgentImpl(99, Tick("once")), 2.0, 5)
    for _ in range(4):
        s.step_state(st)
    # time 0: b (ordering 0) before a; time 1: c joins (queued before b's
    # re-insertion, so first among ordering 0); time 2: once last; c stops
    # after its second step
    assert st.log == ["b", "a", "c", "b", "a", "c", "b", "a", "once", "b", "a"]
    assert s.step == 4 and s.time == 3.0
    assert s.dequeue(None, 1)          # b's queue id
    assert not s.dequeue(None, 1)
    s.step_state(st)
    assert st.log[-1] == "a" and len(s.get_all_events()) == 1


def test_schedule_jumps_to_the_earliest_time_and_runs_empty():
    st, s = Recorder(), kg.Schedule()
    s.schedule_repeating(Tick("late"), 7.5, 0)
    s.step_state(st)
    assert s.time == 7.5 and st.log == ["late"]
    s.dequeue(None, 0)
    s.step_state(st)                   # no agent: the step still counts
    assert s.step == 2 and s.time == 7.5


def params(seed):
    return kg.FlockParams(seed=seed, arith=kg.KB_ARITH_STRICT)


def test_restatement_equals_plain_oracle_run():
    p = params(4)
    ids, xy, dxy = kg.gen_uniform(N0, SIDE, SIDE, 5, 1.0)
    r = BirdQueue(SIDE, SIDE, FLOCK_D, oracle.params_from(p))
    r.init(ids, xy, dxy)
    r.run(6)
    o = oracle.OracleField(SIDE, SIDE, FLOCK_D, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    o.flock_run(oracle.params_from(p), 0, 6)
    a, b = r.state(), o.iter(1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert r.time == 5.0 and r.step == 6


class OracleBackedField:
    """The Field2D methods Flocker uses, served by the CPU oracle."""

    def __init__(self):
        self.o = oracle.OracleField(SIDE, SIDE, FLOCK_D, True)

    def set_locations(self, ids, xy, dxy):
        self.o.set_many(ids, xy, dxy)

    def lazy_update(self):
        self.o.lazy_update()

    def get_state(self):
        ids, st, _ = self.o.iter(1)
        return ids, st

    def num_objects(self):
        return len(self.o.iter(1)[0])

    def flock_compute(self, p, step):
        self.o.flock_compute(oracle.params_from(p), step)

    def flock_compute_agents(self, p, step, ids, states):
        self.o.flock_compute_agents(oracle.params_from(p), step, ids, states)

    def remove_ids(self, ids):
        return self.o.remove_ids(ids)

    def flock_step(self, p, first, n):
        self.o.flock_run(oracle.params_from(p), first, n)


def new_birds(ids, seed):
    rng = np.random.default_rng(seed)
    xy = (rng.random((len(ids), 2)) * SIDE).astype(np.float32)
    dxy = (rng.standard_normal((len(ids), 2)) * 0.5).astype(np.float32)
    return np.asarray(ids, np.uint32), xy, dxy


def test_grouped_bird_schedule_equals_per_bird_restatement():
    p = params(8)
    ids, xy, dxy = kg.gen_uniform(N0, SIDE, SIDE, 5, 1.0)
    g = kg.Flocker((SIDE, SIDE), N0, discretization=FLOCK_D, params=p,
                   init_state=(ids, xy, dxy), field=OracleBackedField())
    s = kg.Schedule()
    g.init(s)
    r = BirdQueue(SIDE, SIDE, FLOCK_D, oracle.params_from(p))
    r.init(ids, xy, dxy)

    def check(what):
        a, b = g.field1.get_state(), r.state()
        assert s.step == r.step and s.time == r.time, what
        assert np.array_equal(a[0], b[0]), what
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), what

    def sched(*args, **kw):
        g.schedule_birds(*args, **kw)
        r.schedule(*args, **kw)

    def run(k):
        g.run_steps(s, k)
        r.run(k)

    run(3)
    check("plain")
    sched(*new_birds(range(300, 350), 1), 5.0)
    sched(*new_birds(range(350, 370), 2), 4.0, repeating=False)
    run(3)
    check("joiners")
    assert g.dequeue_birds(np.arange(0, 30)) == r.dequeue(np.arange(0, 30)) == 30
    run(2)
    check("dequeued")
    sched(*new_birds(range(400, 420), 3), 7.5, the_ordering=1)
    sched(*new_birds(range(420, 430), 4), 7.5, the_ordering=0)
    for k in range(3):
        run(1)
        check(f"half-time step {k}")
    drop = np.concatenate([np.arange(40, 60), np.arange(405, 410), [9999, 5]])
    assert g.dequeue_birds(drop) == r.dequeue(drop)
    run(4)
    check("second dequeue")
    assert g.queued_birds() == len(r.q)


def test_every_bird_leaves_then_a_group_arrives_host():
    p = params(3)
    ids, xy, dxy = kg.gen_uniform(N0, SIDE, SIDE, 5, 1.0)
    g = kg.Flocker((SIDE, SIDE), N0, discretization=FLOCK_D, params=p,
                   init_state=(ids, xy, dxy), field=OracleBackedField())
    s = kg.Schedule()
    g.init(s)
    r = BirdQueue(SIDE, SIDE, FLOCK_D, oracle.params_from(p))
    r.init(ids, xy, dxy)
    g.run_steps(s, 2)
    r.run(2)
    a = new_birds(range(1000, 1040), 9)
    g.schedule_birds(*a, 6.0)
    r.schedule(*a, 6.0)
    assert g.dequeue_birds(np.arange(N0)) == r.dequeue(np.arange(N0)) == N0
    g.run_steps(s, 3)
    r.run(3)
    assert s.time == r.time == 8.0 and s.step == r.step == 5  # times 6, 7, 8
    ga, ra = g.field1.get_state(), r.state()
    assert np.array_equal(ga[0], ra[0]) and np.array_equal(ga[1].view(np.uint32), ra[1].view(np.uint32))
    assert g.field1.num_objects() == 40
    assert g.dequeue_birds(a[0]) == r.dequeue(a[0]) == 40
    g.run_steps(s, 2)
    r.run(2)
    assert g.field1.num_objects() == 0 and g.queued_birds() == 0 and len(r.state()[0]) == 0
    assert s.step == r.step == 7
