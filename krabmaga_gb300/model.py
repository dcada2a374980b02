"""State / Schedule / simulate and the Flockers model over the GPU field.

Mirrors the reference's driver path:
  * ``State`` trait            -- src/engine/state.rs:45-63
  * ``Schedule::step``         -- src/engine/schedule.rs:347-413
  * ``simulate!`` plain loop   -- src/lib.rs:1158-1175
  * ``simulate_old!``          -- src/lib.rs:1473-1582 (returns (seconds, steps/s) per rep)
  * ``Flocker`` State          -- tests/model/flockers/state.rs:11-60
  * ``Bird::step``             -- tests/model/flockers/bird.rs:39-154, run for every bird
                                  at once by ``kb_flock_compute``

The per-agent loop of ``Schedule::step`` cannot run a Python closure per bird
on the GPU, so the drop-in is model-specialised: ``Flocker.before_step``
launches the whole agent pass (every Bird::step) and ``Flocker.update`` is the
field's ``lazy_update``, exactly where the reference calls them.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

from . import _lib as L
from .field import Bird, Field2D, Real2D


@dataclass
class FlockParams:
    """bird.rs:12-17 statics + the bird.rs:41 radius + the jitter seed."""

    cohesion: float = 1.0
    avoidance: float = 1.0
    consistency: float = 1.0
    randomness: float = 1.0
    momentum: float = 1.0
    jump: float = 0.7
    neighbor_radius: float = 10.0
    query_mode: int = L.KB_QUERY_RELAX
    arith: int = L.KB_ARITH_STRICT
    seed: int = 0

    def to_c(self) -> L.FlockParamsC:
        return L.FlockParamsC(self.cohesion, self.avoidance, self.consistency, self.randomness,
                              self.momentum, self.jump, self.neighbor_radius, self.query_mode,
                              self.arith, 0, self.seed)


def gen_uniform(n: int, w: float, h: float, seed: int, heading_scale: float = 1.0):
    """Uniform flock from Philox(seed): (ids, xy[n,2], dxy[n,2])."""
    ids = np.zeros(max(n, 1), np.uint32)
    xy = np.zeros((max(n, 1), 2), np.float32)
    dxy = np.zeros((max(n, 1), 2), np.float32)
    L.call("kb_gen_uniform", C.c_size_t(n), C.c_float(w), C.c_float(h), C.c_uint64(seed),
           C.c_float(heading_scale), L.uptr(ids), L.fptr(xy), L.fptr(dxy))
    return ids[:n], xy[:n], dxy[:n]


def gen_clustered(n: int, w: float, h: float, nclusters: int, sigma: float, angle_sigma: float,
                  seed: int):
    ids = np.zeros(max(n, 1), np.uint32)
    xy = np.zeros((max(n, 1), 2), np.float32)
    dxy = np.zeros((max(n, 1), 2), np.float32)
    L.call("kb_gen_clustered", C.c_size_t(n), C.c_float(w), C.c_float(h), C.c_uint32(nclusters),
           C.c_float(sigma), C.c_float(angle_sigma), C.c_uint64(seed), L.uptr(ids), L.fptr(xy),
           L.fptr(dxy))
    return ids[:n], xy[:n], dxy[:n]


class State:
    """src/engine/state.rs:45-63 (sequential build)."""

    def init(self, schedule: "Schedule") -> None:
        raise NotImplementedError

    def reset(self) -> None:
        pass

    def update(self, step: int) -> None:
        pass

    def before_step(self, schedule: "Schedule") -> None:
        pass

    def after_step(self, schedule: "Schedule") -> None:
        pass

    def end_condition(self, schedule: "Schedule") -> bool:
        return False


class Agent:
    """src/engine/agent.rs:7-40: a host-side agent of the Schedule queue."""

    def step(self, state: State) -> None:
        raise NotImplementedError

    def is_stopped(self, state: State) -> bool:
        return False

    def before_step(self, state: State):
        return None

    def after_step(self, state: State):
        return None


@dataclass
class AgentImpl:
    """src/engine/agentimpl.rs:15-19: an agent with its queue id."""

    id: int
    agent: Agent
    repeating: bool = False


class Schedule:
    """Schedule -- schedule.rs:262-413 (sequential build).

    The queue holds host-side agents (``Agent``) with their priority (time,
    then ordering, lower first: priority.rs:21-38); agents of equal priority
    pop in the order they were queued (the reference leaves that order to its
    priority-queue crate).  The GPU Flocker keeps no per-bird entries here:
    its whole agent pass runs in ``before_step``, where the reference runs
    each bird's step, and its birds' own schedule is ``Flocker.schedule_birds``
    / ``Flocker.dequeue_birds``."""

    def __init__(self):
        self.step = 0
        self.time = 0.0
        self.agent_ids_counting = 0
        self._events = {}  # queue id -> (time, ordering, seq, AgentImpl)
        self._seq = 0

    def _push(self, a: AgentImpl, the_time: float, the_ordering: int) -> bool:
        fresh = a.id not in self._events
        self._events[a.id] = (float(np.float32(the_time)), int(the_ordering), self._seq, a)
        self._seq += 1
        return fresh

    def schedule_once(self, agent: AgentImpl, the_time: float, the_ordering: int = 0) -> None:
        """schedule.rs:283-285"""
        self._push(agent, the_time, the_ordering)

    def schedule_repeating(self, agent: Agent, the_time: float = 0.0, the_ordering: int = 0) -> bool:
        """schedule.rs:295-303: a new queue id; True when the insertion is new."""
        a = AgentImpl(self.agent_ids_counting, agent, True)
        self.agent_ids_counting += 1
        return self._push(a, the_time, the_ordering)

    def dequeue(self, agent: Agent, my_id: int) -> bool:
        """schedule.rs:329-343: remove the entry with queue id my_id."""
        return self._events.pop(my_id, None) is not None

    def get_all_events(self) -> List[Agent]:
        """schedule.rs:316-322 (sequential build)"""
        return [e[3].agent for e in self._events.values()]

    def step_state(self, state: State) -> None:
        """Schedule::step -- schedule.rs:347-413."""
        if self.step == 0:
            state.update(self.step)  # schedule.rs:349-351
        state.before_step(self)
        if self._events:
            self.time = min((e[0], e[1], e[2]) for e in self._events.values())[0]
            due = sorted((e for e in self._events.values() if e[0] <= self.time),
                         key=lambda e: (e[0], e[1], e[2]))
            for e in due:
                del self._events[e[3].id]
            for t, o, _, a in due:
                a.agent.before_step(state)
                a.agent.step(state)
                a.agent.after_step(state)
                if a.repeating and not a.agent.is_stopped(state):
                    self.schedule_once(a, t + 1.0, o)
        state.after_step(self)
        self.step += 1
        state.update(self.step)  # schedule.rs:410-412


@dataclass
class _BirdGroup:
    """Birds waiting in the queue with their own state (not in the field)."""

    time: float
    ordering: int
    seq: int
    ids: np.ndarray
    states: np.ndarray  # n x {x, y, dx, dy}
    repeating: bool


class Flocker(State):
    """tests/model/flockers/state.rs:11-60 on the GPU field.

    ``dim`` and ``initial_flockers`` as in ``Flocker::new``; ``discretization``
    defaults to the reference's 0.5 (state.rs:13), ``toroidal`` to true.
    Initial positions and headings come from Philox(init_seed): ``heading_scale``
    0 gives the reference's zero heading (state.rs:47).

    The birds' own schedule (every bird ``schedule_repeating(bird, 0., 0)`` in
    init, state.rs:52-54) is kept per bird group rather than per bird:

    * the birds of the read buffer that are queued all share one next time;
      they step together in one ``kb_flock_compute``;
    * birds queued with ``schedule_birds`` (schedule_repeating or
      schedule_once at some time, schedule.rs:283-303) wait with their own
      state and step at their time through ``kb_flock_compute_agents``;
    * ``dequeue_birds`` (Schedule::dequeue, schedule.rs:329-343, or a bird
      whose is_stopped turned true after its step, schedule.rs:401) takes
      birds out of the queue; the field drops them when the reference would
      stop writing them.

    Each step runs the queued birds of the earliest queued time (schedule.rs:
    366-393): first those of the read buffer (in read order), then the waiting
    groups by (ordering, queueing order).  A queued bird that does not step
    while the read buffer's others do is not written, so it leaves the field
    at that lazy_update, as in the reference; the read buffer's queued birds
    that wait for a later time than the step's are kept as a waiting group."""

    def __init__(self, dim: Tuple[float, float], initial_flockers: int,
                 discretization: float = 0.5, toroidal: bool = True,
                 params: Optional[FlockParams] = None, init_seed: int = 0,
                 heading_scale: float = 0.0, device: int = 0,
                 init_state: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None,
                 field=None):
        """``field``: a field to use instead of a new ``Field2D`` (for instance
        one created with other options); ``reset`` makes a new ``Field2D``."""
        self.dim = (float(dim[0]), float(dim[1]))
        self.initial_flockers = int(initial_flockers)
        self.discretization = discretization
        self.toroidal = toroidal
        self.params = params or FlockParams()
        self.init_seed = init_seed
        self.heading_scale = heading_scale
        self.device = device
        self.init_state = init_state
        self.step = 0
        self.field1 = field if field is not None else Field2D(
            self.dim[0], self.dim[1], discretization, toroidal, device,
            capacity_hint=self.initial_flockers)
        self._clear_schedule()

    def _clear_schedule(self) -> None:
        self._field_time: Optional[float] = None  # next time of the read buffer's queued birds
        self._field_count = 0                      # how many of them are queued
        self._unqueued: set = set()                # in the read buffer, not queued
        self._groups: List[_BirdGroup] = []
        self._gseq = 0
        self._order_of: dict = {}  # bird id -> its non-zero ordering (birds of the read buffer)

    def reset(self) -> None:
        self.step = 0
        self.field1.close()
        self.field1 = Field2D(self.dim[0], self.dim[1], self.discretization, self.toroidal,
                              self.device, capacity_hint=self.initial_flockers)
        self._clear_schedule()

    def init(self, schedule: Schedule) -> None:
        if self.init_state is not None:
            ids, xy, dxy = self.init_state
        else:
            ids, xy, dxy = gen_uniform(self.initial_flockers, self.dim[0], self.dim[1],
                                       self.init_seed, self.heading_scale)
        self.field1.set_locations(ids, xy, dxy)
        # state.rs:52-54: every bird schedule_repeating(bird, 0., 0)
        self._clear_schedule()
        self._field_count = len(ids)
        self._field_time = 0.0 if len(ids) else None

    # ------------------------------------------------------ bird schedule
    def schedule_birds(self, ids, xy, dxy, the_time: float, the_ordering: int = 0,
                       repeating: bool = True) -> None:
        """Queue new birds (ids, positions, headings) at ``the_time``:
        schedule_repeating when ``repeating``, else schedule_once."""
        ids = np.ascontiguousarray(ids, np.uint32).reshape(-1)
        st = np.concatenate([np.asarray(xy, np.float32).reshape(-1, 2),
                             np.asarray(dxy, np.float32).reshape(-1, 2)], axis=1)
        assert len(ids) == len(st)
        if len(ids) == 0:
            return
        self._groups.append(_BirdGroup(float(np.float32(the_time)), int(the_ordering), self._gseq,
                                       ids, np.ascontiguousarray(st), bool(repeating)))
        self._gseq += 1

    def dequeue_birds(self, ids) -> int:
        """Take birds out of the queue; returns how many were queued."""
        drop = np.unique(np.asarray(ids, np.uint32).reshape(-1))
        found = 0
        kept = []
        for g in self._groups:
            m = np.isin(g.ids, drop)
            found += int(m.sum())
            if not m.all():
                kept.append(_BirdGroup(g.time, g.ordering, g.seq, g.ids[~m], g.states[~m],
                                       g.repeating))
        self._groups = kept
        if self._field_time is not None:
            rid, _ = self.field1.get_state()
            hit = set(rid[np.isin(rid, drop)].tolist()) - self._unqueued
            for i in hit:
                self._order_of.pop(i, None)
            found += len(hit)
            self._unqueued |= hit
            self._field_count -= len(hit)
            if self._field_count == 0:
                self._field_time = None
        return found

    def queued_birds(self) -> int:
        return self._field_count + sum(len(g.ids) for g in self._groups)

    def _plain_steps(self) -> float:
        """How many coming steps step exactly the read buffer's queued birds
        (no bird joins, leaves or waits)."""
        if self._unqueued or self._field_time is None:
            return 0
        if not self._groups:
            return float("inf")
        first = min(g.time for g in self._groups)
        return float(np.ceil(first - self._field_time)) if first > self._field_time else 0

    def before_step(self, schedule: Schedule) -> None:
        # schedule.rs:366-408 for the birds: the earliest queued time steps
        if self._plain_steps() >= 1:
            schedule.time = self._field_time
            self.field1.flock_compute(self.params, schedule.step)
            self._field_time += 1.0
            return
        times = [g.time for g in self._groups]
        if self._field_time is not None:
            times.append(self._field_time)
        if not times:
            self._unqueued = set()
            return  # no bird queued: nothing is written
        cur = min(times)
        schedule.time = cur
        if self._field_time is not None and self._field_time > cur:
            # the read buffer's queued birds wait: keep their own state,
            # one group per ordering, each in read order
            rid, st = self.field1.get_state()
            keep = ~np.isin(rid, np.fromiter(self._unqueued, np.uint32, len(self._unqueued)))
            rid, st = rid[keep], st[keep]
            order = np.array([self._order_of.get(int(i), 0) for i in rid.tolist()], np.int64) \
                if self._order_of else np.zeros(len(rid), np.int64)
            for o in np.unique(order).tolist():
                m = order == o
                self._groups.append(_BirdGroup(self._field_time, int(o), -1, rid[m].copy(),
                                               st[m].copy(), True))
            self._field_time, self._field_count = None, 0
        count = 0
        if self._field_time is not None:
            self.field1.flock_compute(self.params, schedule.step)
            removed = self.field1.remove_ids(sorted(self._unqueued)) if self._unqueued else 0
            count = self.field1.num_objects() - removed
        self._unqueued = set()
        due = sorted((g for g in self._groups if g.time == cur), key=lambda g: (g.ordering, g.seq))
        self._groups = [g for g in self._groups if g.time != cur]
        for g in due:
            self.field1.flock_compute_agents(self.params, schedule.step, g.ids, g.states)
            if g.repeating:
                count += len(g.ids)
                if g.ordering:
                    self._order_of.update(dict.fromkeys(g.ids.tolist(), g.ordering))
            else:
                self._unqueued |= set(g.ids.tolist())  # schedule_once: not queued again
        self._field_count = count
        self._field_time = cur + 1.0 if count else None

    def update(self, step: int) -> None:
        self.step = step
        self.field1.lazy_update()  # state.rs:58-60

    def run_steps(self, schedule: Schedule, nsteps: int) -> None:
        """``nsteps`` Schedule::step calls.  Runs of steps with no bird
        joining or leaving are fused into CUDA-graph replays."""
        if schedule.step == 0:
            self.update(0)
        left = nsteps
        while left > 0:
            k = int(min(left, self._plain_steps()))
            if k == 0:
                self.before_step(schedule)
                schedule.step += 1
                self.update(schedule.step)
                left -= 1
                continue
            self.field1.flock_step(self.params, schedule.step, k)
            schedule.time = self._field_time + (k - 1)
            self._field_time += float(k)
            schedule.step += k
            self.step = schedule.step
            left -= k


def simulate(state: State, n_step: int, reps: int = 1) -> None:
    """simulate! without UI -- lib.rs:1158-1175."""
    for _ in range(reps):
        schedule = Schedule()
        state.init(schedule)
        if isinstance(state, Flocker):
            state.run_steps(schedule, n_step)
            state.field1.synchronize()
        else:
            for _ in range(n_step):
                schedule.step_state(state)
                if state.end_condition(schedule):
                    break


def simulate_old(state: State, n_step: int, reps: int) -> List[Tuple[float, float]]:
    """simulate_old! -- lib.rs:1473-1582: per rep (seconds, steps/s), init excluded."""
    results = []
    for _ in range(reps):
        if isinstance(state, Flocker):
            state.reset()
        schedule = Schedule()
        state.init(schedule)
        t0 = time.perf_counter()
        if isinstance(state, Flocker):
            state.run_steps(schedule, n_step)
            state.field1.synchronize()
        else:
            for _ in range(n_step):
                schedule.step_state(state)
                if state.end_condition(schedule):
                    break
        dt = time.perf_counter() - t0
        results.append((dt, schedule.step / dt if dt > 0 else float("inf")))
    return results
