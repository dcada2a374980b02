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


class Schedule:
    """Schedule::step -- schedule.rs:347-413.  The GPU state runs its whole
    agent pass in before_step, so the queue holds no per-bird entries."""

    def __init__(self):
        self.step = 0
        self.time = 0.0

    def step_state(self, state: State) -> None:
        if self.step == 0:
            state.update(self.step)  # schedule.rs:349-351
        state.before_step(self)
        state.after_step(self)
        self.step += 1
        self.time += 1.0
        state.update(self.step)  # schedule.rs:410-412


class Flocker(State):
    """tests/model/flockers/state.rs:11-60 on the GPU field.

    ``dim`` and ``initial_flockers`` as in ``Flocker::new``; ``discretization``
    defaults to the reference's 0.5 (state.rs:13), ``toroidal`` to true.
    Initial positions and headings come from Philox(init_seed): ``heading_scale``
    0 gives the reference's zero heading (state.rs:47)."""

    def __init__(self, dim: Tuple[float, float], initial_flockers: int,
                 discretization: float = 0.5, toroidal: bool = True,
                 params: Optional[FlockParams] = None, init_seed: int = 0,
                 heading_scale: float = 0.0, device: int = 0,
                 init_state: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None):
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
        self.field1 = Field2D(self.dim[0], self.dim[1], discretization, toroidal, device,
                              capacity_hint=self.initial_flockers)

    def reset(self) -> None:
        self.step = 0
        self.field1.close()
        self.field1 = Field2D(self.dim[0], self.dim[1], self.discretization, self.toroidal,
                              self.device, capacity_hint=self.initial_flockers)

    def init(self, schedule: Schedule) -> None:
        if self.init_state is not None:
            ids, xy, dxy = self.init_state
        else:
            ids, xy, dxy = gen_uniform(self.initial_flockers, self.dim[0], self.dim[1],
                                       self.init_seed, self.heading_scale)
        self.field1.set_locations(ids, xy, dxy)

    def before_step(self, schedule: Schedule) -> None:
        # every Bird::step of schedule.rs:395-408, in one launch
        L.call("kb_flock_compute", self.field1.handle, C.byref(self.params.to_c()),
               C.c_uint64(schedule.step))

    def update(self, step: int) -> None:
        self.step = step
        self.field1.lazy_update()  # state.rs:58-60

    def run_steps(self, schedule: Schedule, nsteps: int) -> None:
        """``nsteps`` Schedule::step calls fused into CUDA-graph replays."""
        if schedule.step == 0:
            self.update(0)
        L.call("kb_flock_step", self.field1.handle, C.byref(self.params.to_c()),
               C.c_uint64(schedule.step), C.c_uint32(nsteps))
        schedule.step += nsteps
        schedule.time += float(nsteps)
        self.step = schedule.step


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
