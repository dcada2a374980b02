"""Test infrastructure: Schedule::step over individual birds, on the CPU oracle.

A restatement of the reference's queue semantics for the Flockers birds
(src/engine/schedule.rs:283-303 schedule_once / schedule_repeating, 329-343
dequeue, 347-413 step) with one queue entry per bird, each stepping through
the oracle's Bird::step (tests/model/flockers/bird.rs:39-154) against the
oracle field's read buffer and writing itself with set_object_location.  It
checks the grouped bookkeeping of ``krabmaga_gb300.Flocker`` (one device pass
per step over the queued birds of the read buffer, waiting groups stepped
with kb_flock_compute_agents).

Birds of equal time pop in the same documented order as the GPU mirror: the
queued birds that are in the read buffer in read order, then the others by
(ordering, queueing key).  Queued birds of the read buffer that wait for a
later time get the key (-1, wait count, read position): they lose their place
in the field and keep their own state, as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Tuple

import numpy as np

import oracle


@dataclass
class Entry:
    time: float
    ordering: int
    key: Tuple
    state: np.ndarray  # own {x, y, dx, dy}
    repeating: bool
    in_field: bool  # its last write is the copy in the read buffer


class BirdQueue:
    def __init__(self, w, h, d, params: oracle.Params):
        self.f = oracle.OracleField(w, h, d, True)
        self.p = params
        self.q: Dict[int, Entry] = {}
        self.step = 0
        self.time = 0.0
        self._gseq = 0
        self._waits = 0

    def init(self, ids, xy, dxy):
        # state.rs:41-56: set every bird, schedule_repeating(bird, 0., 0)
        self.f.set_many(ids, xy, dxy)
        for k, i in enumerate(np.asarray(ids, np.uint32).tolist()):
            st = np.array([xy[k][0], xy[k][1], dxy[k][0], dxy[k][1]], np.float32)
            self.q[i] = Entry(0.0, 0, (self._gseq, k), st, True, True)
        self._gseq += 1

    def schedule(self, ids, xy, dxy, the_time, the_ordering=0, repeating=True):
        t = float(np.float32(the_time))
        for k, i in enumerate(np.asarray(ids, np.uint32).tolist()):
            st = np.array([xy[k][0], xy[k][1], dxy[k][0], dxy[k][1]], np.float32)
            self.q[i] = Entry(t, int(the_ordering), (self._gseq, k), st, repeating, False)
        self._gseq += 1

    def dequeue(self, ids):
        n = 0
        for i in np.asarray(ids, np.uint32).tolist():
            n += self.q.pop(i, None) is not None
        return n

    def run(self, nsteps):
        for _ in range(nsteps):
            self._one()

    def _one(self):
        if self.step == 0:
            self.f.lazy_update()  # schedule.rs:349-351
        rb_ids = self.f.iter(1)[0]
        pos = {int(i): k for k, i in enumerate(rb_ids.tolist())}
        if self.q:
            cur = min(e.time for e in self.q.values())
            self.time = cur
            due, wait_field = [], []
            for i, e in self.q.items():
                if e.time == cur:
                    due.append(i)
                elif e.in_field:
                    wait_field.append(i)
            # queued birds of the read buffer that wait lose their field copy
            wait_field.sort(key=lambda i: pos[i])
            for k, i in enumerate(wait_field):
                e = self.q[i]
                e.key = (-1, self._waits, k)
                e.in_field = False
            if wait_field:
                self._waits += 1
            first = sorted((i for i in due if self.q[i].in_field), key=lambda i: pos[i])
            rest = sorted((i for i in due if not self.q[i].in_field),
                          key=lambda i: (self.q[i].ordering, self.q[i].key))
            order = first + rest
            nxt = [self.f.bird_step(self.p, self.step, i, self.q[i].state) for i in order]
            for i, st in zip(order, nxt):
                self.f.set(i, float(st[0]), float(st[1]), float(st[2]), float(st[3]))
                e = self.q[i]
                if e.repeating:
                    e.time = float(np.float32(cur + 1.0))
                    e.state = st
                    e.in_field = True
                else:
                    del self.q[i]  # schedule_once: not queued again
        self.step += 1
        self.f.lazy_update()  # schedule.rs:410-412

    def state(self):
        ids, st, _ = self.f.iter(1)
        return ids, st
