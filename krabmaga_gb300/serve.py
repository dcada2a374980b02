"""Continuous-batching request server over the C ABI (kb_server_*).

Each request is a whole Flockers simulation (uniform flock of ``nboids`` from
``init_seed``, ``steps`` steps).  The server loop runs in a native thread:
running requests share batched persistent launches; queued ones are
admitted between epochs when a slot is free and their device state fits the
HBM budget.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L
from .model import FlockParams


@dataclass
class Request:
    nboids: int
    side: float
    discretization: float
    steps: int
    params: FlockParams
    init_seed: int
    heading_scale: float = 1.0

    def to_c(self) -> L.RequestC:
        return L.RequestC(self.nboids, self.side, self.discretization, self.steps,
                          self.params.to_c(), self.init_seed, self.heading_scale, 0)


class Server:
    def __init__(self, max_slots: int = 64, hbm_budget_bytes: int = 120 << 30,
                 quantum_steps: int = 100, max_request_boids: int = 262144,
                 max_request_cells: int = 1 << 21, query_mode: int = L.KB_QUERY_RELAX,
                 arith: int = L.KB_ARITH_FAST, device: int = 0):
        d = L.ServerDesc(device, max_slots, hbm_budget_bytes, quantum_steps, max_request_boids,
                         max_request_cells, query_mode, arith, 0)
        h = C.c_void_p()
        L.call("kb_server_create", C.byref(d), C.byref(h))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            L.lib.kb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def submit(self, req: Request) -> int:
        t = C.c_uint64()
        L.call("kb_server_submit", self._h, C.byref(req.to_c()), C.byref(t))
        return t.value

    def poll(self, ticket: int):
        st = C.c_int32()
        lat = C.c_double()
        L.call("kb_server_poll", self._h, C.c_uint64(ticket), C.byref(st), C.byref(lat))
        return st.value, lat.value

    def result(self, ticket: int, nboids: int):
        n = C.c_size_t()
        ids = np.zeros(max(nboids, 1), np.uint32)
        st = np.zeros((max(nboids, 1), 4), np.float32)
        L.call("kb_server_result", self._h, C.c_uint64(ticket), L.uptr(ids), L.fptr(st),
               C.c_size_t(nboids), C.byref(n))
        return ids[: n.value], st[: n.value]

    def release(self, ticket: int) -> None:
        L.call("kb_server_release", self._h, C.c_uint64(ticket))

    def wait_idle(self, timeout_s: float = 600.0) -> None:
        L.call("kb_server_wait_idle", self._h, C.c_double(timeout_s))

    def stats(self) -> dict:
        r = L.ServerReport()
        L.call("kb_server_stats", self._h, C.byref(r))
        return {k: getattr(r, k) for k, _ in L.ServerReport._fields_}


def request_stream(rate_hz: float, seconds: float, n_min: int = 1024, n_max: int = 262144,
                   steps_min: int = 100, steps_max: int = 1000, density: float = 0.025,
                   arith: int = L.KB_ARITH_FAST, seed: int = 77):
    """The served request stream: Poisson arrivals at rate_hz for `seconds`;
    each request has N log-uniform in [n_min, n_max] at the given density,
    steps uniform in [steps_min, steps_max], weights U[0.5,1.5], jump
    U[0.3,1.0], radius U[5,15], discretization radius/1.5, and its own
    seeds.  Returns a list of (arrival offset in s, Request)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    k = 0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= seconds:
            break
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        side = float(np.float32(np.sqrt(n / density)))
        w = rng.uniform(0.5, 1.5, 5)
        jump = float(rng.uniform(0.3, 1.0))
        radius = float(np.float32(rng.uniform(5.0, 15.0)))
        d = float(np.float32(radius) / np.float32(1.5))
        steps = int(rng.integers(steps_min, steps_max + 1))
        p = FlockParams(cohesion=float(w[0]), avoidance=float(w[1]), consistency=float(w[2]),
                        randomness=float(w[3]), momentum=float(w[4]), jump=jump,
                        neighbor_radius=radius, arith=arith, seed=100000 + k)
        out.append((t, Request(n, side, d, steps, p, init_seed=200000 + k)))
        k += 1
    return out
