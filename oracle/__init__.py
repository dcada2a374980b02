"""The oracle: TEST INFRASTRUCTURE ONLY.

ctypes binding of ``build/libkrab_oracle.so``, a CPU restatement of krABMaga's
sequential Field2D + Flockers path (see krab_oracle.cpp for the reference
lines each function follows).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may use it, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "build", "libkrab_oracle.so")
if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} missing: run `make -C oracle`")
lib = C.CDLL(LIB_PATH)

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_U32 = C.POINTER(C.c_uint32)


class Params(C.Structure):
    _fields_ = [
        ("cohesion", C.c_float), ("avoidance", C.c_float), ("consistency", C.c_float),
        ("randomness", C.c_float), ("momentum", C.c_float), ("jump", C.c_float),
        ("radius", C.c_float), ("query_mode", C.c_int32), ("seed", C.c_uint64),
    ]


_SIGS = {
    "orc_philox4x32_10": (None, [_U32, _U32, _U32]),
    "orc_jitter_pair": (None, [C.c_uint64, C.c_uint32, C.c_uint64, _F, _F]),
    "orc_field_new": (_P, [C.c_float, C.c_float, C.c_float, C.c_int]),
    "orc_field_free": (None, [_P]),
    "orc_field_set_cell_wrap": (None, [_P, C.c_int]),
    "orc_field_dims": (None, [_P, C.POINTER(C.c_int32)]),
    "orc_field_nagents": (C.c_size_t, [_P]),
    "orc_field_panicked": (C.c_int, [_P]),
    "orc_field_set": (C.c_int, [_P, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float,
                                C.c_float, C.c_float]),
    "orc_field_set_many": (C.c_int, [_P, C.c_size_t, _U32, _F, _F]),
    "orc_field_remove": (C.c_int, [_P, C.c_uint32, C.c_float, C.c_float]),
    "orc_field_lazy_update": (None, [_P]),
    "orc_field_query": (C.c_int64, [_P, C.c_int, C.c_float, C.c_float, C.c_float, _U32, _F,
                                    C.c_size_t]),
    "orc_field_num_at": (C.c_int64, [_P, C.c_float, C.c_float]),
    "orc_field_empty_bags": (C.c_size_t, [_P, _F, C.c_size_t]),
    "orc_field_iter": (C.c_size_t, [_P, C.c_int, _U32, _F, _U32, C.c_size_t]),
    "orc_neighbor_lists": (C.c_int64, [_P, C.c_int, C.c_float, C.c_size_t, _F, _U32, _U32,
                                       C.c_size_t]),
    "orc_neighbor_digest": (None, [_P, C.c_int, C.c_float, C.c_size_t, _F, _U32, _U32]),
    "orc_flock_run": (C.c_int, [_P, C.POINTER(Params), C.c_uint64, C.c_uint32]),
    "orc_simulate_timed_threads": (C.c_double, [C.c_float, C.c_float, C.c_float, C.POINTER(Params),
                                                 C.c_size_t, _U32, _F, _F, C.c_uint32, C.c_uint32,
                                                 C.POINTER(_P)]),
    "orc_flock_compute": (C.c_int, [_P, C.POINTER(Params), C.c_uint64]),
    "orc_bird_step": (None, [_P, C.POINTER(Params), C.c_uint64, C.c_uint32, _F, _F]),
    "orc_flock_compute_agents": (C.c_int, [_P, C.POINTER(Params), C.c_uint64, C.c_size_t, _U32,
                                           _F]),
    "orc_field_remove_ids": (C.c_size_t, [_P, C.c_size_t, _U32]),
    "orc_flock_step_fp64": (C.c_size_t, [_P, C.POINTER(Params), C.c_uint64, _U32, _D,
                                         C.c_size_t]),
    "orc_simulate_timed": (C.c_double, [C.c_float, C.c_float, C.c_float, C.POINTER(Params),
                                        C.c_size_t, _U32, _F, _F, C.c_uint32, C.POINTER(_P)]),
    "orc_simulate_timed_warm": (C.c_double, [C.c_float, C.c_float, C.c_float, C.POINTER(Params),
                                             C.c_size_t, _U32, _F, _F, C.c_uint32, C.c_uint32,
                                             C.POINTER(_P)]),
    "orc_simulate_timed_threads_warm": (C.c_double, [C.c_float, C.c_float, C.c_float,
                                                     C.POINTER(Params), C.c_size_t, _U32, _F, _F,
                                                     C.c_uint32, C.c_uint32, C.c_uint32,
                                                     C.POINTER(_P)]),
    "orc_gen_uniform": (C.c_int, [C.c_size_t, C.c_float, C.c_float, C.c_uint64, C.c_float, _U32,
                                  _F, _F]),
    "orc_gen_clustered": (C.c_int, [C.c_size_t, C.c_float, C.c_float, C.c_uint32, C.c_float,
                                    C.c_float, C.c_uint64, _U32, _F, _F]),
}
for _n, (_r, _a) in _SIGS.items():
    _fn = getattr(lib, _n)
    _fn.restype = _r
    _fn.argtypes = _a


def _f(a):
    return a.ctypes.data_as(_F)


def _u(a):
    return a.ctypes.data_as(_U32)


def params(cohesion=1.0, avoidance=1.0, consistency=1.0, randomness=1.0, momentum=1.0,
           jump=0.7, radius=10.0, query_mode=0, seed=0) -> Params:
    return Params(cohesion, avoidance, consistency, randomness, momentum, jump, radius,
                  query_mode, seed)


def params_from(fp) -> Params:
    """From a krabmaga_gb300.FlockParams-like object."""
    return Params(fp.cohesion, fp.avoidance, fp.consistency, fp.randomness, fp.momentum,
                  fp.jump, fp.neighbor_radius, fp.query_mode, fp.seed)


def gen_uniform(n, w, h, seed, heading_scale=1.0):
    """The uniform workload flock (workload_gen.cpp): (ids, xy[n,2], dxy[n,2])."""
    ids = np.zeros(n, np.uint32)
    xy = np.zeros((n, 2), np.float32)
    dxy = np.zeros((n, 2), np.float32)
    if lib.orc_gen_uniform(n, w, h, seed, heading_scale, _u(ids), _f(xy), _f(dxy)) != 0:
        raise ValueError("bad workload arguments")
    return ids, xy, dxy


def gen_clustered(n, w, h, nclusters, sigma, angle_sigma, seed):
    """The clustered workload flock (workload_gen.cpp): (ids, xy[n,2], dxy[n,2])."""
    ids = np.zeros(n, np.uint32)
    xy = np.zeros((n, 2), np.float32)
    dxy = np.zeros((n, 2), np.float32)
    if lib.orc_gen_clustered(n, w, h, nclusters, sigma, angle_sigma, seed, _u(ids), _f(xy),
                             _f(dxy)) != 0:
        raise ValueError("bad workload arguments")
    return ids, xy, dxy


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib.orc_philox4x32_10(_u(c), _u(k), _u(o))
    return o


class OracleField:
    """The oracle's Field2D (field_2d.rs:267-1014, f32-faithful)."""

    def __init__(self, w, h, d, toroidal=True, cell_wrap=0):
        """cell_wrap = 1: the true-torus query range (wraps instead of clamping)."""
        self.h = lib.orc_field_new(w, h, d, 1 if toroidal else 0)
        if cell_wrap:
            lib.orc_field_set_cell_wrap(self.h, 1)
        dims = (C.c_int32 * 4)()
        lib.orc_field_dims(self.h, dims)
        self.dw, self.dh, self.max_x, self.max_y = (int(v) for v in dims)

    def __del__(self):
        if getattr(self, "h", None):
            lib.orc_field_free(self.h)
            self.h = None

    @property
    def nagents(self):
        return int(lib.orc_field_nagents(self.h))

    def set(self, id, x, y, dx=0.0, dy=0.0, lx=None, ly=None):
        lx = x if lx is None else lx
        ly = y if ly is None else ly
        return lib.orc_field_set(self.h, id, x, y, dx, dy, lx, ly)

    def set_many(self, ids, xy, dxy):
        ids = np.ascontiguousarray(ids, np.uint32)
        xy = np.ascontiguousarray(xy, np.float32)
        dxy = np.ascontiguousarray(dxy, np.float32)
        return lib.orc_field_set_many(self.h, len(ids), _u(ids), _f(xy), _f(dxy))

    def remove(self, id, lx, ly):
        return lib.orc_field_remove(self.h, id, lx, ly)

    def lazy_update(self):
        lib.orc_field_lazy_update(self.h)

    def query(self, kind, x, y, dist=0.0):
        """kind 0 relax, 1 exact, 2 get_objects, 3 get_objects_unbuffered -> (ids, states)."""
        n = lib.orc_field_query(self.h, kind, x, y, dist, None, None, 0)
        if n < 0:
            raise IndexError("reference panics: location outside the bag matrix")
        ids = np.zeros(max(n, 1), np.uint32)
        st = np.zeros((max(n, 1), 4), np.float32)
        lib.orc_field_query(self.h, kind, x, y, dist, _u(ids), _f(st), n)
        return ids[:n], st[:n]

    def num_at(self, x, y):
        return int(lib.orc_field_num_at(self.h, x, y))

    def empty_bags(self):
        n = lib.orc_field_empty_bags(self.h, None, 0)
        xy = np.zeros((max(n, 1), 2), np.float32)
        lib.orc_field_empty_bags(self.h, _f(xy), n)
        return xy[:n]

    def iter(self, buffered=1):
        n = lib.orc_field_iter(self.h, buffered, None, None, None, 0)
        ids = np.zeros(max(n, 1), np.uint32)
        st = np.zeros((max(n, 1), 4), np.float32)
        cells = np.zeros(max(n, 1), np.uint32)
        lib.orc_field_iter(self.h, buffered, _u(ids), _f(st), _u(cells), n)
        return ids[:n], st[:n], cells[:n]

    def neighbor_lists(self, kind, dist, qxy):
        q = np.ascontiguousarray(qxy, np.float32).reshape(-1, 2)
        counts = np.zeros(max(len(q), 1), np.uint32)
        cap = 1 << 16
        while True:
            ids = np.zeros(cap, np.uint32)
            tot = lib.orc_neighbor_lists(self.h, kind, dist, len(q), _f(q), _u(counts), _u(ids),
                                         cap)
            if tot >= 0:
                return counts[: len(q)], ids[:tot]
            cap *= 4

    def neighbor_digest(self, kind, dist, qxy):
        q = np.ascontiguousarray(qxy, np.float32).reshape(-1, 2)
        counts = np.zeros(max(len(q), 1), np.uint32)
        dig = np.zeros(max(len(q), 1), np.uint32)
        lib.orc_neighbor_digest(self.h, kind, dist, len(q), _f(q), _u(counts), _u(dig))
        return counts[: len(q)], dig[: len(q)]

    def flock_run(self, p: Params, first_step, nsteps):
        r = lib.orc_flock_run(self.h, C.byref(p), first_step, nsteps)
        if r != 0:
            raise IndexError("reference panics during the step")

    def flock_compute(self, p: Params, step):
        """The agent pass only (every bird into the write buffer), no lazy_update."""
        if lib.orc_flock_compute(self.h, C.byref(p), step) != 0:
            raise IndexError("reference panics during the step")

    def bird_step(self, p: Params, step, id, state4):
        """Bird::step of one caller-held agent against the read buffer; its next
        {x, y, dx, dy} (nothing written)."""
        i4 = np.ascontiguousarray(state4, np.float32).reshape(4)
        o4 = np.zeros(4, np.float32)
        lib.orc_bird_step(self.h, C.byref(p), step, id, _f(i4), _f(o4))
        return o4

    def flock_compute_agents(self, p: Params, step, ids, states):
        ids = np.ascontiguousarray(ids, np.uint32)
        st = np.ascontiguousarray(states, np.float32).reshape(-1, 4)
        if lib.orc_flock_compute_agents(self.h, C.byref(p), step, len(ids), _u(ids), _f(st)) != 0:
            raise IndexError("reference panics during the step")

    def remove_ids(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        return int(lib.orc_field_remove_ids(self.h, len(ids), _u(ids)))

    def flock_step_fp64(self, p: Params, step):
        n = self.iter(1)[0].shape[0]
        ids = np.zeros(max(n, 1), np.uint32)
        out = np.zeros((max(n, 1), 4), np.float64)
        lib.orc_flock_step_fp64(self.h, C.byref(p), step, _u(ids),
                                out.ctypes.data_as(_D), n)
        return ids[:n], out[:n]


def simulate_timed_threads(w, h, d, p: Params, ids, xy, dxy, nsteps, threads, keep_field=False,
                           warmup=0):
    """The same run with the agent pass on `threads` host threads (results
    equal to the sequential run); returns (seconds, OracleField or None).
    warmup: untimed steps before the nsteps timed ones."""
    ids = np.ascontiguousarray(ids, np.uint32)
    xy = np.ascontiguousarray(xy, np.float32)
    dxy = np.ascontiguousarray(dxy, np.float32)
    out = C.c_void_p()
    secs = lib.orc_simulate_timed_threads_warm(w, h, d, C.byref(p), len(ids), _u(ids), _f(xy),
                                               _f(dxy), warmup, nsteps, threads,
                                               C.byref(out) if keep_field else None)
    f = None
    if keep_field:
        f = OracleField.__new__(OracleField)
        f.h = out.value
        dims = (C.c_int32 * 4)()
        lib.orc_field_dims(f.h, dims)
        f.dw, f.dh, f.max_x, f.max_y = (int(v) for v in dims)
    return secs, f


def simulate_timed(w, h, d, p: Params, ids, xy, dxy, nsteps, keep_field=False, warmup=0):
    """Reference-equivalent timed run (priority-queue schedule); returns
    (seconds in the step loop, OracleField or None).  warmup: untimed steps
    (0 .. warmup-1) before the nsteps timed ones."""
    ids = np.ascontiguousarray(ids, np.uint32)
    xy = np.ascontiguousarray(xy, np.float32)
    dxy = np.ascontiguousarray(dxy, np.float32)
    out = C.c_void_p()
    secs = lib.orc_simulate_timed_warm(w, h, d, C.byref(p), len(ids), _u(ids), _f(xy), _f(dxy),
                                       warmup, nsteps, C.byref(out) if keep_field else None)
    f = None
    if keep_field:
        f = OracleField.__new__(OracleField)
        f.h = out.value
        dims = (C.c_int32 * 4)()
        lib.orc_field_dims(f.h, dims)
        f.dw, f.dh, f.max_x, f.max_y = (int(v) for v in dims)
    return secs, f
