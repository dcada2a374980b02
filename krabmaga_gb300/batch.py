"""Batched replicas: many independent Flockers simulations in the same launches.

The GPU form of explore_parallel! (src/explore/model_exploration.rs:354-432),
which runs one simulate_explore! (lines 160-190) per configuration x
repetition on rayon threads: here every replica lives in one packed device
field and all of them advance together.  The default step path runs the
force, offsets and rebin kernels once per step over all replicas (each block
belongs to one replica); the tiled paths (set_step_options(2) or (1)) take
``steps_per_launch`` / ``graph_launches`` for their launch grouping.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L
from .model import FlockParams, gen_uniform


@dataclass
class Replica:
    """One simulation: torus side, discretization, parameters, initial flock."""

    width: float
    height: float
    discretization: float
    params: FlockParams
    state: Tuple[np.ndarray, np.ndarray, np.ndarray]  # ids, xy[n,2], dxy[n,2]
    toroidal: bool = True
    cell_wrap: int = L.KB_CELL_WRAP_CLAMP

    @property
    def n(self) -> int:
        return len(self.state[0])


def _fill_desc(d: L.ReplicaDesc, r: Replica) -> None:
    d.width, d.height, d.discretization = r.width, r.height, r.discretization
    d.toroidal = 1 if r.toroidal else 0
    d.cell_wrap = r.cell_wrap
    d.nboids = r.n
    d.params = r.params.to_c()


class Batch:
    def __init__(self, replicas: Sequence[Replica], device: int = 0):
        descs = (L.ReplicaDesc * len(replicas))()
        for d, r in zip(descs, replicas):
            _fill_desc(d, r)
        h = C.c_void_p()
        L.call("kb_batch_create", C.c_int32(device), C.c_uint32(len(replicas)), descs, C.byref(h))
        self._h = h
        self.nrep = len(replicas)
        self.sizes = [r.n for r in replicas]
        for i, r in enumerate(replicas):
            ids = np.ascontiguousarray(r.state[0], np.uint32)
            xy = np.ascontiguousarray(r.state[1], np.float32)
            dxy = np.ascontiguousarray(r.state[2], np.float32)
            L.call("kb_batch_set_replica", self._h, C.c_uint32(i), C.c_size_t(len(ids)),
                   L.uptr(ids), L.fptr(xy), L.fptr(dxy))
        L.call("kb_batch_commit", self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            L.lib.kb_batch_destroy(self._h)
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

    @property
    def handle(self):
        return self._h

    def cuda_stream(self) -> int:
        s = C.c_void_p()
        L.call("kb_batch_cuda_stream", self._h, C.byref(s))
        return s.value or 0

    def set_step_options(self, mode=0, tile_tx: int = 0, tile_ty: int = 0) -> None:
        """Step path: 0 separate kernels (default), 2 tiled split, 1 persistent."""
        mode = {True: 2, False: 0}.get(mode, mode) if isinstance(mode, bool) else int(mode)
        L.call("kb_batch_set_step_options", self._h, C.c_int32(mode), C.c_int32(tile_tx),
               C.c_int32(tile_ty))

    def step(self, first_step: int, nsteps: int, steps_per_launch: int = 0,
             graph_launches: int = 0) -> None:
        L.call("kb_batch_step", self._h, C.c_uint64(first_step), C.c_uint32(nsteps),
               C.c_uint32(steps_per_launch), C.c_uint32(graph_launches))

    def synchronize(self) -> None:
        L.call("kb_batch_synchronize", self._h)

    def moments(self) -> np.ndarray:
        """[nrep, 4]: boids, sum dx, sum dy, sum |(dx, dy)| of each replica's
        headings, reduced on the device in double."""
        out = np.zeros((len(self.sizes), 4), np.float64)
        L.call("kb_batch_moments", self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def add_replica(self, replica: Replica, origin_step: int) -> int:
        """Append a replica to the running batch; its step 0 is the batch's
        step ``origin_step``.  Returns its index."""
        d = L.ReplicaDesc()
        _fill_desc(d, replica)
        ids = np.ascontiguousarray(replica.state[0], np.uint32)
        xy = np.ascontiguousarray(replica.state[1], np.float32)
        dxy = np.ascontiguousarray(replica.state[2], np.float32)
        idx = C.c_uint32()
        L.call("kb_batch_add_replica", self._h, C.byref(d), L.uptr(ids), L.fptr(xy), L.fptr(dxy),
               C.c_uint64(origin_step), C.byref(idx))
        self.sizes.append(replica.n)
        self.nrep += 1
        return int(idx.value)

    def remove_replica(self, r: int) -> None:
        """Drop replica r; later replicas move down one index."""
        L.call("kb_batch_remove_replica", self._h, C.c_uint32(r))
        del self.sizes[r]
        self.nrep -= 1

    def get_replica(self, r: int):
        n = C.c_size_t()
        cap = self.sizes[r]
        ids = np.zeros(max(cap, 1), np.uint32)
        st = np.zeros((max(cap, 1), 4), np.float32)
        L.call("kb_batch_get_replica", self._h, C.c_uint32(r), L.uptr(ids), L.fptr(st),
               C.c_size_t(cap), C.byref(n))
        return ids[: n.value], st[: n.value]

    def autotune(self, first_step: int, steps_per_trial: int = 5, candidates=None):
        """Pick the fastest launch shape by timing real steps.  Tiled step
        modes (1, 2): the tile shape, candidates (tx, ty), returns (tx, ty,
        steps consumed, ms per step).  Separate kernels (modes 0, 3): the force
        pass's threads per block over the packed replicas, candidates
        (threads, 1) with threads 128, 256 or 512 and one replica per block,
        returns (threads, 1, steps consumed, ms per step)."""
        cand = None
        nc = 0
        if candidates:
            flat = [v for pair in candidates for v in pair]
            cand = (C.c_int32 * len(flat))(*flat)
            nc = len(candidates)
        best = (C.c_int32 * 3)()
        ms = C.c_float()
        L.call("kb_batch_autotune", self._h, C.c_uint64(first_step), C.c_uint32(steps_per_trial),
               cand, C.c_int32(nc), best, C.byref(ms))
        return int(best[0]), int(best[1]), int(best[2]), float(ms.value)

    def step_stats(self) -> dict:
        v = np.zeros(4, np.uint32)
        L.call("kb_batch_step_stats", self._h, L.uptr(v))
        return {"overflow_tiles": int(v[0]), "tiles": int(v[1]), "ctas": int(v[2]),
                "tile": (int(v[3]) >> 16, int(v[3]) & 0xFFFF)}


def sweep_replicas(nrep: int, n_min: int = 1024, n_max: int = 65536, density: float = 0.025,
                   arith: int = L.KB_ARITH_FAST, query_mode: int = L.KB_QUERY_RELAX,
                   table_seed: int = 2024) -> List[Replica]:
    """The exploration-sweep workload: replica i has N_i log-uniform in
    [n_min, n_max] at the given density (square torus), weights U[0.5, 1.5],
    jump U[0.3, 1.0], radius U[5, 15], discretization radius/1.5 (a 3x3 bag
    stencil, as the reference's 10 / (10/1.5)), jitter seed i, and a uniform
    initial flock from Philox(i)."""
    rng = np.random.default_rng(table_seed)
    out = []
    for i in range(nrep):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        side = float(np.float32(np.sqrt(n / density)))
        w = rng.uniform(0.5, 1.5, 5)
        jump = float(rng.uniform(0.3, 1.0))
        radius = float(np.float32(rng.uniform(5.0, 15.0)))
        d = float(np.float32(radius) / np.float32(1.5))
        p = FlockParams(cohesion=float(w[0]), avoidance=float(w[1]), consistency=float(w[2]),
                        randomness=float(w[3]), momentum=float(w[4]), jump=jump,
                        neighbor_radius=radius, query_mode=query_mode, arith=arith, seed=i)
        out.append(Replica(side, side, d, p, gen_uniform(n, side, side, i, 1.0)))
    return out
