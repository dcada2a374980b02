"""Field2D over the GPU C ABI, with the reference's method names.

Mirrors ``engine::fields::field_2d::Field2D`` (src/engine/fields/field_2d.rs,
sequential build, lines 267-1014) for objects of the Flockers ``Bird`` shape
``{id, pos, last_d}`` (tests/model/flockers/bird.rs:20-25).  Reads of the read
buffer, writes to the write buffer and the ``lazy_update`` swap keep the
reference's double-buffer semantics; every query runs as a kernel on the
field's device.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Callable, List, Optional, Tuple

import numpy as np

from . import _lib as L


@dataclass(frozen=True)
class Real2D:
    """src/engine/location.rs:17-22 (2 x f32)."""

    x: float
    y: float

    def as_f32(self) -> np.ndarray:
        return np.array([self.x, self.y], dtype=np.float32)


@dataclass(frozen=True)
class Bird:
    """tests/model/flockers/bird.rs:20-25; equality and hashing by id only
    (bird.rs:157-174)."""

    id: int
    pos: Real2D
    last_d: Real2D = Real2D(0.0, 0.0)

    def __eq__(self, other) -> bool:
        return isinstance(other, Bird) and other.id == self.id

    def __hash__(self) -> int:
        return hash(self.id)


def _birds(ids: np.ndarray, st: np.ndarray) -> List[Bird]:
    return [
        Bird(int(i), Real2D(float(s[0]), float(s[1])), Real2D(float(s[2]), float(s[3])))
        for i, s in zip(ids, st)
    ]


class Field2D:
    """Field2D::new(w, h, d, toroidal) -- field_2d.rs:304-322."""

    def __init__(self, w: float, h: float, d: float, toroidal: bool, device: int = 0,
                 capacity_hint: int = 0, cell_wrap: int = L.KB_CELL_WRAP_CLAMP):
        """cell_wrap (toroidal fields): KB_CELL_WRAP_CLAMP, the reference's
        clamped query range, or KB_CELL_WRAP_TORUS, a range that wraps."""
        desc = L.FieldDesc(w, h, d, 1 if toroidal else 0, device, capacity_hint, cell_wrap)
        h_ = C.c_void_p()
        L.call("kb_field_create", C.byref(desc), C.byref(h_))
        self._h = h_
        self.device = int(device)
        self.width = float(np.float32(w))
        self.height = float(np.float32(h))
        self.discretization = float(np.float32(d))
        self.toroidal = bool(toroidal)
        dims = (C.c_int32 * 4)()
        L.call("kb_field_dims", self._h, dims)
        self.dw, self.dh, self.max_x, self.max_y = (int(v) for v in dims)

    # -- lifetime ------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            L.lib.kb_field_destroy(self._h)
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
        L.call("kb_field_cuda_stream", self._h, C.byref(s))
        return s.value or 0

    # -- writes (write buffer) -----------------------------------------
    def set_object_location(self, obj: Bird, loc: Real2D) -> None:
        """field_2d.rs:838-846"""
        pos = obj.pos.as_f32()
        ld = obj.last_d.as_f32()
        lc = loc.as_f32()
        L.call("kb_field_set_object_location", self._h, C.c_uint32(obj.id), L.fptr(pos),
               L.fptr(ld), L.fptr(lc))

    def set_locations(self, ids: np.ndarray, xy: np.ndarray, dxy: np.ndarray) -> None:
        """Bulk set_object_location, each object at its own position."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        xy = np.ascontiguousarray(xy, dtype=np.float32).reshape(-1, 2)
        dxy = np.ascontiguousarray(dxy, dtype=np.float32).reshape(-1, 2)
        assert len(ids) == len(xy) == len(dxy)
        L.call("kb_field_set_locations", self._h, C.c_size_t(len(ids)), L.uptr(ids),
               L.fptr(xy), L.fptr(dxy))

    def remove_object_location(self, obj: Bird, loc: Real2D) -> None:
        """field_2d.rs:885-898"""
        L.call("kb_field_remove_object_location", self._h, C.c_uint32(obj.id),
               L.fptr(loc.as_f32()))

    def get_locations(self, ids, buffered: bool = True):
        """Lookups by id in the read buffer (or, buffered=False, the write
        buffer): (found bool[n], states f32[n, 4]); the first stored object
        when several share an id."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32).reshape(-1)
        st = np.zeros((max(len(ids), 1), 4), np.float32)
        found = np.zeros(max(len(ids), 1), np.int32)
        L.call("kb_field_get_locations", self._h, C.c_int32(1 if buffered else 0),
               C.c_size_t(len(ids)), L.uptr(ids), L.fptr(st),
               found.ctypes.data_as(C.POINTER(C.c_int32)))
        return found[: len(ids)].astype(bool), st[: len(ids)]

    def get(self, obj: Bird) -> Optional[Bird]:
        """Field2D::get (parallel build, field_2d.rs:165-170): the stored copy
        of the object (read buffer), or None."""
        found, st = self.get_locations([obj.id], True)
        return _birds([obj.id], st)[0] if found[0] else None

    def get_location(self, obj: Bird) -> Optional[Real2D]:
        """Field2D::get_location (parallel build, field_2d.rs:189-191)."""
        found, st = self.get_locations([obj.id], True)
        return Real2D(float(st[0, 0]), float(st[0, 1])) if found[0] else None

    def get_unbuffered(self, obj: Bird) -> Optional[Bird]:
        """Field2D::get_unbuffered (parallel build, field_2d.rs:202-217): the
        copy in the write buffer, or None."""
        found, st = self.get_locations([obj.id], False)
        return _birds([obj.id], st)[0] if found[0] else None

    def get_location_unbuffered(self, obj: Bird) -> Optional[Real2D]:
        """Field2D::get_location_unbuffered (parallel build, field_2d.rs:194-197)."""
        found, st = self.get_locations([obj.id], False)
        return Real2D(float(st[0, 0]), float(st[0, 1])) if found[0] else None

    def remove_ids(self, ids) -> int:
        """Remove every write-buffer object with one of these ids (each one as
        remove_object_location at its write location); returns the count."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32).reshape(-1)
        n = C.c_size_t()
        L.call("kb_field_remove_ids", self._h, C.c_size_t(len(ids)), L.uptr(ids), C.byref(n))
        return n.value

    def flock_compute(self, params, step: int) -> None:
        """Bird::step of every agent of the read buffer into the write buffer
        (the agent pass of one Schedule::step)."""
        L.call("kb_flock_compute", self._h, C.byref(params.to_c()), C.c_uint64(step))

    def flock_step(self, params, first_step: int, nsteps: int) -> None:
        """nsteps whole steps (agent pass + lazy_update each), numbered from
        first_step; runs of steps replay CUDA graphs."""
        L.call("kb_flock_step", self._h, C.byref(params.to_c()), C.c_uint64(first_step),
               C.c_uint32(nsteps))

    def flock_compute_agents(self, params, step: int, ids, states) -> None:
        """Bird::step of caller-held agents (states: n x {x, y, dx, dy})
        against the read buffer, appended to the write buffer in order."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32).reshape(-1)
        st = np.ascontiguousarray(states, dtype=np.float32).reshape(-1, 4)
        assert len(ids) == len(st)
        L.call("kb_flock_compute_agents", self._h, C.byref(params.to_c()), C.c_uint64(step),
               C.c_size_t(len(ids)), L.uptr(ids), L.fptr(st))

    # ---- device-resident records: torch CUDA tensors on the field's GPU,
    # ids as int32 holding the u32 bits, records float32 [n, 4] {x, y, dx, dy}
    @staticmethod
    def _dev_arg(t, dtype, what: str):
        import torch

        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
            raise TypeError(f"{what}: a contiguous CUDA tensor of {dtype} is expected")
        # the library reads the tensor on its own stream: finish torch's work first
        torch.cuda.current_stream(t.device).synchronize()
        return C.c_void_p(t.data_ptr())

    def read_buffer_device(self):
        """(ids int32 [n], states float32 [n, 4]): a device copy of the read
        buffer in its order (bags ascending, insertion order in a bag)."""
        import torch

        n = self.num_objects()
        dev = torch.device("cuda", self.device)
        ids = torch.empty(n, dtype=torch.int32, device=dev)
        st = torch.empty((n, 4), dtype=torch.float32, device=dev)
        got = C.c_size_t()
        L.call("kb_field_copy_read_buffer", self._h, self._dev_arg(st, torch.float32, "states"),
               self._dev_arg(ids, torch.int32, "ids"), C.c_size_t(n), C.byref(got))
        return ids, st

    def set_states_device(self, ids, states) -> None:
        """set_locations for records held on the device (appended in order)."""
        import torch

        assert ids.shape[0] == states.shape[0] and states.shape[1:] == (4,)
        L.call("kb_field_set_states_device", self._h, C.c_size_t(ids.shape[0]),
               self._dev_arg(ids, torch.int32, "ids"), self._dev_arg(states, torch.float32, "states"))

    def next_states_device(self, params, step: int, ids, states):
        """Bird::step of device-held agents against the read buffer; returns
        their next states (float32 [n, 4]); the write buffer is untouched."""
        import torch

        assert ids.shape[0] == states.shape[0] and states.shape[1:] == (4,)
        out = torch.empty_like(states)
        L.call("kb_flock_next_states_device", self._h, C.byref(params.to_c()), C.c_uint64(step),
               C.c_size_t(ids.shape[0]), self._dev_arg(ids, torch.int32, "ids"),
               self._dev_arg(states, torch.float32, "states"), self._dev_arg(out, torch.float32, "out"))
        return out

    def lazy_update(self) -> None:
        """Field::lazy_update -- field_2d.rs:905-921"""
        L.call("kb_field_lazy_update", self._h)

    @property
    def nagents(self) -> int:
        """field_2d.rs:276 (counted until the first lazy_update)."""
        n = C.c_size_t()
        L.call("kb_field_num_agents", self._h, C.byref(n))
        return n.value

    def num_objects(self) -> int:
        n = C.c_size_t()
        L.call("kb_field_num_objects", self._h, C.byref(n))
        return n.value

    # -- reads ----------------------------------------------------------
    def _query(self, fn: str, loc: Real2D, dist: float) -> List[Bird]:
        lc = loc.as_f32()
        n = C.c_size_t()
        L.call(fn, self._h, L.fptr(lc), C.c_float(dist), None, None, C.c_size_t(0), C.byref(n))
        cnt = n.value
        ids = np.zeros(max(cnt, 1), np.uint32)
        st = np.zeros((max(cnt, 1), 4), np.float32)
        L.call(fn, self._h, L.fptr(lc), C.c_float(dist), L.uptr(ids), L.fptr(st),
               C.c_size_t(cnt), C.byref(n))
        return _birds(ids[:cnt], st[:cnt])

    def get_neighbors_within_relax_distance(self, loc: Real2D, dist: float) -> List[Bird]:
        """field_2d.rs:472-516"""
        return self._query("kb_field_get_neighbors_within_relax_distance", loc, dist)

    def get_neighbors_within_distance(self, loc: Real2D, dist: float) -> List[Bird]:
        """field_2d.rs:386-440"""
        return self._query("kb_field_get_neighbors_within_distance", loc, dist)

    def _bag(self, fn: str, loc: Real2D) -> List[Bird]:
        lc = loc.as_f32()
        n = C.c_size_t()
        L.call(fn, self._h, L.fptr(lc), None, None, C.c_size_t(0), C.byref(n))
        cnt = n.value
        ids = np.zeros(max(cnt, 1), np.uint32)
        st = np.zeros((max(cnt, 1), 4), np.float32)
        L.call(fn, self._h, L.fptr(lc), L.uptr(ids), L.fptr(st), C.c_size_t(cnt), C.byref(n))
        return _birds(ids[:cnt], st[:cnt])

    def get_objects(self, loc: Real2D) -> List[Bird]:
        """field_2d.rs:544-549"""
        return self._bag("kb_field_get_objects", loc)

    def get_objects_unbuffered(self, loc: Real2D) -> List[Bird]:
        """field_2d.rs:577-582"""
        return self._bag("kb_field_get_objects_unbuffered", loc)

    def num_objects_at_location(self, loc: Real2D) -> int:
        """field_2d.rs:803-808"""
        n = C.c_size_t()
        L.call("kb_field_num_objects_at_location", self._h, L.fptr(loc.as_f32()), C.byref(n))
        return n.value

    def get_empty_bags(self) -> List[Real2D]:
        """field_2d.rs:727-739"""
        n = C.c_size_t()
        L.call("kb_field_get_empty_bags", self._h, None, C.c_size_t(0), C.byref(n))
        xy = np.zeros((max(n.value, 1), 2), np.float32)
        L.call("kb_field_get_empty_bags", self._h, L.fptr(xy), C.c_size_t(n.value), C.byref(n))
        return [Real2D(float(a), float(b)) for a, b in xy[: n.value]]

    def get_random_empty_bag(self, seed: int = 0) -> Optional[Real2D]:
        """field_2d.rs:764-772 (Philox(seed) instead of an unseeded rng)."""
        xy = np.zeros(2, np.float32)
        found = C.c_int32()
        L.call("kb_field_get_random_empty_bag", self._h, C.c_uint64(seed), L.fptr(xy),
               C.byref(found))
        return Real2D(float(xy[0]), float(xy[1])) if found.value else None

    def _iter(self, buffered: int) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = C.c_size_t()
        L.call("kb_field_iter_objects", self._h, C.c_int32(buffered), None, None, None,
               C.c_size_t(0), C.byref(n))
        cnt = n.value
        cxy = np.zeros((max(cnt, 1), 2), np.float32)
        ids = np.zeros(max(cnt, 1), np.uint32)
        st = np.zeros((max(cnt, 1), 4), np.float32)
        L.call("kb_field_iter_objects", self._h, C.c_int32(buffered), L.fptr(cxy), L.uptr(ids),
               L.fptr(st), C.c_size_t(cnt), C.byref(n))
        return cxy[:cnt], ids[:cnt], st[:cnt]

    def iter_objects(self, closure: Callable[[Real2D, Bird], None]) -> None:
        """field_2d.rs:619-640"""
        cxy, ids, st = self._iter(1)
        for c, b in zip(cxy, _birds(ids, st)):
            closure(Real2D(float(c[0]), float(c[1])), b)

    def iter_objects_unbuffered(self, closure: Callable[[Real2D, Bird], None]) -> None:
        """field_2d.rs:677-698"""
        cxy, ids, st = self._iter(0)
        for c, b in zip(cxy, _birds(ids, st)):
            closure(Real2D(float(c[0]), float(c[1])), b)

    # -- bulk state / parity support ---------------------------------
    def get_state(self) -> Tuple[np.ndarray, np.ndarray]:
        """Read buffer in stored order: (ids u32[n], states f32[n,4])."""
        n = C.c_size_t()
        L.call("kb_field_get_state", self._h, None, None, C.c_size_t(0), C.byref(n))
        cnt = n.value
        ids = np.zeros(max(cnt, 1), np.uint32)
        st = np.zeros((max(cnt, 1), 4), np.float32)
        L.call("kb_field_get_state", self._h, L.uptr(ids), L.fptr(st), C.c_size_t(cnt),
               C.byref(n))
        return ids[:cnt], st[:cnt]

    def neighbor_lists(self, kind: int, dist: float, qxy: np.ndarray):
        """Candidate id lists of many query points: (counts, packed ids)."""
        q = np.ascontiguousarray(qxy, dtype=np.float32).reshape(-1, 2)
        counts = np.zeros(max(len(q), 1), np.uint32)
        total = C.c_size_t()
        L.call("kb_field_neighbor_lists", self._h, C.c_int32(kind), C.c_float(dist),
               C.c_size_t(len(q)), L.fptr(q), L.uptr(counts), None, C.c_size_t(0),
               C.byref(total))
        ids = np.zeros(max(total.value, 1), np.uint32)
        L.call("kb_field_neighbor_lists", self._h, C.c_int32(kind), C.c_float(dist),
               C.c_size_t(len(q)), L.fptr(q), L.uptr(counts), L.uptr(ids),
               C.c_size_t(total.value), C.byref(total))
        return counts[: len(q)], ids[: total.value]

    def neighbor_digest(self, kind: int, dist: float, qxy: np.ndarray):
        q = np.ascontiguousarray(qxy, dtype=np.float32).reshape(-1, 2)
        counts = np.zeros(max(len(q), 1), np.uint32)
        dig = np.zeros(max(len(q), 1), np.uint32)
        L.call("kb_field_neighbor_digest", self._h, C.c_int32(kind), C.c_float(dist),
               C.c_size_t(len(q)), L.fptr(q), L.uptr(counts), L.uptr(dig))
        return counts[: len(q)], dig[: len(q)]

    def set_step_options(self, mode=0, tile_tx: int = 0, tile_ty: int = 0) -> None:
        """Step path: 0 separate kernels (default; runs of steps on fields of
        at most 4096 boids take one thread-block cluster), 3 separate kernels
        whatever the size, 2 tiled split,
        1 persistent (True/False mean 2/0); tile shape in bags (0 = automatic)."""
        mode = {True: 2, False: 0}.get(mode, mode) if isinstance(mode, bool) else int(mode)
        L.call("kb_field_set_step_options", self._h, C.c_int32(mode), C.c_int32(tile_tx),
               C.c_int32(tile_ty))

    def set_dense_mode(self, mode: int = L.KB_DENSE_AUTO) -> None:
        """Candidate-list walk: KB_DENSE_AUTO (by bag occupancy), _OFF (one flat
        list, 32-bag rebin segments), _ON (per-run walk, 8-bag segments)."""
        L.call("kb_field_set_dense_mode", self._h, C.c_int32(mode))

    def step_path(self) -> int:
        """KB_PATH_* of the next kb_flock_step."""
        v = C.c_int32()
        L.call("kb_field_step_path", self._h, C.byref(v))
        return v.value

    def dense_active(self) -> bool:
        v = C.c_int32()
        L.call("kb_field_dense_active", self._h, C.byref(v))
        return bool(v.value)

    def autotune(self, params, first_step: int, steps_per_trial: int = 5, candidates=None):
        """Pick the fastest fused tile shape by timing real steps; returns
        (tx, ty, steps consumed, ms per step)."""
        cand = None
        nc = 0
        if candidates:
            flat = [v for pair in candidates for v in pair]
            cand = (C.c_int32 * len(flat))(*flat)
            nc = len(candidates)
        best = (C.c_int32 * 3)()
        ms = C.c_float()
        L.call("kb_field_autotune", self._h, C.byref(params.to_c()), C.c_uint64(first_step),
               C.c_uint32(steps_per_trial), cand, C.c_int32(nc), best, C.byref(ms))
        return int(best[0]), int(best[1]), int(best[2]), float(ms.value)

    def moments(self) -> np.ndarray:
        """[4]: boids, sum dx, sum dy, sum |(dx, dy)| of the read buffer's
        headings, reduced on the device in double."""
        out = np.zeros(4, np.float64)
        L.call("kb_field_moments", self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def set_kernel_timing(self, enable: bool) -> None:
        """Record CUDA events around the force / scan / rebin launches of
        ungraphed separate-kernel steps (kb_flock_step calls of < 4 steps)."""
        L.call("kb_field_set_kernel_timing", self._h, C.c_int32(1 if enable else 0))

    def kernel_times(self) -> Tuple[Tuple[float, float, float], int]:
        """((force_ms, scan_ms, rebin_ms) summed, steps timed) since the last call."""
        ms = (C.c_double * 3)()
        n = C.c_uint64()
        L.call("kb_field_kernel_times", self._h, ms, C.byref(n))
        return (ms[0], ms[1], ms[2]), int(n.value)

    def step_stats(self) -> dict:
        v = np.zeros(4, np.uint32)
        L.call("kb_field_step_stats", self._h, L.uptr(v))
        return {"overflow_tiles": int(v[0]), "tiles": int(v[1]), "ctas": int(v[2]),
                "tile": (int(v[3]) >> 16, int(v[3]) & 0xFFFF)}

    def device_flags(self, clear: bool = False) -> int:
        v = C.c_uint32()
        L.call("kb_field_device_flags", self._h, C.byref(v), C.c_int32(1 if clear else 0))
        return v.value

    def set_wait_test(self, spin_limit: int = 0, withhold: int = 0, index: int = 0) -> None:
        """Bounded device waits: iterations before a wait gives up (0: the
        kernels' defaults), and the test hook KB_WITHHOLD_* that makes the
        look-back tile or persistent block `index` withhold its signal."""
        L.call("kb_field_set_wait_test", self._h, C.c_uint32(spin_limit), C.c_int32(withhold),
               C.c_uint32(index))

    def synchronize(self) -> None:
        L.call("kb_field_synchronize", self._h)
