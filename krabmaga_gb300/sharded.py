"""One Flockers field decomposed over ranks by column strips (one GPU each).

The reference's only domain-decomposed field is its MPI kd-tree field
(src/engine/fields/kdtree_mpi.rs): each process holds its region plus halo
copies of its neighbours' border objects (insert into the halo lists,
kdtree_mpi.rs:519-540), and after each step the processes exchange the
objects that moved or that the neighbours need (message_exchange,
kdtree_mpi.rs:705-795) before the next distributed relaxed query
(kdtree_mpi.rs:797-850).  Here the decomposition is by columns of the bag
matrix of one Field2D (bag index x*dh + y, field_2d.rs:508):

* rank r owns the boids whose bag column lies in [X0, X1) (an even split of
  the dw = max_x + 1 columns) and keeps, in a full-size local Field2D, the
  boids of its region: the owned columns plus `dd` halo columns on each side
  (the relaxed query's reach, field_2d.rs:488-500; the query is clamped at the
  torus seam, so no halo wraps);
* a step computes the next state of every owned boid against the local read
  buffer (kb_flock_compute_agents), then sends each owned boid to every other
  rank whose region holds its new column (halo updates and migrations, the
  seam wrap included), all as one exchange;
* the local read buffer of the next step is built from the owned and received
  boids inserted in their previous global order (bag, then place in the bag),
  the order in which the single field writes them (one set_object_location per
  bird in schedule order), so every local bag equals the single field's bag.

So the candidates of every owned boid, their order and the jitter keys
(seed, id, step) are those of the single field: the owned boids of all ranks
together equal the single field's state bit for bit, in either arithmetic.
The exchange goes through `torch.distributed` point-to-point messages (NCCL
between GPUs, gloo on host memory).  Boids carry their state through host
arrays between the local field and the exchange; a device-resident exchange
is not built.  Requires every strip to be at least dd + 2 columns wide, so
that a boid's new column is in the region of its owner's neighbours at most.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Tuple

import numpy as np

from . import _lib as L
from .field import Field2D
from .model import FlockParams


def geometry(w: float, d: float) -> Tuple[int, int, int]:
    """(max_x, dw, dh) of a square field: ceil(w/d) in f32 (field_2d.rs:304-322)."""
    max_x = int(np.ceil(np.float32(w) / np.float32(d)))
    return max_x, max_x + 1, max_x + 1


def discretize(v: np.ndarray, d: float) -> np.ndarray:
    """floor(fl(v / d)) as i32 (field_2d.rs:328-339), elementwise in f32."""
    q = np.floor(np.asarray(v, np.float32) / np.float32(d))
    return q.astype(np.int64)


def strips(dw: int, world: int) -> List[Tuple[int, int]]:
    """[X0, X1) bag columns owned by each rank."""
    return [(r * dw // world, (r + 1) * dw // world) for r in range(world)]


def query_reach(radius: float, d: float) -> int:
    """dd = floor(radius / d) in f32 (field_2d.rs:488); -1 for radius <= 0."""
    if radius <= 0:
        return -1
    return int(np.floor(np.float32(radius) / np.float32(d)))


class GpuStrip:
    """The local field of one rank on its GPU, through the C ABI."""

    def __init__(self, w: float, d: float, device: int, capacity: int):
        self.field = Field2D(w, w, d, True, device, capacity_hint=capacity)

    def state(self) -> Tuple[np.ndarray, np.ndarray]:
        return self.field.get_state()

    def next_states(self, params: FlockParams, step: int, ids: np.ndarray,
                    states: np.ndarray) -> np.ndarray:
        """Bird::step of the given read-buffer boids against the read buffer;
        nothing is left in the write buffer."""
        if len(ids) == 0:
            return np.zeros((0, 4), np.float32)
        self.field.flock_compute_agents(params, step, ids, states)
        found, nxt = self.field.get_locations(ids, buffered=False)
        self.field.remove_ids(ids)
        if not found.all():
            raise L.KbError(L.KB_ERR_STATE, "GpuStrip.next_states", "an agent's next state is missing")
        return nxt

    def replace(self, ids: np.ndarray, states: np.ndarray) -> None:
        """The read buffer becomes these boids, inserted in this order."""
        st = np.ascontiguousarray(states, np.float32).reshape(-1, 4)
        self.field.set_locations(ids, st[:, :2], st[:, 2:])
        self.field.lazy_update()

    def close(self) -> None:
        self.field.close()


class ShardedFlock:
    """A Flockers simulation on a w x w torus (bags of side d) split over the
    ranks of `group` by column strips.  `make_local(w, d, capacity)` builds the
    local field (GpuStrip on GPU `gpu` by default); `device` is where the
    exchange tensors live ("cpu" for gloo, "cuda" for NCCL: then GPU `gpu`)."""

    def __init__(self, w: float, d: float, params: FlockParams, ids: np.ndarray, xy: np.ndarray,
                 dxy: np.ndarray, group=None, make_local: Optional[Callable] = None,
                 device: str = "cpu", gpu: int = 0):
        import torch.distributed as dist

        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        import torch

        self.w, self.d, self.params = float(w), float(d), params
        # the exchange buffers: host memory for gloo, this rank's GPU for NCCL
        self.device = torch.device("cuda", gpu) if device == "cuda" else torch.device(device)
        self.max_x, self.dw, self.dh = geometry(w, d)
        self.dd = max(query_reach(params.neighbor_radius, d), 0)
        self.strips = strips(self.dw, self.world)
        if min(x1 - x0 for x0, x1 in self.strips) < self.dd + 2:
            raise ValueError("every strip needs at least dd + 2 columns")
        self.regions = [(max(0, x0 - self.dd), min(self.max_x, x1 - 1 + self.dd))
                        for x0, x1 in self.strips]
        ids = np.ascontiguousarray(ids, np.uint32)
        xy = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
        dxy = np.ascontiguousarray(dxy, np.float32).reshape(-1, 2)
        if make_local is None:
            self.local = GpuStrip(self.w, self.d, gpu, len(ids) // self.world + 1)
        else:
            self.local = make_local(self.w, self.d, len(ids) // self.world + 1)
        # the initial write order is the order of the arrays: keep it for the region
        lo, hi = self.regions[self.rank]
        col = discretize(xy[:, 0], self.d)
        keep = (col >= lo) & (col <= hi)
        self.local.replace(ids[keep], np.concatenate([xy, dxy], axis=1)[keep])

    # ------------------------------------------------------------------ step
    def _bags(self, st: np.ndarray) -> np.ndarray:
        return discretize(st[:, 0], self.d) * self.dh + discretize(st[:, 1], self.d)

    def step(self, step_no: int) -> None:
        ids, st = self.local.state()
        bag = self._bags(st)
        col = bag // self.dh
        x0, x1 = self.strips[self.rank]
        own = (col >= x0) & (col < x1)
        # the previous global write order of each boid: its bag, then its place in the bag
        first = np.searchsorted(bag, bag, side="left")
        place = np.arange(len(bag)) - first
        nxt = self.local.next_states(self.params, step_no, ids[own], st[own])
        rec = np.zeros((int(own.sum()), 8), np.int32)
        rec[:, 0] = ids[own].view(np.int32)
        rec[:, 1:5] = nxt.view(np.int32)
        rec[:, 5] = (bag[own] >> 31).astype(np.int32)
        rec[:, 6] = (bag[own] & 0x7FFFFFFF).astype(np.int32)
        rec[:, 7] = place[own].astype(np.int32)
        ncol = discretize(nxt[:, 0], self.d) if len(nxt) else np.zeros(0, np.int64)
        parts = []
        for r in range(self.world):
            lo, hi = self.regions[r]
            parts.append(rec[(ncol >= lo) & (ncol <= hi)])
        mine = self._exchange(parts)
        mine = mine[np.lexsort((mine[:, 7], mine[:, 6].astype(np.int64), mine[:, 5]))]
        self.local.replace(mine[:, 0].view(np.uint32), mine[:, 1:5].view(np.float32))

    def _exchange(self, parts: List[np.ndarray]) -> np.ndarray:
        """Send parts[r] to rank r (r != self.rank); returns own part plus what
        the others sent here."""
        import torch

        dist, me = self.dist, self.rank
        peers = [r for r in range(self.world) if r != me]
        sizes_out = {r: torch.tensor([len(parts[r])], dtype=torch.int64, device=self.device)
                     for r in peers}
        sizes_in = {r: torch.zeros(1, dtype=torch.int64, device=self.device) for r in peers}
        reqs = []
        for r in peers:
            reqs.append(dist.isend(sizes_out[r], r, group=self.group))
            reqs.append(dist.irecv(sizes_in[r], r, group=self.group))
        for q in reqs:
            q.wait()
        out = {r: torch.from_numpy(np.ascontiguousarray(parts[r])).to(self.device) for r in peers}
        inc = {r: torch.zeros((int(sizes_in[r].item()), 8), dtype=torch.int32, device=self.device)
               for r in peers}
        reqs = []
        for r in peers:
            if len(parts[r]):
                reqs.append(dist.isend(out[r], r, group=self.group))
            if inc[r].shape[0]:
                reqs.append(dist.irecv(inc[r], r, group=self.group))
        for q in reqs:
            q.wait()
        got = [parts[me]] + [inc[r].cpu().numpy() for r in peers]
        return np.concatenate(got, axis=0) if got else np.zeros((0, 8), np.int32)

    def run(self, first_step: int, nsteps: int) -> None:
        for k in range(nsteps):
            self.step(first_step + k)

    # ------------------------------------------------------------------ state
    def owned_state(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(ids, states, bag) of this rank's owned boids, in read order."""
        ids, st = self.local.state()
        bag = self._bags(st)
        x0, x1 = self.strips[self.rank]
        own = (bag // self.dh >= x0) & (bag // self.dh < x1)
        return ids[own], st[own], bag[own]

    def gather_state(self) -> Optional[Tuple[np.ndarray, np.ndarray]]:
        """Every rank's owned boids on rank 0, in the single field's read order
        (bags ascending, the strips' bags are disjoint); None elsewhere."""
        ids, st, _ = self.owned_state()
        objs = [None] * self.world if self.rank == 0 else None
        self.dist.gather_object((ids, st), objs, dst=0, group=self.group)
        if self.rank != 0:
            return None
        return (np.concatenate([o[0] for o in objs]), np.concatenate([o[1] for o in objs]))

    def close(self) -> None:
        close = getattr(self.local, "close", None)
        if close:
            close()
