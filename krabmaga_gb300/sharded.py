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
The exchange goes through `torch.distributed` point-to-point messages.  With
device="cuda" (NCCL) the records stay on the GPU throughout: the local field
hands its read buffer and takes its next read buffer as device tensors
(kb_field_copy_read_buffer, kb_flock_next_states_device,
kb_field_set_states_device), the bag keys, ownership masks, destination
regions and the insertion-order sort are torch operations on the GPU, and
the messages are device buffers.  With gloo the records travel through host
arrays.  A step is two phases, prepare() (the records for every rank) and
finish() (the received records become the next read buffer), so that ranks
can also be driven in one process with any exchange in between.  Requires
every strip to be at least dd + 2 columns wide, so that a boid's new column
is in the region of its owner's neighbours at most.
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


def discretize_device(v, d: float):
    """discretize for a float32 CUDA tensor: floor of the IEEE quotient v / d
    (a tensor divisor: PyTorch divides by a host scalar through its
    reciprocal, which is not the reference's rounding)."""
    import torch

    q = torch.div(v, torch.full_like(v, float(np.float32(d))))
    return torch.floor(q).to(torch.int64)


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


class GpuStripDevice:
    """The local field of one rank on its GPU, its records handed over as
    device tensors (ids int32 holding the u32 bits, records float32 [n, 4])."""

    def __init__(self, w: float, d: float, device: int, capacity: int):
        self.field = Field2D(w, w, d, True, device, capacity_hint=capacity)

    def state(self):
        return self.field.read_buffer_device()

    def next_states(self, params: FlockParams, step: int, ids, states):
        """Bird::step of the given read-buffer boids against the read buffer."""
        if ids.shape[0] == 0:
            return states.new_zeros((0, 4))
        return self.field.next_states_device(params, step, ids, states)

    def replace(self, ids, states) -> None:
        """The read buffer becomes these boids, inserted in this order."""
        if ids.shape[0]:
            self.field.set_states_device(ids.contiguous(), states.contiguous())
        self.field.lazy_update()

    def close(self) -> None:
        self.field.close()


class ShardedFlock:
    """A Flockers simulation on a w x w torus (bags of side d) split over the
    ranks of `group` by column strips.  device="cuda": the records stay on
    GPU `gpu` (GpuStripDevice, NCCL messages); device="cpu": they travel
    through host arrays (GpuStrip on GPU `gpu`, gloo messages).
    `make_local(w, d, capacity)` replaces the local field (host path).
    rank/world given: no process group is used, the caller drives the ranks
    (prepare on every rank, then finish with what each rank was sent)."""

    def __init__(self, w: float, d: float, params: FlockParams, ids: np.ndarray, xy: np.ndarray,
                 dxy: np.ndarray, group=None, make_local: Optional[Callable] = None,
                 device: str = "cpu", gpu: int = 0, rank: Optional[int] = None,
                 world: Optional[int] = None):
        import torch

        if rank is None:
            import torch.distributed as dist

            self.dist = dist
            self.rank = dist.get_rank(group)
            self.world = dist.get_world_size(group)
        else:
            self.dist, self.rank, self.world = None, int(rank), int(world)
        self.group = group
        self.w, self.d, self.params = float(w), float(d), params
        self.on_device = device == "cuda"
        # the exchange buffers: host memory for gloo, this rank's GPU for NCCL
        self.device = torch.device("cuda", gpu) if self.on_device else torch.device(device)
        if self.on_device and self.dist is not None:
            # NCCL's object collectives (gather_state) use the current device
            torch.cuda.set_device(self.device)
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
        cap = len(ids) // self.world + 1
        if make_local is not None:
            self.local = make_local(self.w, self.d, cap)
        elif self.on_device:
            self.local = GpuStripDevice(self.w, self.d, gpu, cap)
        else:
            self.local = GpuStrip(self.w, self.d, gpu, cap)
        # the initial write order is the order of the arrays: keep it for the region
        lo, hi = self.regions[self.rank]
        col = discretize(xy[:, 0], self.d)
        keep = (col >= lo) & (col <= hi)
        st0 = np.concatenate([xy, dxy], axis=1)[keep]
        if self.on_device:
            self.local.replace(torch.from_numpy(ids[keep].view(np.int32)).to(self.device),
                               torch.from_numpy(np.ascontiguousarray(st0)).to(self.device))
        else:
            self.local.replace(ids[keep], st0)

    # ------------------------------------------------------------------ step
    def _bags(self, st: np.ndarray) -> np.ndarray:
        return discretize(st[:, 0], self.d) * self.dh + discretize(st[:, 1], self.d)

    def prepare(self, step_no: int) -> list:
        """Phase 1 of a step: the next state of every owned boid, as records
        [id, x, y, dx, dy, bag >> 31, bag & 0x7FFFFFFF, place in the bag]
        (int32 bits) for each rank whose region holds the boid's new column
        (parts[r] for rank r; numpy on the host path, device tensors on the
        device path)."""
        if self.on_device:
            return self._prepare_device(step_no)
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
        return parts

    def _prepare_device(self, step_no: int) -> list:
        import torch

        ids, st = self.local.state()
        bag = discretize_device(st[:, 0], self.d) * self.dh + discretize_device(st[:, 1], self.d)
        col = bag // self.dh
        x0, x1 = self.strips[self.rank]
        own = (col >= x0) & (col < x1)
        first = torch.searchsorted(bag, bag, right=False)
        place = torch.arange(bag.shape[0], device=bag.device) - first
        oid = ids[own].contiguous()
        nxt = self.local.next_states(self.params, step_no, oid, st[own].contiguous())
        rec = torch.empty((oid.shape[0], 8), dtype=torch.int32, device=bag.device)
        rec[:, 0] = oid
        rec[:, 1:5] = nxt.view(torch.int32)
        rec[:, 5] = (bag[own] >> 31).to(torch.int32)
        rec[:, 6] = (bag[own] & 0x7FFFFFFF).to(torch.int32)
        rec[:, 7] = place[own].to(torch.int32)
        ncol = discretize_device(nxt[:, 0].contiguous(), self.d)
        parts = []
        for r in range(self.world):
            lo, hi = self.regions[r]
            parts.append(rec[(ncol >= lo) & (ncol <= hi)].contiguous())
        return parts

    def finish(self, received: list) -> None:
        """Phase 2 of a step: the records sent to this rank (own part
        included, any order of parts) become the local read buffer, inserted
        in their previous global order (bag, then place in the bag)."""
        if self.on_device:
            import torch

            mine = torch.cat(received, dim=0) if received else \
                torch.zeros((0, 8), dtype=torch.int32, device=self.device)
            # lexicographic (bag hi, bag lo, place) by stable sorts, last key first
            for c in (7, 6, 5):
                mine = mine[torch.sort(mine[:, c], stable=True).indices]
            self.local.replace(mine[:, 0].contiguous(), mine[:, 1:5].contiguous().view(torch.float32))
            return
        mine = np.concatenate(received, axis=0) if received else np.zeros((0, 8), np.int32)
        mine = mine[np.lexsort((mine[:, 7], mine[:, 6].astype(np.int64), mine[:, 5]))]
        self.local.replace(mine[:, 0].view(np.uint32), mine[:, 1:5].view(np.float32))

    def step(self, step_no: int) -> None:
        self.finish(self._exchange(self.prepare(step_no)))

    def _exchange(self, parts: list) -> list:
        """Send parts[r] to rank r (r != self.rank); returns own part plus what
        the others sent here."""
        import torch

        dist, me = self.dist, self.rank
        if dist is None:
            raise RuntimeError("ranks driven by the caller: call prepare() and finish()")
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
        if self.on_device:
            out = {r: parts[r] for r in peers}
        else:
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
        if self.on_device:
            return [parts[me]] + [inc[r] for r in peers]
        return [parts[me]] + [inc[r].cpu().numpy() for r in peers]

    def run(self, first_step: int, nsteps: int) -> None:
        for k in range(nsteps):
            self.step(first_step + k)

    # ------------------------------------------------------------------ state
    def owned_state(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(ids, states, bag) of this rank's owned boids, in read order (host arrays)."""
        ids, st = self.local.state()
        if self.on_device:
            ids, st = ids.cpu().numpy().view(np.uint32), st.cpu().numpy()
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
