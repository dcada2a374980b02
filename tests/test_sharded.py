"""One field split over ranks by column strips (krabmaga_gb300/sharded.py),
as world-size-2 and -3 gloo process groups on the CPU.

Each rank's local field is the oracle here (the decomposition logic is host
code: strips, halo regions, the exchange of owned boids by their new column,
the insertion order of the next read buffer).  After several steps the owned
boids of all ranks, in strip order, equal the single field's read buffer bit
for bit in strict arithmetic, with boids crossing strip borders and the torus
seam.  The GPU form of the same test is tests/test_gpu_sharded.py."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
D = float(np.float32(10.0) / np.float32(1.5))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleStrip:
    """A rank's local field on the oracle (test infrastructure)."""

    def __init__(self, w, d, capacity):
        import oracle

        self.oracle, self.w, self.d = oracle, w, d
        self.f = oracle.OracleField(w, w, d, True)

    def state(self):
        ids, st, _ = self.f.iter(1)
        return ids, st

    def next_states(self, params, step, ids, states):
        p = self.oracle.params_from(params)
        return np.array([self.f.bird_step(p, step, int(i), s) for i, s in zip(ids, states)],
                        np.float32).reshape(-1, 4)

    def replace(self, ids, states):
        st = np.ascontiguousarray(states, np.float32).reshape(-1, 4)
        self.f = self.oracle.OracleField(self.w, self.w, self.d, True)
        self.f.set_many(ids, st[:, :2], st[:, 2:])
        self.f.lazy_update()


def flock(n, side, seed):
    import oracle

    return oracle.gen_uniform(n, side, side, seed, 1.0)


def _rank_main(rank, world, port, case, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist

    from krabmaga_gb300.model import FlockParams
    from krabmaga_gb300.sharded import ShardedFlock
    from test_sharded import OracleStrip, flock

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n, side, seed, steps, jump = case
        ids, xy, dxy = flock(n, side, seed)
        p = FlockParams(seed=seed, jump=jump)
        sf = ShardedFlock(side, D, p, ids, xy, dxy, make_local=OracleStrip, device="cpu")
        sf.run(0, steps)
        got = sf.gather_state()
        owned = len(sf.owned_state()[0])
        if rank == 0:
            q.put(("state", got[0], got[1]))
        q.put(("owned", rank, owned))
    finally:
        dist.destroy_process_group()


def _run(world, case):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, case, q)) for r in range(world)]
    for p in procs:
        p.start()
    msgs = [q.get(timeout=300) for _ in range(world + 1)]
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs)
    state = [m for m in msgs if m[0] == "state"][0]
    owned = sorted(m[1:] for m in msgs if m[0] == "owned")
    return state[1], state[2], owned


def _single(case):
    import oracle

    from krabmaga_gb300.model import FlockParams

    n, side, seed, steps, jump = case
    ids, xy, dxy = flock(n, side, seed)
    o = oracle.OracleField(side, side, D, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    o.flock_run(oracle.params_from(FlockParams(seed=seed, jump=jump)), 0, steps)
    oids, ost, _ = o.iter(1)
    return oids, ost


@pytest.mark.parametrize("world,case", [(2, (3000, 346.41, 7, 8, 3.0)),
                                        (3, (2500, 316.23, 11, 6, 2.0))])
def test_strips_equal_the_single_field(world, case):
    gids, gst, owned = _run(world, case)
    oids, ost = _single(case)
    assert [o[0] for o in owned] == list(range(world)) and all(o[1] > 0 for o in owned)
    assert sum(o[1] for o in owned) == case[0]
    assert np.array_equal(gids, oids)
    assert np.array_equal(gst.view(np.uint32), ost.view(np.uint32))
    # boids changed strips on the way, across inner borders and the torus seam
    from krabmaga_gb300.sharded import discretize, geometry, strips

    n, side, seed, steps, jump = case
    ids0, xy0, _ = flock(n, side, seed)
    _, dw, _ = geometry(side, D)
    bounds = np.array([x1 for _, x1 in strips(dw, world)])
    strip0 = np.searchsorted(bounds, discretize(xy0[:, 0], D), side="right")
    x1 = np.empty(n, np.float32)
    x1[oids] = ost[:, 0]
    strip1 = np.searchsorted(bounds, discretize(x1[ids0], D), side="right")
    assert np.count_nonzero(strip0 != strip1) > 10
    assert np.count_nonzero(np.abs(x1[ids0] - xy0[:, 0]) > side / 2) > 0  # wrapped at the seam


def test_strip_geometry():
    from krabmaga_gb300.sharded import geometry, query_reach, strips

    max_x, dw, dh = geometry(346.41, D)
    assert (max_x, dw, dh) == (52, 53, 53)
    s = strips(dw, 3)
    assert s[0][0] == 0 and s[-1][1] == dw and all(a[1] == b[0] for a, b in zip(s, s[1:]))
    assert query_reach(10.0, D) == 1 and query_reach(0.0, D) == -1


def test_ranks_driven_in_one_process_equal_the_single_field():
    """The two phases of a step (prepare on every rank, then finish with
    what each rank was sent) driven in one process, no process group: the
    same bits as the single field, over 2 and 3 strips."""
    from krabmaga_gb300.model import FlockParams
    from krabmaga_gb300.sharded import ShardedFlock

    for world, case in ((2, (3000, 346.41, 7, 6, 3.0)), (3, (2500, 316.23, 11, 5, 2.0))):
        n, side, seed, steps, jump = case
        ids, xy, dxy = flock(n, side, seed)
        p = FlockParams(seed=seed, jump=jump)
        ranks = [ShardedFlock(side, D, p, ids, xy, dxy, make_local=OracleStrip, rank=r, world=world)
                 for r in range(world)]
        for k in range(steps):
            parts = [sf.prepare(k) for sf in ranks]
            for r, sf in enumerate(ranks):
                sf.finish([parts[src][r] for src in range(world)])
        own = [sf.owned_state() for sf in ranks]
        gids = np.concatenate([o[0] for o in own])
        gst = np.concatenate([o[1] for o in own])
        oids, ost = _single(case)
        assert np.array_equal(gids, oids)
        assert np.array_equal(gst.view(np.uint32), ost.view(np.uint32))


def test_strips_in_the_exact_query_mode_and_a_wider_ring():
    """The in-tree Bird's exact query (four-corner rule) and a radius of two
    bags (dd = 2, two halo columns each side): still the single field's bits."""
    import oracle

    from krabmaga_gb300 import _lib as L
    from krabmaga_gb300.model import FlockParams
    from krabmaga_gb300.sharded import ShardedFlock

    for qmode, radius in ((L.KB_QUERY_EXACT, 10.0), (L.KB_QUERY_RELAX, 14.0)):
        n, side, seed, steps = 2500, 316.23, 21, 5
        ids, xy, dxy = flock(n, side, seed)
        p = FlockParams(seed=seed, jump=2.0, neighbor_radius=radius, query_mode=qmode)
        world = 3
        ranks = [ShardedFlock(side, D, p, ids, xy, dxy, make_local=OracleStrip, rank=r, world=world)
                 for r in range(world)]
        assert ranks[0].dd == (1 if radius == 10.0 else 2)
        for k in range(steps):
            parts = [sf.prepare(k) for sf in ranks]
            for r, sf in enumerate(ranks):
                sf.finish([parts[s][r] for s in range(world)])
        own = [sf.owned_state() for sf in ranks]
        o = oracle.OracleField(side, side, D, True)
        o.set_many(ids, xy, dxy)
        o.lazy_update()
        o.flock_run(oracle.params_from(p), 0, steps)
        oids, ost, _ = o.iter(1)
        assert np.array_equal(np.concatenate([x[0] for x in own]), oids)
        assert np.array_equal(np.concatenate([x[1] for x in own]).view(np.uint32), ost.view(np.uint32))
