"""The Flockers step on the GPU against the oracle.

Bars (all through the C ABI):
  * neighbour sets: bit-exact (ids, in the reference's visiting order) at
    every step;
  * KB_ARITH_STRICT trajectories: bit-exact against the oracle and the
    committed golden fixtures (the oracle is f32-faithful, so this is stronger
    than the FP64 tolerance below);
  * one step, either arithmetic: positions and headings within 1e-5 of the
    domain size of the FP64 oracle;
  * long runs of KB_ARITH_FAST: flock order parameter and mean neighbour count
    within 1% of the strict run.
"""
import ctypes as C
import os

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D, SIDE_1K
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_REL_DOMAIN = 1e-5  # the stated tolerance of one step against FP64, relative to the side


def gpu_field(side, d, ids, xy, dxy, tor=True):
    f = kg.Field2D(side, side, d, tor, capacity_hint=len(ids))
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    return f


def oracle_field(side, d, ids, xy, dxy, tor=True):
    o = oracle.OracleField(side, side, d, tor)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    return o


def step(f, p, first, n):
    L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(first), C.c_uint32(n))


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", ["flock1k_relax_strict.npz", "flock1k_exact_strict.npz"])
def test_1k_flock_matches_golden_fixtures(gpu, name):
    g = np.load(os.path.join(GOLDEN, name))
    f = gpu_field(SIDE_1K, FLOCK_D, g["ids0"], g["xy0"], g["dxy0"])
    p = kg.FlockParams(seed=int(g["seed"]), query_mode=int(g["kind"]), arith=kg.KB_ARITH_STRICT)
    ids, st = f.get_state()
    counts, lists = f.neighbor_lists(int(g["kind"]), 10.0, st[:, :2])
    assert np.array_equal(counts, g["nb_counts0"]) and np.array_equal(lists, g["nb_ids0"])
    done = 0
    for c in g["checkpoints"]:
        step(f, p, done, int(c) - done)
        done = int(c)
        ids, st = f.get_state()
        assert np.array_equal(ids, g[f"ids_{c}"]), f"ids differ at step {c}"
        assert same_bits(st, g[f"st_{c}"]), f"state differs at step {c}"


@pytest.mark.parametrize("kind", [kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT])
def test_1k_flock_neighbour_sets_bit_exact_every_step(gpu, kind):
    ids0, xy0, dxy0 = kg.gen_uniform(1000, SIDE_1K, SIDE_1K, 42, 1.0)
    f = gpu_field(SIDE_1K, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(SIDE_1K, FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=42, query_mode=kind, arith=kg.KB_ARITH_STRICT)
    op = oracle.params_from(p)
    for t in range(200):
        ids, st = f.get_state()
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"state differs at step {t}"
        gc, gl = f.neighbor_lists(kind, 10.0, st[:, :2])
        oc, ol = o.neighbor_lists(kind, 10.0, ost[:, :2])
        assert np.array_equal(gc, oc) and np.array_equal(gl, ol), f"neighbour sets differ at {t}"
        step(f, p, t, 1)
        o.flock_run(op, t, 1)


def test_compute_plus_lazy_update_equals_fused_steps(gpu):
    ids0, xy0, dxy0 = kg.gen_uniform(3000, 300.0, 300.0, 3, 1.0)
    p = kg.FlockParams(seed=9)
    b = gpu_field(300.0, FLOCK_D, ids0, xy0, dxy0)
    state = kg.Flocker((300.0, 300.0), 3000, FLOCK_D, params=p, init_state=(ids0, xy0, dxy0))
    sched = kg.Schedule()
    state.init(sched)
    for t in range(30):  # the reference's per-step path: update at step 0, agents, update
        sched.step_state(state)
    assert sched.step == 30 and sched.time == 29.0
    step(b, p, 0, 30)  # graph-replayed steps
    ia, sa = state.field1.get_state()
    ib, sb = b.get_state()
    assert np.array_equal(ia, ib) and same_bits(sa, sb)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("tile", [(0, 0), (1, 1), (4, 4), (16, 8), (64, 128)])
@pytest.mark.parametrize("kind", [kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT])
def test_fused_tiles_match_oracle(gpu, tile, kind, mode):
    # every tile shape gives the oracle's trajectory bit for bit; 64x128-bag
    # tiles exceed the shared-memory capacity and run the global scratch path
    n, side = 6000, 490.0
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 21, 1.0)
    f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    f.set_step_options(mode, *tile)
    o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=5, query_mode=kind)
    step(f, p, 0, 7)
    step(f, p, 7, 6)
    o.flock_run(oracle.params_from(p), 0, 13)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    stats = f.step_stats()
    assert stats["ctas"] > 0
    if tile == (64, 128):
        assert stats["overflow_tiles"] > 0


def test_step_modes_agree(gpu):
    ids0, xy0, dxy0 = kg.gen_uniform(50000, 1400.0, 1400.0, 8, 1.0)
    p = kg.FlockParams(seed=2, arith=kg.KB_ARITH_FAST)
    out = []
    for mode in (0, 1, 2):
        f = gpu_field(1400.0, FLOCK_D, ids0, xy0, dxy0)
        f.set_step_options(mode)
        step(f, p, 0, 40)
        step(f, p, 40, 3)
        out.append(f.get_state())
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0]) and same_bits(out[0][1], o[1])


def test_fused_sweep_radius_two_rings(gpu):
    # radius 14 with bags of 10/1.5 gives a query ring of two bags
    ids0, xy0, dxy0 = kg.gen_uniform(3000, 350.0, 350.0, 13, 1.0)
    p = kg.FlockParams(seed=3, neighbor_radius=14.0, jump=0.9, cohesion=0.6, avoidance=1.4)
    f = gpu_field(350.0, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(350.0, FLOCK_D, ids0, xy0, dxy0)
    step(f, p, 0, 20)
    o.flock_run(oracle.params_from(p), 0, 20)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)


@pytest.mark.parametrize("side,d,jump,radius", [
    (284.82, 2.005, 0.795, 5.012),   # last column 0.12 wide: wraps from three lines in
    (200.0, FLOCK_D, 0.7, 10.0),        # side/d an exact integer: the x = w line exists
    (101.3, 4.99, 0.98, 12.0),       # ring of two bags, last column 1.5 wide
    (60.05, 6.0, 0.6, 6.5),          # small field, last column 0.05 wide
])
def test_seam_geometries_match_oracle(gpu, side, d, jump, radius):
    n = int(side * side * 0.03)
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 17, 1.0)
    # crowd a band along each seam so wrapping moves happen every step
    xy0[: n // 4, 0] = np.float32(side) - (xy0[: n // 4, 0] % np.float32(1.5))
    xy0[n // 4: n // 2, 1] = xy0[n // 4: n // 2, 1] % np.float32(1.5)
    p = kg.FlockParams(seed=4, jump=jump, neighbor_radius=radius)
    for fused in (2, 1, 0):
        f = gpu_field(side, d, ids0, xy0, dxy0)
        f.set_step_options(fused)
        o = oracle_field(side, d, ids0, xy0, dxy0)
        step(f, p, 0, 15)
        o.flock_run(oracle.params_from(p), 0, 15)
        ids, st = f.get_state()
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"fused={fused}"
        assert f.device_flags() == 0


def test_general_rebuild_path_matches_oracle(gpu):
    # A jump longer than a bag (1.2 > d = 1.0) can carry a boid past the
    # neighbouring bag, so every step takes the general stable sort instead of
    # the stencil gather; the result must still equal the oracle bit for bit.
    ids0, xy0, dxy0 = kg.gen_uniform(2000, 120.0, 120.0, 4, 1.0)
    p = kg.FlockParams(seed=1, jump=1.2, neighbor_radius=2.0)
    d = 1.0  # jump > d: general path
    f = gpu_field(120.0, d, ids0, xy0, dxy0)
    o = oracle_field(120.0, d, ids0, xy0, dxy0)
    step(f, p, 0, 25)
    o.flock_run(oracle.params_from(p), 0, 25)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)


def test_steps_are_deterministic(gpu):
    ids0, xy0, dxy0 = kg.gen_uniform(20000, 900.0, 900.0, 5, 1.0)
    outs = []
    for _ in range(2):
        f = gpu_field(900.0, FLOCK_D, ids0, xy0, dxy0)
        step(f, kg.FlockParams(seed=3, arith=kg.KB_ARITH_FAST), 0, 50)
        outs.append(f.get_state())
    assert np.array_equal(outs[0][0], outs[1][0]) and same_bits(outs[0][1], outs[1][1])


def _fp64_one_step(side, d, ids0, xy0, dxy0, kind, arith):
    f = gpu_field(side, d, ids0, xy0, dxy0)
    o = oracle_field(side, d, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=77, query_mode=kind, arith=arith)
    oid, ref = o.flock_step_fp64(oracle.params_from(p), 0)
    step(f, p, 0, 1)
    ids, st = f.get_state()
    order = np.argsort(ids)
    oorder = np.argsort(oid)
    got = st[order].astype(np.float64)
    want = ref[oorder]
    dpos = np.abs(got[:, :2] - want[:, :2])
    dpos = np.minimum(dpos, side - dpos)  # across the seam
    dhead = np.abs(got[:, 2:] - want[:, 2:])
    return max(dpos.max(), dhead.max()) / side


@pytest.mark.parametrize("arith", [kg.KB_ARITH_STRICT, kg.KB_ARITH_FAST])
@pytest.mark.parametrize("kind", [kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT])
def test_one_step_within_fp64_tolerance(gpu, arith, kind):
    ids0, xy0, dxy0 = kg.gen_uniform(1000, SIDE_1K, SIDE_1K, 42, 1.0)
    err = _fp64_one_step(SIDE_1K, FLOCK_D, ids0, xy0, dxy0, kind, arith)
    assert err <= TOL_REL_DOMAIN, err


def _order_and_neighbours(f, jump):
    """Local order parameter (mean over boids of the norm of the mean unit
    heading of its candidate neighbours) and mean candidate count."""
    ids, st = f.get_state()
    counts, lists = f.neighbor_lists(kg.KB_QUERY_RELAX, 10.0, st[:, :2])
    pos = np.empty(int(ids.max()) + 1, np.int64)
    pos[ids] = np.arange(len(ids))
    h = st[:, 2:].astype(np.float64) / jump
    owner = np.repeat(np.arange(len(ids)), counts)
    sums = np.zeros((len(ids), 2))
    np.add.at(sums, owner, h[pos[lists]])
    local = np.linalg.norm(sums, axis=1) / np.maximum(counts, 1)
    return local.mean(), counts.mean()


def _ensemble(arith, seeds, jitter_base, n, side):
    vals = []
    for seed in seeds:
        ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 100 + seed, 1.0)
        f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
        step(f, kg.FlockParams(seed=jitter_base + seed, arith=arith), 0, 200)
        vals.append(_order_and_neighbours(f, 0.7))
        f.close()
    return np.array(vals)


def test_long_run_statistics_fast_vs_strict(gpu):
    """Flocks at density 0.025 boids per unit^2, 200 steps, 32
    initial flocks of 20,000 boids: the ensemble means of the local order
    parameter and of the mean neighbour count under the fast arithmetic agree
    with the strict ones within 1%.  Chaos makes the two runs independent
    samples after a few dozen steps, so the same comparison of strict against
    strict with another jitter seed is printed as the noise floor."""
    n = 20000
    side = float(np.sqrt(n / 0.025))
    seeds = range(32)
    strict = _ensemble(kg.KB_ARITH_STRICT, seeds, 0, n, side)
    fast = _ensemble(kg.KB_ARITH_FAST, seeds, 0, n, side)
    control = _ensemble(kg.KB_ARITH_STRICT, seeds, 1000, n, side)
    s, q, c = strict.mean(0), fast.mean(0), control.mean(0)
    se = strict.std(0, ddof=1) / np.sqrt(len(strict))
    print("strict", s, "fast", q, "strict/other jitter", c, "standard error", se)
    assert abs(q[0] - s[0]) / s[0] < 0.01, (q, s, c, se)
    assert abs(q[1] - s[1]) / s[1] < 0.01, (q, s, c, se)


def test_1m_flock_full_size_one_step(gpu):
    """1,048,576 boids at density 0.025: neighbour digests of every boid and
    the one-step state (strict) equal the oracle's."""
    n = 1 << 20
    side = float(np.float32(np.sqrt(n / 0.025)))
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 7, 1.0)
    f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    gc, gd = f.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, st[:, :2])
    oc, od = o.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, st[:, :2])
    assert np.array_equal(gc, oc) and np.array_equal(gd, od)
    p = kg.FlockParams(seed=7)
    step(f, p, 0, 1)
    o.flock_run(oracle.params_from(p), 0, 1)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    assert f.device_flags() == 0


def test_1m_flock_ten_strict_steps_match_oracle(gpu):
    """The C2 workload (1,048,576 boids) for ten strict steps, graph-replayed on
    the separate kernels: the whole state equals the oracle's after them."""
    n = 1 << 20
    side = float(np.float32(np.sqrt(n / 0.025)))
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 7, 1.0)
    f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=7, arith=kg.KB_ARITH_STRICT)
    step(f, p, 0, 10)
    o.flock_run(oracle.params_from(p), 0, 10)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    assert f.device_flags() == 0


def test_1m_flock_invariants_after_300_fast_steps(gpu):
    """Size-independent properties of the C2 workload after 300 fast steps
    (the benchmark's arithmetic): every id once, every heading of length jump,
    every position on the torus, the read buffer in canonical bag order with
    each boid in the bag of its position, and neighbour counts and digests of
    a sample equal to the oracle's on the same read buffer."""
    n = 1 << 20
    side = np.float32(np.sqrt(n / 0.025))
    ids0, xy0, dxy0 = kg.gen_uniform(n, float(side), float(side), 7, 1.0)
    f = gpu_field(float(side), FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=7, arith=kg.KB_ARITH_FAST)
    step(f, p, 0, 300)
    assert f.device_flags() == 0
    ids, st = f.get_state()
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    speed = np.hypot(st[:, 2].astype(np.float64), st[:, 3].astype(np.float64))
    assert np.all(np.abs(speed - 0.7) < 1e-5)
    assert np.all((st[:, :2] >= 0) & (st[:, :2] <= side))
    d = np.float32(FLOCK_D)
    cx = np.floor(st[:, 0] / d).astype(np.int64)
    cy = np.floor(st[:, 1] / d).astype(np.int64)
    dh = int(np.ceil(side / d)) + 1
    bag = cx * dh + cy
    assert np.all(np.diff(bag) >= 0)  # bags ascending in read order
    o = oracle.OracleField(float(side), float(side), FLOCK_D, True)
    o.set_many(ids, st[:, :2], st[:, 2:])
    o.lazy_update()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)  # same canonical order
    q = st[::53, :2]
    gc, gd = f.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, q)
    oc, od = o.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, q)
    assert np.array_equal(gc, oc) and np.array_equal(gd, od)


def test_4m_clustered_quarter_size_digests(gpu):
    """Clustered stress (256 Gaussian clusters, sigma 40) at a quarter of the
    4,194,304-boid size: after 3 strict steps the state equals the oracle's
    and so do the neighbour digests of a sample of boids."""
    n = 1 << 20
    side = 12952.0 / 2
    ids0, xy0, dxy0 = kg.gen_clustered(n, side, side, 256, 40.0, 0.3, 11)
    f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=11)
    step(f, p, 0, 3)
    o.flock_run(oracle.params_from(p), 0, 3)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    q = st[:: 97, :2]
    gc, gd = f.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, q)
    oc, od = o.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, q)
    assert np.array_equal(gc, oc) and np.array_equal(gd, od)
    assert gc.max() > 100  # dense cluster cores are exercised
    assert f.dense_active()  # the per-run walk and 8-bag rebin segments ran


@pytest.mark.parametrize("arith", [kg.KB_ARITH_STRICT, kg.KB_ARITH_FAST])
def test_dense_walk_gives_the_same_bits(gpu, arith):
    # A clustered flock takes the per-run candidate walk and 8-bag rebin
    # segments by itself; forcing the flat walk gives the same bits over
    # graph-replayed steps, and strict arithmetic equals the oracle.
    n, side = 1 << 16, 1600.0
    ids0, xy0, dxy0 = kg.gen_clustered(n, side, side, 16, 30.0, 0.3, 5)
    p = kg.FlockParams(seed=3, arith=arith)
    a = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    b = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    assert a.dense_active()
    b.set_dense_mode(kg.KB_DENSE_OFF)
    assert not b.dense_active()
    step(a, p, 0, 12)
    step(b, p, 0, 12)
    ia, sa = a.get_state()
    ib, sb = b.get_state()
    assert np.array_equal(ia, ib) and same_bits(sa, sb)
    assert a.device_flags() == 0 and b.device_flags() == 0
    if arith == kg.KB_ARITH_STRICT:
        o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
        o.flock_run(oracle.params_from(p), 0, 12)
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ia, oids) and same_bits(sa, ost)


def test_dense_walk_forced_on_a_uniform_flock(gpu):
    n = 20000
    side = float(np.float32(np.sqrt(n / 0.025)))
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 9, 1.0)
    p = kg.FlockParams(seed=4, arith=kg.KB_ARITH_FAST)
    u = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    v = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    assert not u.dense_active()
    u.set_dense_mode(kg.KB_DENSE_ON)
    assert u.dense_active()
    step(u, p, 0, 10)
    step(v, p, 0, 10)
    iu, su = u.get_state()
    iv, sv = v.get_state()
    assert np.array_equal(iu, iv) and same_bits(su, sv)
    # back to automatic: the next step measures the occupancies again
    u.set_dense_mode(kg.KB_DENSE_AUTO)
    step(u, p, 10, 1)
    u.synchronize()
    assert not u.dense_active()
    with pytest.raises(kg.KbError):
        u.set_dense_mode(7)


def test_device_jitter_matches_oracle_philox(gpu):
    # a lone bird (no neighbours but itself) moves by momentum + jitter only:
    # its heading reveals the device's Philox draws for (seed, id, step)
    side = 100.0
    ids = np.array([12345], np.uint32)
    xy = np.array([[50.0, 50.0]], np.float32)
    dxy = np.array([[0.0, 0.0]], np.float32)
    f = gpu_field(side, FLOCK_D, ids, xy, dxy)
    o = oracle_field(side, FLOCK_D, ids, xy, dxy)
    p = kg.FlockParams(seed=(7 << 32) | 99, momentum=0.0)
    for t in range(5):
        step(f, p, t, 1)
        o.flock_run(oracle.params_from(p), t, 1)
        assert same_bits(f.get_state()[1], o.iter(1)[1])


@pytest.mark.parametrize("kind", [kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT])
@pytest.mark.parametrize("side,radius", [(300.0, 10.0), (40.0, 14.0), (30.0, 16.0)])
def test_true_torus_option_matches_oracle(gpu, kind, side, radius):
    # KB_CELL_WRAP_TORUS: the query's cell range wraps (the reference clamps
    # it); trajectories and per-step neighbour lists stay bit-exact against
    # the oracle with the same option, including rings that cover the field
    n = int(side * side * 0.025) + 40
    ids0, xy0, dxy0 = kg.gen_uniform(n, side, side, 17, 1.0)
    p = kg.FlockParams(seed=6, query_mode=kind, neighbor_radius=radius, arith=kg.KB_ARITH_STRICT)
    f = kg.Field2D(side, side, FLOCK_D, True, capacity_hint=n, cell_wrap=kg.KB_CELL_WRAP_TORUS)
    f.set_locations(ids0, xy0, dxy0)
    f.lazy_update()
    o = oracle.OracleField(side, side, FLOCK_D, True, cell_wrap=1)
    o.set_many(ids0, xy0, dxy0)
    o.lazy_update()
    for s in range(0, 24, 6):
        step(f, p, s, 6)
        o.flock_run(oracle.params_from(p), s, 6)
        ids, st = f.get_state()
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), s
        gc, gl = f.neighbor_lists(kind, radius, st[:, :2])
        oc, ol = o.neighbor_lists(kind, radius, st[:, :2])
        assert np.array_equal(gc, oc) and np.array_equal(gl, ol), s
    # across the seam the wrapped range finds more than the clamped one
    g2 = kg.Field2D(side, side, FLOCK_D, True)
    g2.set_locations(ids, st[:, :2].copy(), st[:, 2:].copy())
    g2.lazy_update()
    cc, _ = g2.neighbor_lists(kind, radius, st[:, :2])
    assert (gc >= cc).all() and gc.sum() > cc.sum()


def test_births_and_deaths_between_steps_match_oracle(gpu):
    # A changing population, as the reference runs one: an agent that stops
    # is not re-inserted (schedule.rs:401-407), a newborn is inserted during
    # the step, and both show after lazy_update.  Here: the agent pass
    # (kb_flock_compute), removals and insertions on the write buffer, then
    # lazy_update; the oracle does the same and the read buffers must agree.
    side = 300.0
    ids0, xy0, dxy0 = kg.gen_uniform(2000, side, side, 21, 1.0)
    f = gpu_field(side, FLOCK_D, ids0, xy0, dxy0)
    o = oracle_field(side, FLOCK_D, ids0, xy0, dxy0)
    p = kg.FlockParams(seed=8, arith=kg.KB_ARITH_STRICT)
    rng = np.random.default_rng(4)
    next_id, alive = 2000, 2000
    for s in range(8):
        L.call("kb_flock_compute", f.handle, C.byref(p.to_c()), C.c_uint64(s))
        o.flock_compute(oracle.params_from(p), s)
        wids, wst, _ = o.iter(0)  # the write buffer after the agent pass
        for k in rng.choice(len(wids), size=25, replace=False):
            loc = kg.Real2D(float(wst[k, 0]), float(wst[k, 1]))
            f.remove_object_location(kg.Bird(int(wids[k]), loc), loc)
            o.remove(int(wids[k]), float(wst[k, 0]), float(wst[k, 1]))
        nb = 15 + 5 * s
        bid = np.arange(next_id, next_id + nb, dtype=np.uint32)
        bxy = (rng.random((nb, 2)) * side).astype(np.float32)
        bdxy = (rng.standard_normal((nb, 2)) * 0.5).astype(np.float32)
        next_id += nb
        alive += nb - 25
        f.set_locations(bid, bxy, bdxy)
        o.set_many(bid, bxy, bdxy)
        f.lazy_update()
        o.lazy_update()
        ids, st = f.get_state()
        oids, ost, _ = o.iter(1)
        assert len(ids) == alive
        assert np.array_equal(ids, oids) and same_bits(st, ost), s
    # whole steps continue from the edited population
    step(f, p, 8, 5)
    o.flock_run(oracle.params_from(p), 8, 5)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)


def test_duplicate_ids_exclude_each_other_as_the_reference_does(gpu):
    # Bird::step skips every candidate whose id equals its own (bird.rs:50),
    # so boids sharing an id ignore each other.  With unique ids the force
    # pass excludes the boid's own slot instead; with repeats it must compare
    # ids, and the trajectories still equal the oracle's.
    ids0, xy0, dxy0 = kg.gen_uniform(3000, 350.0, 350.0, 5, 1.0)
    ids0 = ids0.copy()
    ids0[1::7] = ids0[0::7][: len(ids0[1::7])]
    assert len(np.unique(ids0)) < len(ids0)
    p = kg.FlockParams(seed=3, arith=kg.KB_ARITH_STRICT)
    for kind in (kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT):
        p.query_mode = kind
        f = gpu_field(350.0, FLOCK_D, ids0, xy0, dxy0)
        o = oracle_field(350.0, FLOCK_D, ids0, xy0, dxy0)
        step(f, p, 0, 20)
        o.flock_run(oracle.params_from(p), 0, 20)
        ids, st = f.get_state()
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), kind
        # removing the repeats (a new population through lazy_update) goes
        # back to the slot test, still equal to the oracle
        keep = np.unique(ids, return_index=True)[1]
        g = gpu_field(350.0, FLOCK_D, ids[keep], st[keep, :2].copy(), st[keep, 2:].copy())
        q = oracle_field(350.0, FLOCK_D, ids[keep], st[keep, :2].copy(), st[keep, 2:].copy())
        step(g, p, 20, 10)
        q.flock_run(oracle.params_from(p), 20, 10)
        gi, gs = g.get_state()
        qi, qs, _ = q.iter(1)
        assert np.array_equal(gi, qi) and same_bits(gs, qs), kind
