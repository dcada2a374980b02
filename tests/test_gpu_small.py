"""Whole steps of a small field in one thread-block cluster, the default step
path for runs of steps on plain fields of at most 4096 boids and 4096 bags
(kb_small.cu): bit-exact
against the oracle in strict arithmetic, and the same bits as the separate
kernels (step mode 3) in fast arithmetic."""
import ctypes as C

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu

CASES = {
    # name: (w, h, d, toroidal, cell_wrap, n, radius)
    "c1": (101.0, 101.0, FLOCK_D, True, kg.KB_CELL_WRAP_CLAMP, 256, 10.0),
    # the reference's own test field (tests/engine/field_2d.rs: 10x10, d 0.5)
    "ref10": (10.0, 10.0, 0.5, True, kg.KB_CELL_WRAP_CLAMP, 100, 10.0),
    "non_toroidal": (90.0, 90.0, FLOCK_D, False, kg.KB_CELL_WRAP_CLAMP, 200, 10.0),
    "true_torus": (80.0, 80.0, FLOCK_D, True, kg.KB_CELL_WRAP_TORUS, 160, 10.0),
    # dense: about 40 candidates per boid
    "full": (40.0, 40.0, FLOCK_D, True, kg.KB_CELL_WRAP_CLAMP, 256, 10.0),
    # the 1,000-boid Flockers case and the largest field the cluster takes
    "c1k": (200.0, 200.0, FLOCK_D, True, kg.KB_CELL_WRAP_CLAMP, 1000, 10.0),
    "max": (405.0, 405.0, FLOCK_D, True, kg.KB_CELL_WRAP_CLAMP, 4096, 10.0),
    # many bags: 4096 (64 x 64, the most the cluster takes)
    "wide": (float(np.float32(63.0) * np.float32(FLOCK_D)), float(np.float32(63.0) * np.float32(FLOCK_D)),
             FLOCK_D, True, kg.KB_CELL_WRAP_CLAMP, 250, 10.0),
}


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def fields(case, seed=3, dup=0):
    w, h, d, tor, wrap, n, _ = CASES[case]
    ids, xy, dxy = kg.gen_uniform(n, w, h, seed, 1.0)
    if dup:
        ids = ids.copy()
        ids[-dup:] = ids[:dup]  # repeated ids: self is found by id
    f = kg.Field2D(w, h, d, tor, cell_wrap=wrap, capacity_hint=n)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    o = oracle.OracleField(w, h, d, tor, cell_wrap=wrap)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    return f, o


def step(f, p, first, n):
    L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(first), C.c_uint32(n))


@pytest.mark.parametrize("kind", [kg.KB_QUERY_RELAX, kg.KB_QUERY_EXACT])
@pytest.mark.parametrize("case", sorted(CASES))
def test_small_path_matches_oracle(gpu, case, kind):
    f, o = fields(case)
    assert f.step_path() == kg.KB_PATH_SMALL, f.step_path()
    p = kg.FlockParams(seed=5, query_mode=kind, neighbor_radius=CASES[case][6],
                       arith=kg.KB_ARITH_STRICT)
    op = oracle.params_from(p)
    step(f, p, 0, 25)              # one launch
    o.flock_run(op, 0, 25)
    for t in range(25, 28):        # one launch per call
        step(f, p, t, 1)
        o.flock_run(op, t, 1)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    assert f.device_flags() == 0


def test_small_path_with_repeated_ids(gpu):
    f, o = fields("c1", dup=20)
    p = kg.FlockParams(seed=2, arith=kg.KB_ARITH_STRICT)
    step(f, p, 0, 12)
    o.flock_run(oracle.params_from(p), 0, 12)
    ids, st = f.get_state()
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)


@pytest.mark.parametrize("case", ["c1", "full", "c1k", "max"])
def test_small_path_equals_separate_kernels(gpu, case):
    a, _ = fields(case, seed=8)
    b, _ = fields(case, seed=8)
    b.set_step_options(3)
    assert a.step_path() == kg.KB_PATH_SMALL
    # the dense case takes the per-run walk on the separate kernels
    assert b.step_path() == (kg.KB_PATH_DENSE if case == "full" else kg.KB_PATH_SEPARATE)
    p = kg.FlockParams(seed=6, arith=kg.KB_ARITH_FAST)
    step(a, p, 0, 150)
    step(b, p, 0, 150)             # graph-replayed chunks
    step(a, p, 150, 2)
    step(b, p, 150, 2)
    ia, sa = a.get_state()
    ib, sb = b.get_state()
    assert np.array_equal(ia, ib) and same_bits(sa, sb)
    # the field's other entry points see the small path's result
    ca, da = a.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, sa[:, :2])
    cb, db = b.neighbor_digest(kg.KB_QUERY_RELAX, 10.0, sb[:, :2])
    assert np.array_equal(ca, cb) and np.array_equal(da, db)


@pytest.mark.parametrize("mode", [0, 3])
def test_positions_outside_the_matrix_are_flagged_on_both_paths(gpu, mode):
    # y wraps with the width (bird.rs:147): on a field wider than high a lone
    # bird heading up leaves the bag matrix; the reference panics there, and
    # both step paths raise the key-range flag
    f = kg.Field2D(200.0, 20.0, FLOCK_D, True)
    f.set_step_options(mode)
    f.set_locations(np.array([7], np.uint32), np.array([[199.0, 19.0]], np.float32),
                    np.array([[0.0, 1.0]], np.float32))
    f.lazy_update()
    assert f.step_path() == (kg.KB_PATH_SMALL if mode == 0 else kg.KB_PATH_SEPARATE)
    p = kg.FlockParams(seed=1, arith=kg.KB_ARITH_STRICT, jump=6.0)
    with pytest.raises(kg.KbError):
        step(f, p, 0, 30)
        f.synchronize()
    assert f.device_flags(clear=True) & 0x1  # KB_FLAG_KEY_RANGE


def test_small_path_random_fields_equal_separate_kernels(gpu):
    # seeded random small fields (size, density, bag size, torus options, query kind): the
    # cluster path and the separate kernels give the same bits over a run of steps
    rng = np.random.default_rng(2024)
    ran = 0
    for case in range(24):
        n = int(rng.choice([1, 2, 31, 200, 999, 2500, 4096]))
        dens = float(rng.uniform(0.01, 0.2))
        side = float(np.float32(max(20.0, np.sqrt(n / dens))))
        d = float(np.float32(rng.choice([10.0 / 1.5, 5.0, 10.0])))
        tor = bool(rng.integers(0, 2))
        wrap = kg.KB_CELL_WRAP_TORUS if (tor and rng.integers(0, 2)) else kg.KB_CELL_WRAP_CLAMP
        kind = int(rng.integers(0, 2))
        cells = (int(np.ceil(np.float32(side) / np.float32(d))) + 1) ** 2
        ids, xy, dxy = kg.gen_uniform(n, side, side, 100 + case, 1.0)
        p = kg.FlockParams(seed=case, query_mode=kind, arith=kg.KB_ARITH_FAST,
                           jump=float(rng.uniform(0.3, 1.5)))
        out = []
        for mode in (0, 3):
            f = kg.Field2D(side, side, d, tor, cell_wrap=wrap, capacity_hint=n)
            f.set_step_options(mode)
            f.set_locations(ids, xy, dxy)
            f.lazy_update()
            if mode == 0 and cells <= 4096:
                assert f.step_path() == kg.KB_PATH_SMALL, (case, n, cells)
                ran += 1
            step(f, p, 0, 12)
            out.append(f.get_state())
            assert f.device_flags() == 0, case
            f.close()
        (ia, sa), (ib, sb) = out
        assert np.array_equal(ia, ib) and same_bits(sa, sb), (case, n, side, d, tor, wrap, kind)
    assert ran >= 12
