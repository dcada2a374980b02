"""Bounded device waits run out without a fault, and the field recovers.

The library's kernels wait on one another in two places: the single-pass
look-back scan of the largest bag matrices (a tile waits for its
predecessors' published sums; the scan test hook selects it for any size)
and the persistent tiled step (blocks meet at grid barriers).
Every such wait is bounded.  Here the test hook makes one publisher withhold
its signal, with a short iteration limit, so that the waits give up on
purpose: the kernel returns, the error word carries KB_FLAG_SPIN_TIMEOUT,
kb_field_synchronize reports KB_ERR_DEVICE_FLAG, and once the flag is cleared
(which also resets the waits' control words and empties the read buffer) the
same field, given its state anew, runs steps that equal the oracle's again.
The reference has no device waits; it panics on its errors
(src/engine/schedule.rs:374)."""
import ctypes as C

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from conftest import FLOCK_D
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu
SHORT = 1 << 12  # iterations before a wait gives up (well under a millisecond)


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def step(f, p, first, n):
    L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(first), C.c_uint32(n))


def oracle_state(side, d, ids, xy, dxy, p, steps):
    o = oracle.OracleField(side, side, d, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    if steps:
        o.flock_run(oracle.params_from(p), 0, steps)
    oids, ost, _ = o.iter(1)
    return oids, ost


def expect_timeout(f):
    with pytest.raises(kg.KbError) as e:
        f.synchronize()
    assert e.value.status == L.KB_ERR_DEVICE_FLAG
    flags = f.device_flags(clear=True)
    assert flags & L.KB_FLAG_SPIN_TIMEOUT
    assert f.device_flags() == 0


def test_lookback_scan_wait_runs_out_and_the_field_recovers(gpu):
    # a 2201 x 2201 bag matrix (d = 0.5 on a 1100 torus) takes the single-pass
    # look-back scan in lazy_update's general sort
    side, d, n = 1100.0, 0.5, 3000
    ids, xy, dxy = kg.gen_uniform(n, side, side, 3, 1.0)
    f = kg.Field2D(side, side, d, True, capacity_hint=n)
    try:
        f.set_wait_test(SHORT, L.KB_WITHHOLD_SCAN_PUBLISH, 5)
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        expect_timeout(f)
        # the same field, the hook off: set the state anew, step, compare
        f.set_wait_test(0, L.KB_WITHHOLD_NONE, 0)
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        p = kg.FlockParams(seed=3, neighbor_radius=1.0)
        step(f, p, 0, 3)
        gids, gst = f.get_state()
        assert f.device_flags() == 0
        oids, ost = oracle_state(side, d, ids, xy, dxy, p, 3)
        assert np.array_equal(gids, oids) and same_bits(gst, ost)
    finally:
        f.close()


def test_grid_barrier_wait_runs_out_and_the_field_recovers(gpu):
    # the persistent tiled step: block 0 leaves before its first grid barrier
    side, n = 490.0, 6000
    ids, xy, dxy = kg.gen_uniform(n, side, side, 21, 1.0)
    p = kg.FlockParams(seed=5)
    f = kg.Field2D(side, side, FLOCK_D, True, capacity_hint=n)
    try:
        f.set_step_options(1)
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        step(f, p, 0, 2)  # the persistent path, no hook
        f.synchronize()
        assert f.step_path() == L.KB_PATH_FUSED and f.step_stats()["ctas"] > 0
        f.set_wait_test(SHORT, L.KB_WITHHOLD_GRID_ARRIVAL, 0)
        step(f, p, 2, 4)
        expect_timeout(f)
        f.set_wait_test(0, L.KB_WITHHOLD_NONE, 0)
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        step(f, p, 0, 4)
        gids, gst = f.get_state()
        assert f.device_flags() == 0
        oids, ost = oracle_state(side, FLOCK_D, ids, xy, dxy, p, 4)
        assert np.array_equal(gids, oids) and same_bits(gst, ost)
    finally:
        f.close()


def test_wait_test_rejects_unknown_hooks(gpu):
    f = kg.Field2D(100.0, 100.0, FLOCK_D, True)
    try:
        with pytest.raises(kg.KbError) as e:
            f.set_wait_test(0, 7, 0)
        assert e.value.status == L.KB_ERR_ARG
    finally:
        f.close()


def test_large_bag_matrices_scan_without_waits(gpu):
    # over 4096 scan tiles the bag offsets take three launches (tile sums, one
    # block scanning them, the tiles): 9 M bags need two rounds of that block
    side, d, n = 1500.0, 0.5, 4000
    ids, xy, dxy = kg.gen_uniform(n, side, side, 8, 1.0)
    f = kg.Field2D(side, side, d, True, capacity_hint=n)
    try:
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        p = kg.FlockParams(seed=4, jump=0.3, neighbor_radius=1.0, arith=kg.KB_ARITH_STRICT)
        step(f, p, 0, 3)
        gids, gst = f.get_state()
        oids, ost = oracle_state(side, d, ids, xy, dxy, p, 3)
        assert np.array_equal(gids, oids) and same_bits(gst, ost)
    finally:
        f.close()
