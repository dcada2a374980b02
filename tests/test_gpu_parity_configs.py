"""Parity at the configurations and in the arithmetic the benchmark times.

Through the C ABI on the GPU, against the oracle:
  * one KB_ARITH_FAST step of the 1,048,576-boid uniform flock and of the
    4,194,304-boid clustered flock within TOL_REL_DOMAIN of an FP64 step;
  * three strict steps of the full 4,194,304-boid clustered flock, bit for bit;
  * the benchmark's own 512-replica sweep table for 20 steps in its step mode:
    every replica equal to that replica run alone on a plain field (fast
    arithmetic, bit for bit) and, in strict arithmetic, a 16-replica sample
    equal to the oracle;
  * long runs of the 1,000-boid flock: GPU fast arithmetic against the strict
    oracle, flock order parameter and mean neighbour count within 1%;
  * simulate_old on the GPU Flocker, as the reference's own smoke test of it.
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
TOL_REL_DOMAIN = 1e-5  # one step against FP64, relative to the side of the torus
STAT_TOL = 0.01        # long-run order parameter and mean neighbour count
THREADS = max(1, min(16, os.cpu_count() or 1))

C2_N = 1 << 20
C2_SIDE = float(np.float32(np.sqrt(C2_N / 0.025)))
C3_N = 1 << 22
C3_SIDE = 12952.0


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def gpu_field(side, ids, xy, dxy, d=FLOCK_D):
    f = kg.Field2D(side, side, d, True, capacity_hint=len(ids))
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    return f


def step(f, p, first, n):
    L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(first), C.c_uint32(n))


def fp64_error(side, ids0, xy0, dxy0, p):
    """max |GPU - FP64| over positions (across the seam) and headings after
    one step, relative to the side."""
    o = oracle.OracleField(side, side, FLOCK_D, True)
    o.set_many(ids0, xy0, dxy0)
    o.lazy_update()
    oid, ref = o.flock_step_fp64(oracle.params_from(p), 0)
    del o
    f = gpu_field(side, ids0, xy0, dxy0)
    step(f, p, 0, 1)
    ids, st = f.get_state()
    assert f.device_flags() == 0
    f.close()
    got = st[np.argsort(ids)].astype(np.float64)
    want = ref[np.argsort(oid)]
    assert len(got) == len(want) == len(ids0)
    dpos = np.abs(got[:, :2] - want[:, :2])
    dpos = np.minimum(dpos, side - dpos)
    dhead = np.abs(got[:, 2:] - want[:, 2:])
    return max(dpos.max(), dhead.max()) / side


def test_c2_one_fast_step_within_fp64_tolerance(gpu):
    ids0, xy0, dxy0 = kg.gen_uniform(C2_N, C2_SIDE, C2_SIDE, 7, 1.0)
    p = kg.FlockParams(seed=7, arith=kg.KB_ARITH_FAST)
    err = fp64_error(C2_SIDE, ids0, xy0, dxy0, p)
    print("C2 fast step vs FP64, relative to the side:", err)
    assert err <= TOL_REL_DOMAIN, err


def test_c3_one_fast_step_within_fp64_tolerance(gpu):
    ids0, xy0, dxy0 = kg.gen_clustered(C3_N, C3_SIDE, C3_SIDE, 256, 40.0, 0.3, 11)
    p = kg.FlockParams(seed=11, arith=kg.KB_ARITH_FAST)
    err = fp64_error(C3_SIDE, ids0, xy0, dxy0, p)
    print("C3 fast step vs FP64, relative to the side:", err)
    assert err <= TOL_REL_DOMAIN, err


def test_c3_full_size_three_strict_steps_bit_exact(gpu):
    """4,194,304 clustered boids (256 clusters, sigma 40, side 12952): three
    strict steps equal the oracle's (its agent pass spread over host threads,
    which gives the sequential run's bits)."""
    ids0, xy0, dxy0 = kg.gen_clustered(C3_N, C3_SIDE, C3_SIDE, 256, 40.0, 0.3, 11)
    p = kg.FlockParams(seed=11, arith=kg.KB_ARITH_STRICT)
    f = gpu_field(C3_SIDE, ids0, xy0, dxy0)
    step(f, p, 0, 3)
    ids, st = f.get_state()
    assert f.device_flags() == 0
    assert f.dense_active()
    f.close()
    _, o = oracle.simulate_timed_threads(C3_SIDE, C3_SIDE, FLOCK_D, oracle.params_from(p), ids0,
                                         xy0, dxy0, 3, THREADS, keep_field=True)
    oids, ost, _ = o.iter(1)
    assert np.array_equal(ids, oids) and same_bits(st, ost)


def _sweep_alone(rep, steps):
    f = kg.Field2D(rep.width, rep.height, rep.discretization, True, capacity_hint=rep.n)
    f.set_locations(*rep.state)
    f.lazy_update()
    step(f, rep.params, 0, steps)
    out = f.get_state()
    f.close()
    return out


def test_bench_sweep_table_batched_equals_alone_and_oracle(gpu):
    """The benchmark's sweep: 512 replicas, N log-uniform over [1024, 65536],
    per-replica weights, jump and radius, 20 steps in the benchmark's step
    mode (separate kernels over the packed table, 10-step graphs)."""
    steps = 20
    reps = kg.sweep_replicas(512)
    assert sum(r.n for r in reps) > 7_000_000
    b = kg.Batch(reps)
    b.set_step_options(0)
    b.step(0, steps, 1, 10)
    b.synchronize()  # raises on a device error word
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        aids, ast = _sweep_alone(rep, steps)
        assert np.array_equal(ids, aids) and same_bits(st, ast), f"replica {i}"
    b.close()
    # strict arithmetic: a sample of 16 replicas against the oracle
    sreps = kg.sweep_replicas(512, arith=kg.KB_ARITH_STRICT)
    b = kg.Batch(sreps)
    b.set_step_options(0)
    b.step(0, steps, 1, 10)
    for i in range(0, 512, 32):
        rep = sreps[i]
        ids, st = b.get_replica(i)
        o = oracle.OracleField(rep.width, rep.height, rep.discretization, True)
        o.set_many(*rep.state)
        o.lazy_update()
        o.flock_run(oracle.params_from(rep.params), 0, steps)
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"
    b.close()


def _stats(ids, st, counts, lists, jump):
    """Local order parameter (mean over boids of the norm of the mean unit
    heading of its candidate neighbours) and the mean candidate count."""
    pos = np.empty(int(ids.max()) + 1, np.int64)
    pos[ids] = np.arange(len(ids))
    h = st[:, 2:].astype(np.float64) / jump
    owner = np.repeat(np.arange(len(ids)), counts)
    sums = np.zeros((len(ids), 2))
    np.add.at(sums, owner, h[pos[lists]])
    local = np.linalg.norm(sums, axis=1) / np.maximum(counts, 1)
    return local.mean(), counts.mean()


def test_long_run_fast_gpu_against_strict_oracle(gpu):
    """The 1,000-boid flock (200x200 torus, density 0.025), 128 initial flocks,
    200 steps: the ensemble means of the local order parameter and of the mean
    neighbour count, averaged over steps 150, 175 and 200, agree within 1%
    between the GPU in fast arithmetic and the strict oracle.  The runs are
    chaotic, so they are independent samples; the standard error is printed."""
    seeds = range(128)
    checks = (150, 175, 200)
    gpu_vals, orc_vals = [], []
    for s in seeds:
        ids0, xy0, dxy0 = kg.gen_uniform(1000, SIDE_1K, SIDE_1K, 500 + s, 1.0)
        pf = kg.FlockParams(seed=42 + s, arith=kg.KB_ARITH_FAST)
        ps = oracle.params_from(kg.FlockParams(seed=42 + s, arith=kg.KB_ARITH_STRICT))
        f = gpu_field(SIDE_1K, ids0, xy0, dxy0)
        o = oracle.OracleField(SIDE_1K, SIDE_1K, FLOCK_D, True)
        o.set_many(ids0, xy0, dxy0)
        o.lazy_update()
        g, r = [], []
        done = 0
        for c in checks:
            step(f, pf, done, c - done)
            o.flock_run(ps, done, c - done)
            done = c
            ids, st = f.get_state()
            cnt, lst = f.neighbor_lists(kg.KB_QUERY_RELAX, 10.0, st[:, :2])
            g.append(_stats(ids, st, cnt, lst, 0.7))
            oids, ost, _ = o.iter(1)
            ocnt, olst = o.neighbor_lists(kg.KB_QUERY_RELAX, 10.0, ost[:, :2])
            r.append(_stats(oids, ost, ocnt, olst, 0.7))
        f.close()
        gpu_vals.append(np.mean(g, axis=0))
        orc_vals.append(np.mean(r, axis=0))
    gv, ov = np.array(gpu_vals), np.array(orc_vals)
    gm, om = gv.mean(0), ov.mean(0)
    se = ov.std(0, ddof=1) / np.sqrt(len(ov))
    print("GPU fast", gm, "oracle strict", om, "standard error", se)
    assert abs(gm[0] - om[0]) / om[0] < STAT_TOL, (gm, om, se)
    assert abs(gm[1] - om[1]) / om[1] < STAT_TOL, (gm, om, se)


def test_simulate_old_on_the_gpu_flocker(gpu):
    """tests/explore/simulate.rs:18-38: simulate_old!(Flocker::new((200, 200),
    100), 10, reps) returns one (duration, steps/s) entry per repetition, each
    positive, and the flock has stepped on the device."""
    reps = 3
    state = kg.Flocker((200.0, 200.0), 100, FLOCK_D, params=kg.FlockParams(seed=1))
    out = kg.simulate_old(state, 10, reps)
    assert len(out) == reps
    for dur, sps in out:
        assert dur > 0.0 and sps > 0.0
    assert state.step == 10
    ids, st = state.field1.get_state()
    assert len(ids) == 100 and np.all(np.isfinite(st))
