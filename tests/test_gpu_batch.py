"""Batched replicas on the GPU: every replica of a packed batch equals the
oracle run of that replica alone, bit for bit (strict arithmetic), whatever
the launch grouping; and a batch equals plain single-field runs."""
import ctypes as C

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def small_sweep(arith, qmode=kg.KB_QUERY_RELAX):
    reps = kg.sweep_replicas(7, n_min=300, n_max=5000, arith=arith, query_mode=qmode, table_seed=5)
    # one replica with a two-bag query ring (bags of radius / 2.5)
    r = reps[3]
    r.discretization = float(np.float32(r.params.neighbor_radius) / np.float32(2.5))
    return reps


def oracle_run(rep, nsteps):
    o = oracle.OracleField(rep.width, rep.height, rep.discretization, True)
    o.set_many(*rep.state)
    o.lazy_update()
    o.flock_run(oracle.params_from(rep.params), 0, nsteps)
    ids, st, _ = o.iter(1)
    return ids, st


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("grouping", [(0, 0), (1, 0), (1, 4), (3, 2)])
def test_batch_replicas_match_oracle(gpu, grouping, mode):
    spl, graphs = grouping
    reps = small_sweep(kg.KB_ARITH_STRICT)
    b = kg.Batch(reps)
    b.set_step_options(mode)
    b.step(0, 12, spl, graphs)
    b.step(12, 9, spl, graphs)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 21)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_graphs_follow_a_tile_change(gpu, mode):
    # graphs replayed before a tile change are not replayed after it: the
    # change rebuilds the tile table, and the next steps capture new graphs
    reps = small_sweep(kg.KB_ARITH_STRICT)[:4]
    b = kg.Batch(reps)
    b.set_step_options(mode, 4, 4)
    b.step(0, 8, 1, 4)
    assert b.step_stats()["tile"] == (4, 4)
    b.set_step_options(mode, 16, 8)
    b.step(8, 8, 1, 4)
    assert b.step_stats()["tile"] == (16, 8)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 16)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


def test_batch_autotune_refuses_tiles_out_of_range(gpu):
    # candidates obey the bounds of set_step_options; a refused call runs no step
    reps = small_sweep(kg.KB_ARITH_STRICT)[:3]
    b = kg.Batch(reps)
    b.set_step_options(1)
    for bad in [(8, 16), (65, 8)], [(4, 129)], [(-1, 8)]:
        with pytest.raises(kg.KbError) as e:
            b.autotune(0, 2, candidates=bad)
        assert e.value.status == L.KB_ERR_ARG
    b.step(0, 6, 1, 0)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 6)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


def test_batch_exact_query_matches_oracle(gpu):
    reps = small_sweep(kg.KB_ARITH_STRICT, kg.KB_QUERY_EXACT)[:4]
    b = kg.Batch(reps)
    b.step(0, 10, 1, 5)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 10)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


@pytest.mark.parametrize("mode", [0, 2])
def test_batch_equals_plain_fields(gpu, mode):
    # fast arithmetic: the batch (either step path) and the plain field (its
    # default path) give the same bits
    reps = small_sweep(kg.KB_ARITH_FAST)
    b = kg.Batch(reps)
    b.set_step_options(mode)
    b.step(0, 30, 1, 10)
    for i, rep in enumerate(reps):
        f = kg.Field2D(rep.width, rep.height, rep.discretization, True)
        f.set_locations(*rep.state)
        f.lazy_update()
        L.call("kb_flock_step", f.handle, C.byref(rep.params.to_c()), C.c_uint64(0), C.c_uint32(30))
        fi, fs = f.get_state()
        bi, bs = b.get_replica(i)
        assert np.array_equal(fi, bi) and same_bits(fs, bs), f"replica {i}"


def test_batch_unfused_path_matches(gpu):
    reps = small_sweep(kg.KB_ARITH_STRICT)[:3]
    b = kg.Batch(reps)
    b.set_step_options(False)
    b.step(0, 8)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 8)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


def test_batch_rejects_mixed_modes(gpu):
    reps = small_sweep(kg.KB_ARITH_FAST)[:2]
    reps[1].params.arith = kg.KB_ARITH_STRICT
    with pytest.raises(kg.KbError):
        kg.Batch(reps)


@pytest.mark.parametrize("mode", [0, 2])
def test_batch_true_torus_replica_matches_oracle(gpu, mode):
    # a true-torus replica beside clamped ones: the tiled path leaves the
    # batch to the separate kernels (the tiles assume the clamped range)
    reps = small_sweep(kg.KB_ARITH_STRICT)[:4]
    reps[1].cell_wrap = kg.KB_CELL_WRAP_TORUS
    b = kg.Batch(reps)
    b.set_step_options(mode)
    b.step(0, 15, 1, 5)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        o = oracle.OracleField(rep.width, rep.height, rep.discretization, True,
                               cell_wrap=rep.cell_wrap)
        o.set_many(*rep.state)
        o.lazy_update()
        o.flock_run(oracle.params_from(rep.params), 0, 15)
        oids, ost, _ = o.iter(1)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


@pytest.mark.parametrize("mode", [0, 2])
def test_batch_add_and_remove_replicas_match_oracle(gpu, mode):
    # replicas join and leave a running batch: each one still equals the
    # oracle run of it alone over the steps it took part in (strict bits)
    reps = small_sweep(kg.KB_ARITH_STRICT)
    b = kg.Batch(reps[:4])
    b.set_step_options(mode)
    live = [(reps[i], 0) for i in range(4)]  # (replica, batch step of its step 0)
    b.step(0, 10, 1, 5)
    b.remove_replica(1)
    del live[1]
    assert b.add_replica(reps[5], 10) == 3    # grows the bag arrays
    live.append((reps[5], 10))
    b.step(10, 10, 1, 5)
    assert b.add_replica(reps[6], 20) == 4
    live.append((reps[6], 20))
    b.remove_replica(0)
    del live[0]
    b.step(20, 5, 1, 5)
    assert b.nrep == len(live) == 4
    m = b.moments()
    for i, (rep, origin) in enumerate(live):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 25 - origin)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"
        assert m[i, 0] == rep.n


def test_batch_add_replica_errors_leave_the_batch_unchanged(gpu):
    reps = small_sweep(kg.KB_ARITH_STRICT)[:3]
    b = kg.Batch(reps[:2])
    b.step(0, 4)
    bad = kg.Replica(reps[2].width, reps[2].height, reps[2].discretization, reps[2].params,
                     (reps[2].state[0], reps[2].state[1].copy(), reps[2].state[2]))
    bad.state[1][7] = (reps[2].width * 3, 1.0)        # outside the bag matrix
    with pytest.raises(L.KbError) as err:
        b.add_replica(bad, 4)
    assert err.value.status == L.KB_ERR_RANGE and "object 7" in str(err.value)
    bad.state[1][7] = (np.nan, 1.0)
    with pytest.raises(L.KbError) as err:
        b.add_replica(bad, 4)
    assert err.value.status == L.KB_ERR_ARG
    fast = kg.Replica(reps[2].width, reps[2].height, reps[2].discretization,
                      kg.FlockParams(arith=kg.KB_ARITH_FAST), reps[2].state)
    with pytest.raises(L.KbError):
        b.add_replica(fast, 4)
    with pytest.raises(L.KbError) as err:
        b.remove_replica(2)
    assert err.value.status == L.KB_ERR_ARG
    assert b.nrep == 2
    b.step(4, 6)
    for i, rep in enumerate(reps[:2]):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, 10)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"
    b.remove_replica(0)
    with pytest.raises(L.KbError) as err:
        b.remove_replica(0)                          # the last replica stays
    assert err.value.status == L.KB_ERR_STATE


def test_batch_closes_as_a_context_manager(gpu):
    reps = small_sweep(kg.KB_ARITH_STRICT)[:2]
    with kg.Batch(reps) as b:
        b.step(0, 3)
        ids, st = b.get_replica(1)
    oids, ost = oracle_run(reps[1], 3)
    assert np.array_equal(ids, oids) and same_bits(st, ost)
    assert b.handle is None


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_mode0_force_block_sizes_match_oracle(gpu, threads):
    # the separate-kernel step over packed replicas at each force block size
    # the autotuner may pick (one candidate: the autotuner keeps it)
    reps = small_sweep(kg.KB_ARITH_STRICT)
    b = kg.Batch(reps)
    b.set_step_options(0)
    t, per_block, used, ms = b.autotune(0, 2, candidates=[(threads, 1)])
    assert (t, per_block) == (threads, 1) and used == 3 and ms > 0
    b.step(used, 9, 1, 0)
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, used + 9)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"


def test_mode0_autotune_picks_a_block_size_and_refuses_others(gpu):
    reps = small_sweep(kg.KB_ARITH_FAST)
    b = kg.Batch(reps)
    b.set_step_options(0)
    t, per_block, used, ms = b.autotune(0, 2)
    assert t in (128, 256, 512) and per_block == 1 and used == 9
    for bad in [[(64, 1)], [(256, 2)]]:
        with pytest.raises(kg.KbError) as e:
            b.autotune(used, 2, candidates=bad)
        assert e.value.status == L.KB_ERR_ARG


def test_mode0_graphs_follow_a_block_size_change(gpu):
    # separate-kernel steps replayed from graphs, then a force block size set
    # by the autotuner, then graphs again: the graphs captured before the
    # change are not replayed after it, every replica still equals the oracle
    reps = small_sweep(kg.KB_ARITH_STRICT)
    b = kg.Batch(reps)
    b.set_step_options(0)
    b.step(0, 8, 1, 4)
    done = 8
    for threads in (512, 128):
        t, _, used, _ = b.autotune(done, 1, candidates=[(threads, 1)])
        assert t == threads
        done += used
        b.step(done, 9, 1, 4)
        done += 9
    for i, rep in enumerate(reps):
        ids, st = b.get_replica(i)
        oids, ost = oracle_run(rep, done)
        assert np.array_equal(ids, oids) and same_bits(st, ost), f"replica {i}"
