"""kb_field_neighbor_digest_noalloc through the C ABI on the GPU.

The no-alloc entry point stages its queries and results in one fixed device
array per device instead of per-call buffers.  Its counts and digests must
equal those of kb_field_neighbor_digest (integer outputs: bit-exact) on two
calls in a row, the second one smaller than the first so that the array still
holds the first call's leftovers.  Collected last so that it also runs after
every other GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

import krabmaga_gb300 as kg
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu

N = 50_000
SIDE = float(np.sqrt(N / 0.025))          # density 0.025, as the Flockers benchmark
D = float(np.float32(10.0) / np.float32(1.5))


def _noalloc(field, kind, dist, q):
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, 2)
    counts = np.full(max(len(q), 1), 0xDEADBEEF, np.uint32)
    dig = np.full(max(len(q), 1), 0xDEADBEEF, np.uint32)
    L.call("kb_field_neighbor_digest_noalloc", field.handle, C.c_int32(kind), C.c_float(dist),
           C.c_size_t(len(q)), L.fptr(q), L.uptr(counts), L.uptr(dig))
    return counts[: len(q)], dig[: len(q)]


def _flock(steps):
    ids, xy, dxy = kg.gen_uniform(N, SIDE, SIDE, 31, 1.0)
    f = kg.Field2D(SIDE, SIDE, D, True)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    if steps:
        p = kg.FlockParams(seed=9)
        L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(1), C.c_uint32(steps))
    return f


@pytest.mark.parametrize("kind", [L.KB_QUERY_RELAX, L.KB_QUERY_EXACT])
def test_noalloc_digest_matches_allocating_entry_point(gpu, kind):
    f = _flock(steps=3)
    try:
        ids, st = f.get_state()
        rng = np.random.default_rng(17 + kind)
        # call 1: every boid's own position plus random points, 60,000 queries
        q1 = np.concatenate([st[:, :2], rng.uniform(0, SIDE, (10_000, 2))]).astype(np.float32)
        # call 2 (right after): 7,000 other points; slots past 7,000 keep call 1's data
        q2 = rng.uniform(0, SIDE, (7_000, 2)).astype(np.float32)
        n1, d1 = _noalloc(f, kind, 10.0, q1)
        n2, d2 = _noalloc(f, kind, 10.0, q2)
        e1, g1 = f.neighbor_digest(kind, 10.0, q1)
        e2, g2 = f.neighbor_digest(kind, 10.0, q2)
        assert np.array_equal(n1, e1) and np.array_equal(d1, g1)
        assert np.array_equal(n2, e2) and np.array_equal(d2, g2)
        assert n1[:N].min() >= 1          # a boid always finds itself
        assert f.device_flags() == 0
    finally:
        f.close()


def test_noalloc_after_steps_and_at_the_limit(gpu):
    f = _flock(steps=0)
    try:
        p = kg.FlockParams(seed=4)
        L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(1), C.c_uint32(2))
        # the read buffer is materialised by the no-alloc call itself here
        q = np.random.default_rng(3).uniform(0, SIDE, (L.KB_NOALLOC_MAX_QUERIES, 2))
        a = _noalloc(f, L.KB_QUERY_RELAX, 10.0, q)
        b = f.neighbor_digest(L.KB_QUERY_RELAX, 10.0, q)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        e = _noalloc(f, L.KB_QUERY_RELAX, 10.0, q[:0])
        assert len(e[0]) == 0
    finally:
        f.close()


def test_noalloc_rejects_more_than_its_staging_array(gpu):
    f = _flock(steps=0)
    try:
        q = np.zeros((L.KB_NOALLOC_MAX_QUERIES + 1, 2), np.float32)
        with pytest.raises(L.KbError) as err:
            _noalloc(f, L.KB_QUERY_RELAX, 10.0, q)
        assert err.value.status == L.KB_ERR_ARG
        assert "split" in str(err.value)
        # the field is untouched and the entry point still works
        a = _noalloc(f, L.KB_QUERY_RELAX, 10.0, q[:100])
        b = f.neighbor_digest(L.KB_QUERY_RELAX, 10.0, q[:100])
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    finally:
        f.close()


def test_noalloc_call_makes_no_device_allocation(gpu):
    """The promise itself: no device allocation or free by the library (its
    own counter of every cudaMalloc / cudaFree it makes), none by torch's
    allocator, and the device's free memory unchanged.  The first call here
    also materialises a read buffer left virtual by tiled steps."""
    import torch

    f = _flock(steps=0)
    g = _flock(steps=0)
    try:
        # tiled steps leave the read buffer virtual (the last write list plus offsets)
        f.set_step_options(2)
        p = kg.FlockParams(seed=5)
        L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(1), C.c_uint32(4))
        f.synchronize()
        q = np.random.default_rng(8).uniform(0, SIDE, (20_000, 2)).astype(np.float32)
        torch.cuda.synchronize()
        a0 = L.allocation_counts()
        t0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
        n1, d1 = _noalloc(f, L.KB_QUERY_RELAX, 10.0, q)
        assert L.allocation_counts() == a0
        # a second field's queries, once the array and both query kernels are
        # loaded on this device (module loading is not an allocation of the call)
        _noalloc(g, L.KB_QUERY_RELAX, 10.0, q)
        _noalloc(g, L.KB_QUERY_EXACT, 10.0, q)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        a1 = L.allocation_counts()
        n2, d2 = _noalloc(g, L.KB_QUERY_EXACT, 10.0, q)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert L.allocation_counts() == a1 == a0
        assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == t0
        # and the results are still those of the allocating entry point
        e1, g1 = f.neighbor_digest(L.KB_QUERY_RELAX, 10.0, q)
        e2, g2 = g.neighbor_digest(L.KB_QUERY_EXACT, 10.0, q)
        assert np.array_equal(n1, e1) and np.array_equal(d1, g1)
        assert np.array_equal(n2, e2) and np.array_equal(d2, g2)
    finally:
        f.close()
        g.close()
