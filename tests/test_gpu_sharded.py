"""One field split over two ranks by column strips, each rank's local field on
the GPU through the C ABI (krabmaga_gb300/sharded.py, GpuStrip), as a gloo
process group of two processes on the same GPU (the ranks' kernels never wait
on one another: every exchange is a host message between steps).  The owned
boids of both ranks equal the single GPU field bit for bit in fast arithmetic
and the oracle in strict arithmetic."""
import ctypes as C
import os
import socket
import sys

import numpy as np
import pytest

import krabmaga_gb300 as kg
import oracle
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
D = float(np.float32(10.0) / np.float32(1.5))
CASE = (20000, 894.43, 13, 10, 2.0)  # boids, side (density 0.025), seed, steps, jump


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, arith, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import krabmaga_gb300 as kg
    from krabmaga_gb300.sharded import ShardedFlock

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n, side, seed, steps, jump = CASE
        ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
        p = kg.FlockParams(seed=seed, jump=jump, arith=arith)
        sf = ShardedFlock(side, D, p, ids, xy, dxy, device="cpu", gpu=0)
        sf.run(0, steps)
        got = sf.gather_state()
        sf.close()
        if rank == 0:
            q.put((got[0], got[1]))
    finally:
        dist.destroy_process_group()


def _sharded(arith):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, arith, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=600)
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    return got


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_two_gpu_strips_equal_the_single_gpu_field(gpu):
    n, side, seed, steps, jump = CASE
    gids, gst = _sharded(kg.KB_ARITH_FAST)
    ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
    f = kg.Field2D(side, side, D, True, capacity_hint=n)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    p = kg.FlockParams(seed=seed, jump=jump, arith=kg.KB_ARITH_FAST)
    L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(0), C.c_uint32(steps))
    sids, sst = f.get_state()
    f.close()
    assert np.array_equal(gids, sids) and _same(gst, sst)


def test_two_gpu_strips_equal_the_oracle_strict(gpu):
    n, side, seed, steps, jump = CASE
    gids, gst = _sharded(kg.KB_ARITH_STRICT)
    ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
    o = oracle.OracleField(side, side, D, True)
    o.set_many(ids, xy, dxy)
    o.lazy_update()
    o.flock_run(oracle.params_from(kg.FlockParams(seed=seed, jump=jump)), 0, steps)
    oids, ost, _ = o.iter(1)
    assert np.array_equal(gids, oids) and _same(gst, ost)


def _device_ranks(world, arith, case=CASE):
    """Every rank's strip on this GPU with its records kept on the device
    (GpuStripDevice), the ranks driven in this process: prepare on each,
    then finish with the device tensors each rank was sent."""
    from krabmaga_gb300.sharded import ShardedFlock

    n, side, seed, steps, jump = case
    ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
    p = kg.FlockParams(seed=seed, jump=jump, arith=arith)
    ranks = [ShardedFlock(side, D, p, ids, xy, dxy, device="cuda", gpu=0, rank=r, world=world)
             for r in range(world)]
    sent = 0
    for k in range(steps):
        parts = [sf.prepare(k) for sf in ranks]
        assert all(t.is_cuda for pr in parts for t in pr)
        sent += sum(int(parts[s][r].shape[0]) for s in range(world) for r in range(world) if r != s)
        for r, sf in enumerate(ranks):
            sf.finish([parts[s][r] for s in range(world)])
    own = [sf.owned_state() for sf in ranks]
    for sf in ranks:
        sf.close()
    return np.concatenate([o[0] for o in own]), np.concatenate([o[1] for o in own]), sent


@pytest.mark.parametrize("world", [2, 3])
def test_device_resident_strips_equal_the_single_gpu_field(gpu, world):
    n, side, seed, steps, jump = CASE
    for arith in (kg.KB_ARITH_FAST, kg.KB_ARITH_STRICT):
        gids, gst, sent = _device_ranks(world, arith)
        assert sent > 0  # halo and migration records crossed ranks
        ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
        f = kg.Field2D(side, side, D, True, capacity_hint=n)
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        p = kg.FlockParams(seed=seed, jump=jump, arith=arith)
        L.call("kb_flock_step", f.handle, C.byref(p.to_c()), C.c_uint64(0), C.c_uint32(steps))
        sids, sst = f.get_state()
        f.close()
        assert np.array_equal(gids, sids) and _same(gst, sst)


def test_device_record_entry_points_match_the_host_ones(gpu):
    """kb_field_copy_read_buffer / kb_flock_next_states_device /
    kb_field_set_states_device against get_state / compute_agents /
    set_locations on the same flock."""
    import torch

    n, side, seed = 3000, 346.41, 5
    ids, xy, dxy = kg.gen_uniform(n, side, side, seed, 1.0)
    p = kg.FlockParams(seed=seed, jump=2.0)
    f = kg.Field2D(side, side, D, True, capacity_hint=n)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    hid, hst = f.get_state()
    did, dst = f.read_buffer_device()
    assert np.array_equal(did.cpu().numpy().view(np.uint32), hid)
    assert _same(dst.cpu().numpy(), hst)
    # next states of every other boid, on the device and through the write buffer
    sel = np.arange(0, n, 2)
    out = f.next_states_device(p, 3, did[sel].contiguous(), dst[sel].contiguous()).cpu().numpy()
    g = kg.Field2D(side, side, D, True, capacity_hint=n)
    g.set_locations(ids, xy, dxy)
    g.lazy_update()
    g.flock_compute_agents(p, 3, hid[sel], hst[sel])
    found, want = g.get_locations(hid[sel], buffered=False)
    assert found.all() and _same(out, want)
    # records set from the device make the same read buffer as from the host
    h = kg.Field2D(side, side, D, True, capacity_hint=n)
    h.set_states_device(did.flip(0).contiguous(), dst.flip(0).contiguous())
    h.lazy_update()
    k = kg.Field2D(side, side, D, True, capacity_hint=n)
    k.set_locations(hid[::-1], hst[::-1, :2], hst[::-1, 2:])
    k.lazy_update()
    a, b = h.get_state(), k.get_state()
    assert np.array_equal(a[0], b[0]) and _same(a[1], b[1])
    # a record outside the bag matrix is refused and the write buffer is left as it was
    bad = dst[:4].clone()
    bad[2, 0] = -5.0
    with pytest.raises(L.KbError):
        h.set_states_device(did[:4].contiguous(), bad)
    h.lazy_update()
    assert h.num_objects() == 0
    # an output shorter than the read buffer is refused with the length reported
    n_out = C.c_size_t()
    small_st = torch.empty((10, 4), dtype=torch.float32, device=dst.device)
    small_id = torch.empty(10, dtype=torch.int32, device=dst.device)
    with pytest.raises(L.KbError):
        L.call("kb_field_copy_read_buffer", f.handle, C.c_void_p(small_st.data_ptr()),
               C.c_void_p(small_id.data_ptr()), C.c_size_t(10), C.byref(n_out))
    assert n_out.value == n
    # empty calls are no-ops
    L.call("kb_field_set_states_device", f.handle, C.c_size_t(0), None, None)
    L.call("kb_flock_next_states_device", f.handle, C.byref(p.to_c()), C.c_uint64(0),
           C.c_size_t(0), None, None, None)
    assert f.num_objects() == n
    for fld in (f, g, h, k):
        fld.close()


def test_device_discretize_matches_the_reference_rounding(gpu):
    """discretize_device on the GPU is floor(fl(v / d)) bit for bit at bag
    edges (k * d and its neighbouring floats), where a product with the
    reciprocal of d can land on the other side."""
    import torch

    from krabmaga_gb300.sharded import discretize, discretize_device

    d = np.float32(D)
    k = np.arange(1, 2000, dtype=np.float32)
    edge = (k * d).astype(np.float32)
    vals = np.concatenate([edge, np.nextafter(edge, np.float32(0)), np.nextafter(edge, np.float32(1e9)),
                           np.random.default_rng(1).random(5000).astype(np.float32) * 6000])
    got = discretize_device(torch.from_numpy(vals).cuda(), float(d)).cpu().numpy()
    want = discretize(vals, float(d))
    assert np.array_equal(got, want)
    # the reciprocal product disagrees somewhere on these edges, so the test can tell them apart
    rec = np.floor(vals * (np.float32(1) / d)).astype(np.int64)
    assert (rec != want).any()
