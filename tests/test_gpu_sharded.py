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
