"""The N > 1 path on CPU (gloo, world size 2): the step does not shard, so
every rank runs its own replica ("replicas only"); the only collectives are
the barriers around the timed region and the max of the ranks' times.
Under torchrun the reference arm runs on rank 0 alone and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    ws, r, local = bench.dist_setup()
    bench.barrier(ws)
    got = bench.allmax(ws, 1.5 + r)  # rank 1 is the slowest
    bench.barrier(ws)
    q.put((r, ws, local, got))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--workload", "flock1k", "--steps", "2", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    # rank 0 alone runs the one-core CPU arm: one GPU's worth of work
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["ranks"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_does_not_load_the_gpu_library():
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'flock1k', "
            "'--steps', '2', '--warmup', '0']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('GPU_LIB_LOADED' if 'libkrabgpu' in maps else 'GPU_LIB_ABSENT'); "
            "print('ORACLE_LOADED' if 'libkrab_oracle' in maps else 'ORACLE_ABSENT')")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "GPU_LIB_ABSENT" in r.stdout and "ORACLE_LOADED" in r.stdout
