"""The replicas-only sharding of an exploration (krabmaga_gb300.explore
.explore_distributed, after src/explore/mpi/model_exploration.rs:120-300) as
world-size-2 and -3 gloo process groups on the CPU.

Every rank's runs go through the oracle here (the sharding is host logic:
the round-robin assignment of configurations, the per-rank labels, the
gather to rank 0 in rank order).  Rank 0's dataframe must hold every row of
the single-process exploration, regrouped by rank, and every other rank an
empty list.  The GPU form is in tests/test_gpu_explore.py."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TIMING = ("Run Duration", "Step per sec")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def oracle_runner(replicas, nstep, device):
    """Each replica alone on the oracle; the moments the device batch reports
    (boids, sum dx, sum dy, sum |d| of the final headings, in double)."""
    import oracle

    mom = np.zeros((len(replicas), 4), np.float64)
    for k, r in enumerate(replicas):
        f = oracle.OracleField(r.width, r.height, r.discretization, r.toroidal)
        f.set_many(*r.state)
        f.lazy_update()
        f.flock_run(oracle.params_from(r.params), 0, nstep)
        _, st, _ = f.iter(1)
        d = st[:, 2:].astype(np.float64)
        mom[k] = (len(st), d[:, 0].sum(), d[:, 1].sum(), np.hypot(d[:, 0], d[:, 1]).sum())
    return mom, 1.0


CASES = {
    "exhaustive": dict(inputs={"cohesion": [0.5, 1.5], "neighbor_radius": [8.0, 12.0, 10.0]},
                       mode="Exaustive"),
    "matched": dict(inputs={"jump": [0.3, 0.5, 0.7, 0.9, 1.0], "avoidance": [1.0, 0.5, 1.5, 1.2, 0.8]},
                    mode="Matched"),
}


def _explore_args(case):
    import krabmaga_gb300 as kg

    c = CASES[case]
    base = kg.FlockerConfig(initial_flockers=120, dim=70.0, init_seed=40)
    return (4, 2, c["inputs"], ["order", "mean_speed", "boids"], getattr(kg.ExploreMode, c["mode"]),
            base)


def _rank_main(rank, world, port, case, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist

    import krabmaga_gb300 as kg
    from test_explore_distributed import _explore_args, oracle_runner

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rows = kg.explore_distributed(*_explore_args(case), device=0, runner=oracle_runner)
        q.put((rank, rows))
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
    got = dict(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs)
    return got


@pytest.mark.parametrize("world,case", [(2, "exhaustive"), (3, "matched"), (2, "matched")])
def test_rank_zero_gathers_every_row_in_rank_order(world, case):
    import krabmaga_gb300 as kg

    got = _run(world, case)
    single = kg.explore(*_explore_args(case), runner=oracle_runner)
    n_conf = len(single) // 2
    assert all(got[r] == [] for r in range(1, world))
    expect = []
    for r in range(world):
        for i, g in enumerate(range(r, n_conf, world)):  # rank r: configurations r, r + P, ...
            for j in range(2):
                row = dict(single[2 * g + j])
                row["Simulation"] = i  # the configuration's index on its rank
                expect.append(row)
    assert len(got[0]) == len(expect) == len(single)
    for a, b in zip(got[0], expect):
        assert {k: v for k, v in a.items() if k not in TIMING} == \
            {k: v for k, v in b.items() if k not in TIMING}


def _rank_edge(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist

    import krabmaga_gb300 as kg
    from test_explore_distributed import oracle_runner

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        base = kg.FlockerConfig(initial_flockers=80, dim=60.0, init_seed=5)
        # two configurations over three ranks (rank 2 gets none), rep_conf 0 counts as 1
        rows = kg.explore_distributed(3, 0, {"jump": [0.4, 0.8]}, ["boids"],
                                      kg.ExploreMode.Matched, base, device=0, runner=oracle_runner)
        q.put((rank, rows))
    finally:
        dist.destroy_process_group()


def test_fewer_configurations_than_ranks_and_zero_repetitions():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_edge, args=(r, 3, port, q)) for r in range(3)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=300) for _ in range(3))
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs)
    assert got[1] == [] and got[2] == []
    rows = got[0]
    assert [(r["Simulation"], r["Run"], r["jump"], r["boids"]) for r in rows] == \
        [(0, 0, 0.4, 80), (0, 0, 0.8, 80)]
