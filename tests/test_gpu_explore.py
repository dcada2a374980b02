"""The exploration adapter on the GPU: every row of an exhaustive exploration
equals the same run done alone on a plain field, with the observable
computed on the host from its final state."""
import ctypes as C
import importlib

import numpy as np
import pytest

import krabmaga_gb300 as kg
from krabmaga_gb300 import _lib as L

pytestmark = pytest.mark.gpu
ex = importlib.import_module("krabmaga_gb300.explore")


def host_order(st):
    d = st[:, 2:].astype(np.float64)
    return float(np.hypot(d[:, 0].sum(), d[:, 1].sum()) / np.hypot(d[:, 0], d[:, 1]).sum())


def test_exhaustive_rows_equal_single_runs(gpu, tmp_path):
    base = kg.FlockerConfig(initial_flockers=400, dim=130.0, init_seed=100,
                            params=kg.FlockParams(arith=kg.KB_ARITH_STRICT))
    inputs = {"cohesion": [0.5, 1.5], "neighbor_radius": [8.0, 12.0]}
    rows = kg.explore(25, 2, inputs, ["order", "mean_speed", "boids"], kg.ExploreMode.Exaustive,
                      base)
    assert len(rows) == 8
    assert [(r["Simulation"], r["Run"]) for r in rows] == [(i, j) for i in range(4) for j in range(2)]
    assert [(r["cohesion"], r["neighbor_radius"]) for r in rows[::2]] == \
        [(0.5, 8.0), (0.5, 12.0), (1.5, 8.0), (1.5, 12.0)]
    for k, r in enumerate(rows):
        cfg = base
        for name in inputs:
            cfg = ex._apply(cfg, name, r[name])
        rep = ex._replica(cfg, base.init_seed + k)
        f = kg.Field2D(rep.width, rep.height, rep.discretization, True)
        f.set_locations(*rep.state)
        f.lazy_update()
        L.call("kb_flock_step", f.handle, C.byref(rep.params.to_c()), C.c_uint64(0), C.c_uint32(25))
        _, st = f.get_state()
        assert r["boids"] == 400
        assert r["order"] == pytest.approx(host_order(st), rel=1e-9)
        m = f.moments()
        assert m[0] == 400 and r["mean_speed"] == pytest.approx(m[3] / 400, rel=1e-12)
        f.close()
    assert rows[0]["Step per sec"] > 0
    path = kg.write_csv(str(tmp_path / "flockers"), rows)
    assert open(path).readline().strip() == \
        "Simulation,Run,cohesion,neighbor_radius,order,mean_speed,boids,Run Duration,Step per sec"


def test_matched_mode(gpu):
    rows = kg.explore(10, 1, {"jump": [0.3, 0.9], "initial_flockers": [200, 500]}, ["boids"],
                      kg.ExploreMode.Matched, kg.FlockerConfig(dim=100.0))
    assert [(r["jump"], r["initial_flockers"], r["boids"]) for r in rows] == \
        [(0.3, 200, 200), (0.9, 500, 500)]


def test_random_search_keeps_the_best_and_stops_at_target(gpu):
    base = kg.FlockerConfig(initial_flockers=300, dim=110.0, init_seed=7,
                            params=kg.FlockParams(arith=kg.KB_ARITH_STRICT))

    def gen(best, rng):
        return ex._apply(ex._apply(best, "cohesion", float(rng.uniform(0.2, 2.0))),
                         "jump", float(rng.uniform(0.3, 1.0)))

    def cost(obs):  # seek a disordered flock
        return obs["order"]

    best, c, hist = kg.random_search(base, 4, -1.0, cost, gen, batch_size=3, step=15, reps=2,
                                     seed=3)
    assert len(hist) == 4 and all(b >= a for a, b in zip(hist[1:], hist[:-1]))
    assert c == hist[-1]
    # the reported cost is the mean over its runs, recomputed alone here
    # recompute every sample of the search, in the same order, one run at a time
    rng = np.random.default_rng(3)
    b_cur, b_cost, run = base, float(np.finfo(np.float32).max), 0
    for it in range(4):
        batch = [gen(b_cur, rng) for _ in range(3)]
        costs = []
        for smp in batch:
            vals = []
            for r in range(2):
                rep = ex._replica(smp, base.init_seed + run)
                run += 1
                f = kg.Field2D(rep.width, rep.height, rep.discretization, True)
                f.set_locations(*rep.state)
                f.lazy_update()
                L.call("kb_flock_step", f.handle, C.byref(rep.params.to_c()), C.c_uint64(0),
                       C.c_uint32(15))
                _, st = f.get_state()
                vals.append(host_order(st))
                f.close()
            costs.append(float(np.mean(vals)))
        k = int(np.argmin(costs))
        if costs[k] < b_cost:
            b_cur, b_cost = batch[k], costs[k]
        assert hist[it] == pytest.approx(b_cost, rel=1e-9)
    assert best == b_cur
    # a target that the first iteration already meets stops the search
    _, cost2, hist2 = kg.random_search(base, 5, 10.0, cost, gen, batch_size=2, step=5, reps=1)
    assert len(hist2) == 1 and cost2 <= 10.0


def test_evolutionary_search_rows_equal_single_runs(gpu):
    base = kg.FlockerConfig(initial_flockers=250, dim=100.0, init_seed=40,
                            params=kg.FlockParams(arith=kg.KB_ARITH_STRICT))
    rng = np.random.default_rng(9)

    def init_population():
        return [f"{c:.3f};{j:.3f}" for c, j in zip(rng.uniform(0.3, 1.8, 4), rng.uniform(0.3, 1.0, 4))]

    def make_config(ind, r):
        c, j = (float(v) for v in ind.split(";"))
        return ex._apply(ex._apply(base, "cohesion", c), "jump", j)

    def fitness(obs):
        return float(np.mean([o["order"] for o in obs]))

    def selection(pop):
        pop.sort(key=lambda t: -t[1])
        del pop[2:]

    def crossover(population):
        a, b = population[0].split(";"), population[1].split(";")
        population.extend([f"{a[0]};{b[1]}", f"{b[0]};{a[1]}"])

    def mutation(ind):
        c, j = (float(v) for v in ind.split(";"))
        return f"{min(2.0, c * 1.05):.3f};{j:.3f}"

    rows = kg.evolutionary_search(init_population, make_config, fitness, selection, mutation,
                                  crossover, lambda a, b: a > b, 2.0, 3, step=12, reps=2,
                                  init_seed=base.init_seed)
    assert [r["generation"] for r in rows] == [1] * 4 + [2] * 4 + [3] * 4
    # every row's fitness equals its runs done one at a time
    run = 0
    for r in rows:
        vals = []
        for k in range(2):
            rep = ex._replica(make_config(r["individual"], k), base.init_seed + run)
            run += 1
            f = kg.Field2D(rep.width, rep.height, rep.discretization, True)
            f.set_locations(*rep.state)
            f.lazy_update()
            L.call("kb_flock_step", f.handle, C.byref(rep.params.to_c()), C.c_uint64(0),
                   C.c_uint32(12))
            _, st = f.get_state()
            vals.append(host_order(st))
            f.close()
        assert r["fitness"] == pytest.approx(float(np.mean(vals)), rel=1e-9)
    # a desired fitness reached in the first generation stops the search there
    rows2 = kg.evolutionary_search(init_population, make_config, fitness, selection, mutation,
                                   crossover, lambda a, b: a > b, -1.0, 5, step=5, reps=1)
    assert {r["generation"] for r in rows2} == {1}


def test_bayesian_search_over_flock_runs(gpu):
    # the objective is a flock run on the device: the order parameter of two
    # runs of 40 steps as a function of the consistency weight
    import numpy as np
    ex = importlib.import_module("krabmaga_gb300.explore")
    base = kg.FlockerConfig(initial_flockers=400, dim=130.0)
    order = lambda obs: float(np.mean([o["order"] for o in obs]))
    f = ex.flock_objective(base, ["consistency"], order, step=40, reps=2, init_seed=3)
    g = ex.flock_objective(base, ["consistency"], order, step=40, reps=2, init_seed=3)
    assert f(np.array([1.0])) == g(np.array([1.0]))  # the same runs, the same value

    def gen(xs):
        return np.random.default_rng(len(xs)).uniform(0.0, 3.0, (64, 1))

    x, y = ex.bayesian_search(lambda: [[0.1], [2.0]], f, gen, 4)
    assert 0.0 <= x[0] <= 3.0 and 0.0 <= y <= 1.0


def _dist_rank(rank, world, port, q):
    import os
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank))
    sys.path.insert(0, root)
    import torch.distributed as dist

    import krabmaga_gb300 as kg

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rows = kg.explore_distributed(*_dist_args(), device=0)
        q.put((rank, rows))
    finally:
        dist.destroy_process_group()


def _dist_args():
    base = kg.FlockerConfig(initial_flockers=300, dim=110.0, init_seed=21,
                            params=kg.FlockParams(arith=kg.KB_ARITH_STRICT))
    return (15, 2, {"cohesion": [0.5, 1.0, 1.5], "jump": [0.4, 0.9]}, ["order", "mean_speed", "boids"],
            kg.ExploreMode.Exaustive, base)


def test_distributed_exploration_equals_the_single_process_rows(gpu):
    """explore_distributed on two ranks (two processes sharing this GPU, each
    running its own batch; a gloo group gathers the rows): rank 0's dataframe
    holds every single-process row, regrouped by rank in the reference's
    round-robin order, with the same outputs."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_dist_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs)
    single = kg.explore(*_dist_args())
    assert got[1] == [] and len(got[0]) == len(single) == 12
    expect = []
    for r in range(2):
        for i, g in enumerate(range(r, 6, 2)):
            for j in range(2):
                expect.append(dict(single[2 * g + j], Simulation=i))
    timing = ("Run Duration", "Step per sec")
    for a, b in zip(got[0], expect):
        assert {k: v for k, v in a.items() if k not in timing} == \
            {k: v for k, v in b.items() if k not in timing}
