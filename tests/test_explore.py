"""The exploration adapter's host logic (no GPU): the configuration table of
build_configurations! (lib.rs:1724-1749), the two explore modes, and the CSV
layout of build_dataframe! / write_csv (model_exploration.rs:451-520,
lib.rs:1781-1792)."""
import csv
import importlib
import itertools
import os

import pytest

import krabmaga_gb300 as kg
ex = importlib.import_module("krabmaga_gb300.explore")  # the module (the package exports the function)


def reference_table(n_conf, inputs):
    # a line-by-line transcription of the macro's loops: each row gets n_conf
    # blocks of `rep` equal indices, of which the first n_conf are used
    table = []
    rep = n_conf
    for values in inputs:
        row = []
        size = len(values)
        rep //= size
        i = 0
        for _ in range(n_conf):
            for _ in range(rep):
                row.append(i)
            i = (i + 1) % size
        table.append(row[:n_conf])
    return table


@pytest.mark.parametrize("sizes", [[2, 3], [3, 1, 2], [4], [2, 2, 2, 2]])
def test_configuration_table_matches_the_macro(sizes):
    inputs = [list(range(s)) for s in sizes]
    n = 1
    for s in sizes:
        n *= s
    got = kg.build_configurations(n, inputs)
    assert got == reference_table(n, inputs)
    # the first input varies slowest: the cartesian product in input order
    combos = [tuple(got[m][i] for m in range(len(sizes))) for i in range(n)]
    assert combos == list(itertools.product(*inputs))


def test_unknown_names_are_rejected():
    with pytest.raises(ValueError):
        ex._apply(ex.FlockerConfig(), "gravity", 1.0)
    with pytest.raises(ValueError):
        kg.explore(10, 1, {"cohesion": [1.0]}, ["temperature"])


def test_matched_mode_needs_equal_lengths():
    with pytest.raises(ValueError):
        kg.explore(10, 1, {"cohesion": [1.0, 2.0], "jump": [0.5]}, ["order"],
                   kg.ExploreMode.Matched)


def test_inputs_reach_the_replica():
    cfg = ex.FlockerConfig(initial_flockers=50, dim=100.0)
    cfg = ex._apply(cfg, "neighbor_radius", 12.0)
    cfg = ex._apply(cfg, "initial_flockers", 70)
    r = ex._replica(cfg, seed=5)
    assert r.n == 70 and r.params.neighbor_radius == 12.0 and r.params.seed == 5
    assert r.discretization == pytest.approx(8.0)


def test_csv_layout(tmp_path):
    rows = [{"Simulation": 0, "Run": 0, "cohesion": 1.0, "initial_flockers": 300,
             "order": 0.25, "Run Duration": 0.5, "Step per sec": 2000.0},
            {"Simulation": 0, "Run": 1, "cohesion": 1.0, "initial_flockers": 300,
             "order": 0.125, "Run Duration": 0.5, "Step per sec": 2000.0}]
    path = kg.write_csv(os.path.join(tmp_path, "exp"), rows)
    assert path.endswith("exp.csv")
    with open(path) as fh:
        got = list(csv.reader(fh))
    assert got[0] == ["Simulation", "Run", "cohesion", "initial_flockers", "order",
                      "Run Duration", "Step per sec"]
    # inputs/outputs as Rust's {:?} (1.0 keeps its fraction), the timings as
    # f32 to_string() (2000 has none)
    assert got[1] == ["0", "0", "1.0", "300", "0.25", "0.5", "2000"]
    assert got[2][4] == "0.125"


# bayesian_search! (src/explore/bayesian.rs) on the host: the reference's own
# doc example, x^2 + y^2 minimised by maximising its negative, both patterns


def _init():
    return [[-2.0, -2.0], [8.0, 1.0], [-1.0, 5.0], [4.0, -2.0]]


def _objective_square(x):
    return -1.0 * (x[0] ** 2 + x[1] ** 2)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_bayesian_search_optional_pattern_finds_the_minimum(seed):
    ex = importlib.import_module("krabmaga_gb300.explore")
    x, y = ex.bayesian_search(_init, _objective_square, 2, 20, batch_size=500, scale=10.0,
                              seed=seed)
    assert abs(x[0]) < 1.0 and abs(x[1]) < 1.0
    assert y == _objective_square(x)


def test_bayesian_search_main_pattern_and_its_parts():
    import numpy as np
    ex = importlib.import_module("krabmaga_gb300.explore")

    def gen(xs):
        return np.random.default_rng(len(xs)).uniform(-10.0, 10.0, (500, 2))

    x, y = ex.bayesian_search(_init, _objective_square, gen, 20)
    assert abs(x[0]) < 1.0 and abs(x[1]) < 1.0
    # the surrogate interpolates its samples; expected improvement is 0 where
    # the variance is 0 and positive elsewhere; the acquisition takes the max
    pts = np.array(_init(), float)
    vals = [_objective_square(p) for p in pts]
    gp = ex.GaussianProcess(pts, vals)
    assert np.allclose(gp.predict(pts), vals, atol=1e-3 * max(abs(v) for v in vals))
    assert gp.predict_variance(pts).max() < 1e-3 * np.var(vals)
    cand = ex.generate_samples(50, 10.0, 2, np.random.default_rng(0))
    ei = ex.expected_improvement(pts, cand, gp)
    assert (ei >= 0).all() and ei.max() > 0
    assert np.array_equal(ex.acquisition_function(pts, cand, gp), cand[int(np.argmax(ei))])


def test_gen_param_as_the_macro():
    import numpy as np
    ex = importlib.import_module("krabmaga_gb300.explore")
    rng = np.random.default_rng(1)
    u = ex.gen_param(int, 0, 10, 5, rng)
    assert len(u) == 5 and all(isinstance(v, int) and 0 <= v < 10 for v in u)
    f = ex.gen_param(float, 10.0, 0.0, 50, rng)          # a reversed range is swapped
    assert len(f) == 50 and all(0.0 <= v < 10.0 for v in f)
    assert ex.gen_param(int, 3, 3, 4, rng) == [3, 3, 3, 3]  # an empty range widens by 1
    assert ex.gen_param(float, 0.0, 1.0, 0, rng) == []
    assert len(ex.gen_param(float, 0.0, 1.0)) == 1


def test_load_csv_columns_by_position(tmp_path):
    ex = importlib.import_module("krabmaga_gb300.explore")
    p = tmp_path / "params.csv"
    p.write_text("cohesion,jump,n\n0.5,0.7,100\n1.5,0.9,200\n")
    coh, jump, n = ex.load_csv(str(p), ("cohesion", float), ("jump", float), ("n", int))
    assert coh == [0.5, 1.5] and jump == [0.7, 0.9] and n == [100, 200]


# ---------------------------------------------------------------- search loops
# The drivers' host loops against the reference's, with the device batch
# replaced by a fake: each run's moments row is a function of its replica's
# parameters and seed ({boids, n*jump, 0, n*jump}: order 1, mean_speed jump).
class FakeRunner:
    def __init__(self):
        self.calls = []  # one list of (jump, cohesion, seed) per device batch

    def __call__(self, replicas, nstep, device):
        import numpy as np
        self.calls.append([(r.params.jump, r.params.cohesion, r.params.seed) for r in replicas])
        rows = []
        for r in replicas:
            n = float(r.state[0].shape[0])
            rows.append([n, n * r.params.jump, 0.0, n * r.params.jump])
        return np.array(rows, np.float64)


@pytest.fixture
def fake_runner(monkeypatch):
    fake = FakeRunner()
    monkeypatch.setattr(ex, "_run_batch", fake)
    return fake


def test_random_search_loop_as_the_macro(fake_runner):
    # random_search.rs:44-118: batch_size samples from the best so far, each
    # run reps times; the mean cost per sample; keep the lowest; stop at target
    import numpy as np
    base = kg.FlockerConfig(initial_flockers=40, dim=30.0, init_seed=100)
    jumps = iter([0.9, 0.8, 0.95, 0.61, 0.7, 0.59, 0.9, 0.9, 0.9])

    def gen(best, rng):
        return ex._apply(best, "jump", next(jumps))

    def cost(obs):
        return abs(obs["mean_speed"] - 0.6)

    best, c, hist = kg.random_search(base, 5, 0.015, cost, gen, batch_size=3, step=7, reps=2)
    # iteration 1: best 0.8 (0.2); iteration 2: 0.61 (0.01 <= target): stop
    assert len(fake_runner.calls) == 2 and len(hist) == 2
    assert best.params.jump == 0.61 and c == pytest.approx(0.01, abs=1e-6)
    assert hist[0] == pytest.approx(0.2, abs=1e-6) and hist[1] == c
    # one device batch per iteration, batch_size * reps runs; run k seeded init_seed + k
    seeds = [s for call in fake_runner.calls for (_, _, s) in call]
    assert seeds == list(range(100, 100 + 12))
    assert [j for (j, _, _) in fake_runner.calls[0]] == [0.9, 0.9, 0.8, 0.8, 0.95, 0.95]
    # an unreachable target runs every iteration and the history never rises
    jumps = iter(np.linspace(1.0, 0.3, 12).tolist())
    _, _, hist = kg.random_search(base, 4, -1.0, cost, gen, batch_size=3, step=7, reps=1)
    assert len(hist) == 4 and all(b <= a for a, b in zip(hist, hist[1:]))


def _ga(fake_runner, desired, generations, survivors=2):
    base = kg.FlockerConfig(initial_flockers=30, dim=25.0, init_seed=5)
    log = []

    def init_population():
        return [0.3, 0.5, 0.7, 0.9]

    def make_config(ind, r):
        return ex._apply(base, "jump", ind)

    def fitness(obs):
        return float(sum(o["mean_speed"] for o in obs) / len(obs))

    def selection(pop):
        log.append(("selection", [i for i, _ in pop]))
        pop.sort(key=lambda t: -t[1])
        del pop[survivors:]

    def crossover(population):
        log.append(("crossover", list(population)))
        population.append(round((population[0] + population[-1]) / 2, 6) if population else 0.0)

    def mutation(ind):
        log.append(("mutation", ind))
        return round(min(1.0, ind + 0.01), 6)

    rows = kg.evolutionary_search(init_population, make_config, fitness, selection, mutation,
                                  crossover, lambda a, b: a >= b, desired, generations, step=3,
                                  reps=2, init_seed=base.init_seed)
    return rows, log


def test_evolutionary_search_loop_as_the_macro(fake_runner):
    # genetic.rs:626-826: evaluate, stop on the desired fitness, else
    # selection, crossover of the survivors, then mutation of every individual
    rows, log = _ga(fake_runner, 5.0, 3)
    assert [r["generation"] for r in rows] == [1] * 4 + [2] * 3 + [3] * 3
    assert [r["index"] for r in rows] == [0, 1, 2, 3, 0, 1, 2, 0, 1, 2]
    assert [r["individual"] for r in rows[:4]] == [0.3, 0.5, 0.7, 0.9]
    assert [r["fitness"] for r in rows[:4]] == pytest.approx([0.3, 0.5, 0.7, 0.9], abs=1e-6)
    # selection keeps the two fittest; crossover appends their mean; each is mutated
    assert log[0] == ("selection", [0.3, 0.5, 0.7, 0.9])
    assert log[1] == ("crossover", [0.9, 0.7])
    assert [e for e in log[2:5]] == [("mutation", 0.9), ("mutation", 0.7), ("mutation", 0.8)]
    assert [r["individual"] for r in rows[4:7]] == [0.91, 0.71, 0.81]
    # the generation limit is checked at the top of the loop (genetic.rs:674-678), so
    # selection runs after the last generation too; runs seeded init_seed + k in order
    assert sum(1 for e in log if e[0] == "selection") == 3
    seeds = [s for call in fake_runner.calls for (_, _, s) in call]
    assert seeds == list(range(5, 5 + 2 * 10))


def test_evolutionary_search_stops_on_the_desired_fitness(fake_runner):
    rows, log = _ga(fake_runner, 0.85, 0)  # generation_num 0: no limit
    assert {r["generation"] for r in rows} == {1} and len(rows) == 4 and log == []


def test_evolutionary_search_stops_when_selection_empties_the_population(fake_runner):
    rows, log = _ga(fake_runner, 5.0, 4, survivors=0)
    assert {r["generation"] for r in rows} == {1}
    assert [e[0] for e in log] == ["selection"]


def test_explore_rows_as_the_macro(monkeypatch):
    # every run of every configuration in one device batch (faked here); the
    # rows in configuration order (first input slowest), runs 0-based, run k
    # of configuration i seeded init_seed + i * rep_conf + k
    import numpy as np
    seen = []

    def fake(replicas, nstep, device):
        seen.append([(r.params.jump, r.n, r.params.seed) for r in replicas])
        m = np.array([[r.n, r.n * r.params.jump, 0.0, r.n * r.params.jump] for r in replicas], float)
        return m, 0.5

    monkeypatch.setattr(ex, "_run_batch_timed", fake)
    base = kg.FlockerConfig(initial_flockers=20, dim=30.0, init_seed=9)
    rows = kg.explore(40, 2, {"jump": [0.3, 0.6], "initial_flockers": [10, 20, 30]},
                      ["mean_speed", "boids"], base=base)
    assert len(seen) == 1 and len(seen[0]) == 12 and len(rows) == 12
    assert [(r["Simulation"], r["Run"], r["jump"], r["initial_flockers"]) for r in rows[:4]] == \
        [(0, 0, 0.3, 10), (0, 1, 0.3, 10), (1, 0, 0.3, 20), (1, 1, 0.3, 20)]
    assert (rows[-1]["Simulation"], rows[-1]["jump"], rows[-1]["initial_flockers"]) == (5, 0.6, 30)
    for r in rows:
        assert r["mean_speed"] == pytest.approx(r["jump"]) and r["boids"] == r["initial_flockers"]
        assert r["Run Duration"] == 0.5 and r["Step per sec"] == 80.0
        assert list(r)[:2] == ["Simulation", "Run"]
    assert [s for (_, _, s) in seen[0]] == list(range(9, 21))
    # the matched mode pairs the inputs by position
    rows = kg.explore(5, 1, {"jump": [0.3, 0.6], "initial_flockers": [10, 20]}, ["boids"],
                      mode=ex.ExploreMode.Matched, base=base)
    assert [(r["jump"], r["initial_flockers"], r["boids"]) for r in rows] == [(0.3, 10, 10), (0.6, 20, 20)]
