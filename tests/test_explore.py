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
