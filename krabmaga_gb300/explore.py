"""Model exploration on the device: the explore! / explore_parallel! macros
(src/explore/model_exploration.rs:56-151, 354-432) for the Flockers model.

Every run of every configuration becomes one replica of a single batch
(kb_batch_*), so a whole exploration advances in the same launches; the
outputs are flock observables reduced on the device (kb_batch_moments).
The dataframe has the reference's columns (build_dataframe!,
model_exploration.rs:451-520) and write_csv follows lib.rs:1781-1792.
random_search and evolutionary_search drive the same batches
(random_search.rs, genetic.rs).
"""
from __future__ import annotations

import csv
import enum
import time
from dataclasses import dataclass, field, replace
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L
from .batch import Batch, Replica
from .model import FlockParams, gen_uniform


class ExploreMode(enum.Enum):
    """lib.rs:481-486 (the reference's spelling)."""

    Exaustive = 0  # every combination of the inputs
    Matched = 1    # the i-th value of every input together


def build_configurations(n_conf: int, inputs: Sequence[Sequence]) -> List[List[int]]:
    """Index table of the exhaustive mode (lib.rs:1724-1749): row m holds, for
    configuration i, the index into input m.  The first input varies slowest
    and the last fastest (the cartesian product in input order)."""
    table = []
    rep = n_conf
    for values in inputs:
        size = len(values)
        rep //= size
        table.append([(i // rep) % size for i in range(n_conf)])
    return table


@dataclass
class FlockerConfig:
    """The non-swept part of a Flockers exploration.  Any field, or any
    FlockParams field, may be named as an input instead."""

    initial_flockers: int = 1000
    dim: float = 200.0                      # square torus side
    discretization: Optional[float] = None  # None: neighbor_radius / 1.5 (a 3x3 stencil)
    heading_scale: float = 1.0              # initial headings: unit vectors (0: the reference's zero)
    params: FlockParams = field(default_factory=FlockParams)
    init_seed: int = 0                      # run k (in row order) starts from Philox(init_seed + k)


_CONFIG_FIELDS = ("initial_flockers", "dim", "discretization", "heading_scale")
_PARAM_FIELDS = ("cohesion", "avoidance", "consistency", "randomness", "momentum", "jump",
                 "neighbor_radius")


def _order(m: np.ndarray) -> float:
    return float(np.hypot(m[1], m[2]) / m[3]) if m[3] > 0 else 0.0


# Output observables: name -> function of a replica's moments row
# {boids, sum dx, sum dy, sum |d|}.
OUTPUTS = {
    "order": _order,                                                # polar order parameter
    "mean_speed": lambda m: float(m[3] / m[0]) if m[0] else 0.0,    # mean |last_d|
    "mean_heading_x": lambda m: float(m[1] / m[0]) if m[0] else 0.0,
    "mean_heading_y": lambda m: float(m[2] / m[0]) if m[0] else 0.0,
    "boids": lambda m: int(m[0]),
}


def _apply(cfg: FlockerConfig, name: str, value) -> FlockerConfig:
    if name in _CONFIG_FIELDS:
        return replace(cfg, **{name: value})
    if name in _PARAM_FIELDS:
        return replace(cfg, params=replace(cfg.params, **{name: float(value)}))
    raise ValueError(f"unknown input {name!r}: one of {_CONFIG_FIELDS + _PARAM_FIELDS}")


def _replica(cfg: FlockerConfig, seed: int) -> Replica:
    side = float(np.float32(cfg.dim))
    d = cfg.discretization
    if d is None:
        d = float(np.float32(cfg.params.neighbor_radius) / np.float32(1.5))
    params = replace(cfg.params, seed=seed)
    state = gen_uniform(int(cfg.initial_flockers), side, side, seed, cfg.heading_scale)
    return Replica(side, side, float(d), params, state)


def _configurations(inputs: Dict[str, Sequence], outputs: Sequence[str], mode: ExploreMode,
                    base: FlockerConfig) -> Tuple[List[str], List[list], List[FlockerConfig]]:
    """The input names, each configuration's input values and its
    FlockerConfig, in the reference's configuration order."""
    names = list(inputs)
    values = [list(inputs[k]) for k in names]
    for o in outputs:
        if o not in OUTPUTS:
            raise ValueError(f"unknown output {o!r}: one of {sorted(OUTPUTS)}")
    if mode == ExploreMode.Exaustive:
        n_conf = int(np.prod([len(v) for v in values])) if values else 1
        table = build_configurations(n_conf, values)
        conf_values = [[values[m][table[m][i]] for m in range(len(names))] for i in range(n_conf)]
    else:
        lens = {len(v) for v in values}
        if len(lens) > 1:
            raise ValueError("ExploreMode.Matched needs inputs of equal length")
        n_conf = lens.pop() if lens else 1
        conf_values = [[v[i] for v in values] for i in range(n_conf)]
    conf_list = []
    for vals in conf_values:
        cfg = base
        for k, v in zip(names, vals):
            cfg = _apply(cfg, k, v)
        conf_list.append(cfg)
    return names, conf_values, conf_list


def _rows(confs: Sequence[int], labels: Sequence[int], rep_conf: int, names: Sequence[str],
          conf_values: Sequence[list], conf_list: Sequence[FlockerConfig], outputs: Sequence[str],
          nstep: int, base: FlockerConfig, device: int, runner: Optional[Callable]) -> List[dict]:
    """Run rep_conf runs of each configuration in confs as one batch; row k
    of configuration confs[i] is labelled Simulation labels[i], Run k.  Run
    k of configuration g starts from Philox(init_seed + g * rep_conf + k)."""
    if not confs:
        return []
    reps = [_replica(conf_list[g], base.init_seed + g * rep_conf + j)
            for g in confs for j in range(rep_conf)]
    mom, secs = (runner or _run_batch_timed)(reps, nstep, device)
    rows = []
    for i, g in enumerate(confs):
        for j in range(rep_conf):
            row = {"Simulation": labels[i], "Run": j}
            row.update({k: v for k, v in zip(names, conf_values[g])})
            m = mom[i * rep_conf + j]
            row.update({o: OUTPUTS[o](m) for o in outputs})
            row["Run Duration"] = secs
            row["Step per sec"] = nstep / secs if secs > 0 else float("inf")
            rows.append(row)
    return rows


def explore(nstep: int, rep_conf: int, inputs: Dict[str, Sequence], outputs: Sequence[str],
            mode: ExploreMode = ExploreMode.Exaustive, base: Optional[FlockerConfig] = None,
            device: int = 0, runner: Optional[Callable] = None) -> List[dict]:
    """Run every configuration rep_conf times for nstep steps, all runs as one
    device batch, and return the dataframe rows: "Simulation" (configuration
    index), "Run" (0-based, as explore_parallel!), the inputs, the outputs,
    "Run Duration" (seconds of the whole batch) and "Step per sec".

    With ExploreMode.Matched every input must have the same length.
    runner(replicas, nstep, device) -> (moments [nrep, 4], seconds) replaces
    the device batch (tests run the oracle there)."""
    base = base or FlockerConfig()
    names, conf_values, conf_list = _configurations(inputs, outputs, mode, base)
    n_conf = len(conf_list)
    if n_conf == 0 or rep_conf <= 0:
        return []
    return _rows(list(range(n_conf)), list(range(n_conf)), rep_conf, names, conf_values,
                 conf_list, outputs, nstep, base, device, runner)


def explore_distributed(nstep: int, rep_conf: int, inputs: Dict[str, Sequence],
                        outputs: Sequence[str], mode: ExploreMode = ExploreMode.Exaustive,
                        base: Optional[FlockerConfig] = None, group=None,
                        device: Optional[int] = None,
                        runner: Optional[Callable] = None) -> List[dict]:
    """explore_distributed_mpi! (src/explore/mpi/model_exploration.rs:120-300)
    over the ranks of a torch.distributed group, one GPU per rank: the
    replicas-only sharding of an exploration.

    As in the reference, rank r takes configurations r, r + P, r + 2P, ...
    (P ranks; the first n_conf % P ranks take one more), runs each of them
    rep_conf times (rep_conf <= 0 counts as 1), here all as one device batch
    on its GPU, and rank 0 gathers every rank's rows in rank order (the
    gather_varcount_into_root of the reference).  Rank 0 returns the whole
    dataframe, the other ranks an empty list.  "Simulation" is the
    configuration's index among its rank's configurations, as the reference
    writes it (conf_num = i); the input columns name the configuration.  A
    run starts from the same Philox stream as in explore, so every row equals
    the single-process row of the same configuration and run.

    device: this rank's GPU (default: LOCAL_RANK); runner as in explore."""
    import os

    import torch.distributed as dist

    base = base or FlockerConfig()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    if device is None:
        device = int(os.environ.get("LOCAL_RANK", "0"))
    rep_conf = max(int(rep_conf), 1)
    names, conf_values, conf_list = _configurations(inputs, outputs, mode, base)
    mine = list(range(rank, len(conf_list), world))
    rows = _rows(mine, list(range(len(mine))), rep_conf, names, conf_values, conf_list, outputs,
                 nstep, base, device, runner)
    root = dist.get_global_rank(group, 0) if group is not None else 0
    parts = [None] * world if rank == 0 else None
    dist.gather_object(rows, parts, dst=root, group=group)
    if rank != 0:
        return []
    return [r for part in parts for r in part]


def _debug(v) -> str:
    """Rust's {:?} of the value: floats keep a fractional part ("1.0")."""
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        s = np.format_float_positional(np.float64(v), unique=True, trim="-")
        return s if ("." in s or "inf" in s or "nan" in s) else s + ".0"
    return repr(v)


def _display(v) -> str:
    """Rust's to_string() of an f32 (shortest repr, no forced fraction)."""
    return np.format_float_positional(np.float32(v), unique=True, trim="-")


def write_csv(name: str, rows: Sequence[dict]) -> str:
    """lib.rs:1781-1792: "<name>.csv", one header row (the dataframe's field
    names), then one row per run.  Returns the path."""
    path = f"{name}.csv"
    with open(path, "w", newline="") as fh:
        w = csv.writer(fh)
        if rows:
            keys = list(rows[0])
            w.writerow(keys)
            for r in rows:
                w.writerow([str(r[k]) if k in ("Simulation", "Run")
                            else _display(r[k]) if k in ("Run Duration", "Step per sec")
                            else _debug(r[k]) for k in keys])
    return path


def _run_batch(replicas: List[Replica], nstep: int, device: int) -> np.ndarray:
    """Run every replica nstep steps as one device batch (CUDA graphs of
    100 steps) and return their heading moments, one row per replica: the
    one device call of each search iteration, generation or evaluation."""
    b = Batch(replicas, device=device)
    try:
        b.step(0, nstep, 1, 100)
        return b.moments()
    finally:
        b.close()


def _run_batch_timed(replicas: List[Replica], nstep: int, device: int) -> Tuple[np.ndarray, float]:
    """_run_batch, also returning the wall seconds of the steps alone (the
    batch is synchronised on both sides of them)."""
    b = Batch(replicas, device=device)
    try:
        b.synchronize()
        t0 = time.perf_counter()
        b.step(0, nstep, 1, 100)
        b.synchronize()
        secs = time.perf_counter() - t0
        return b.moments(), secs
    finally:
        b.close()


def _observables(m: np.ndarray) -> dict:
    return {name: fn(m) for name, fn in OUTPUTS.items()}


def random_search(init: FlockerConfig, n_iter: int, target: float,
                  cost_function: Callable[[dict], float],
                  gen_sample: Callable[[FlockerConfig, np.random.Generator], FlockerConfig],
                  batch_size: int, step: int, reps: int, seed: int = 0,
                  device: int = 0) -> Tuple[FlockerConfig, float, List[float]]:
    """random_search! (src/explore/random_search.rs:1-80) on the device.

    Each iteration draws batch_size samples from the best configuration so
    far (gen_sample(best, rng)), runs every sample reps times for step steps
    (all batch_size * reps runs as one device batch), averages
    cost_function over a sample's runs (it receives the run's observables,
    the OUTPUTS of explore), and keeps the lowest; the search stops once the
    best cost is <= target.  Returns (best configuration, its cost, the best
    cost after every iteration).  Run k of the whole search starts from
    Philox(init.init_seed + k), so a search is reproducible."""
    rng = np.random.default_rng(seed)
    best, min_cost = init, float(np.finfo(np.float32).max)
    history: List[float] = []
    run = 0
    for _ in range(int(n_iter)):
        samples = [gen_sample(best, rng) for _ in range(int(batch_size))]
        reps_list = []
        for smp in samples:
            for _ in range(int(reps)):
                reps_list.append(_replica(smp, init.init_seed + run))
                run += 1
        mom = _run_batch(reps_list, int(step), device)
        costs = [float(np.mean([cost_function(_observables(mom[i * reps + r])) for r in range(reps)]))
                 for i in range(len(samples))]
        k = int(np.argmin(costs))
        if costs[k] < min_cost:
            best, min_cost = samples[k], costs[k]
        history.append(min_cost)
        if min_cost <= target:
            break
    return best, min_cost, history


def evolutionary_search(init_population: Callable[[], List],
                        make_config: Callable[[object, int], FlockerConfig],
                        fitness: Callable[[List[dict]], float],
                        selection: Callable[[List[Tuple[object, float]]], None],
                        mutation: Callable[[object], object],
                        crossover: Callable[[List], None],
                        cmp: Callable[[float, float], bool],
                        desired_fitness: float, generation_num: int, step: int, reps: int = 1,
                        init_seed: int = 0, device: int = 0) -> List[dict]:
    """explore_ga_parallel! (src/explore/genetic.rs:626-826) on the device.

    Every generation runs each individual reps times for step steps, all of
    them as one device batch; make_config(individual, r) builds run r of an
    individual (the reference's new_with_parameters).  fitness gets the runs'
    observables (the OUTPUTS of explore), cmp(a, b) says that fitness a is
    better than b.  The search stops after generation_num generations (0: no
    limit) or in the first generation where an individual reaches
    desired_fitness; otherwise selection(pop_fitness) filters the
    (individual, fitness) list in place, crossover(population) edits the
    survivors in place and mutation(individual) returns each new individual.
    Returns one row per evaluated individual: generation, index, fitness,
    individual and its last run's observables ("state"), as BufferGA."""
    population = list(init_population())
    rows: List[dict] = []
    generation, run = 0, 0
    while population:
        if generation_num != 0 and generation == generation_num:
            break
        generation += 1
        reps_list = []
        for ind in population:
            for r in range(int(reps)):
                reps_list.append(_replica(make_config(ind, r), init_seed + run))
                run += 1
        mom = _run_batch(reps_list, int(step), device)
        pop_fitness = []
        reached = False
        for i, ind in enumerate(population):
            obs = [_observables(mom[i * reps + r]) for r in range(int(reps))]
            fit = float(fitness(obs))
            rows.append({"generation": generation, "index": i, "fitness": fit, "individual": ind,
                         "state": repr(obs[-1])})
            pop_fitness.append((ind, fit))
            if cmp(fit, desired_fitness):
                reached = True
        if reached:
            break
        selection(pop_fitness)
        if len(pop_fitness) < 1:
            break
        population = [ind for ind, _ in pop_fitness]
        crossover(population)
        population = [mutation(ind) for ind in population]
    return rows


# ------------------------------------------------------------ bayesian_search!
class GaussianProcess:
    """Gaussian-process regression, the surrogate of bayesian_search!
    (src/explore/bayesian.rs:135, 214, through the friedrich crate, which is
    not part of the reference tree).  Restated from the standard equations:
    a constant prior mean (the mean of the outputs), a Gaussian kernel
    k(a, b) = s^2 exp(-|a - b|^2 / (2 l^2)) with s^2 the variance of the
    outputs and l the median distance between the inputs, and a small noise
    term on the diagonal.  The kernel is refitted when samples are added."""

    def __init__(self, x, y, noise: float = 1e-6):
        self.noise = float(noise)
        self.x = np.asarray(x, np.float64).reshape(len(y), -1)
        self.y = np.asarray(y, np.float64).reshape(-1)
        self._fit()

    def _fit(self) -> None:
        x, y = self.x, self.y
        self.mean = float(y.mean())
        self.s2 = float(y.var()) if y.var() > 0 else 1.0
        d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
        off = d[np.triu_indices(len(x), 1)]
        self.l = float(np.median(off)) if off.size and np.median(off) > 0 else 1.0
        k = self._k(x, x) + self.noise * self.s2 * np.eye(len(x))
        self.chol = np.linalg.cholesky(k)
        self.alpha = np.linalg.solve(self.chol.T, np.linalg.solve(self.chol, y - self.mean))

    def _k(self, a, b):
        d2 = ((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)
        return self.s2 * np.exp(-d2 / (2.0 * self.l * self.l))

    def add_samples(self, x, y) -> None:
        """GaussianProcess::add_samples (bayesian.rs:159)."""
        self.x = np.vstack([self.x, np.asarray(x, np.float64).reshape(len(y), -1)])
        self.y = np.concatenate([self.y, np.asarray(y, np.float64).reshape(-1)])
        self._fit()

    def predict(self, x):
        """Posterior mean at one point (a 1-d array) or at every row of x."""
        q = np.asarray(x, np.float64)
        one = q.ndim == 1
        q = q.reshape(-1, self.x.shape[1])
        m = self.mean + self._k(q, self.x) @ self.alpha
        return float(m[0]) if one else m

    def predict_variance(self, x):
        """Posterior variance at one point or at every row of x."""
        q = np.asarray(x, np.float64)
        one = q.ndim == 1
        q = q.reshape(-1, self.x.shape[1])
        v = np.linalg.solve(self.chol, self._k(self.x, q))
        var = np.maximum(self.s2 - (v * v).sum(0), 0.0)
        return float(var[0]) if one else var


def generate_samples(batch_size: int, scale: float, num_of_params: int,
                     rng: Optional[np.random.Generator] = None) -> np.ndarray:
    """bayesian.rs:246-258: batch_size points, each coordinate uniform in
    [-scale, scale] (a seeded generator instead of the reference's rand::rng)."""
    rng = rng if rng is not None else np.random.default_rng()
    return rng.uniform(-1.0, 1.0, (int(batch_size), int(num_of_params))) * float(scale)


def expected_improvement(x_init, x, gp: GaussianProcess):
    """bayesian.rs:296-329: (mu - best) Phi(z) + sigma phi(z), z = (mu - best) /
    sigma, best the largest posterior mean over the evaluated points; 0 where
    sigma is 0.  x may be one point or a matrix of points (one result each)."""
    import math
    q = np.asarray(x, np.float64)
    one = q.ndim == 1
    q = q.reshape(-1, gp.x.shape[1])
    mu = np.atleast_1d(gp.predict(q))
    sigma = np.sqrt(np.atleast_1d(gp.predict_variance(q)))
    best = float(np.max(np.atleast_1d(gp.predict(np.asarray(x_init, np.float64)))))
    ei = np.zeros(len(q))
    ok = sigma > 0
    z = (mu[ok] - best) / sigma[ok]
    cdf = 0.5 * (1.0 + np.vectorize(math.erf)(z / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)
    ei[ok] = (mu[ok] - best) * cdf + sigma[ok] * pdf
    return float(ei[0]) if one else ei


def acquisition_function(x_init, x_samples, gp: GaussianProcess) -> np.ndarray:
    """bayesian.rs:268-289: the sample with the highest expected improvement
    (the first one among equals)."""
    xs = np.asarray(x_samples, np.float64)
    return xs[int(np.argmax(expected_improvement(x_init, xs, gp)))].copy()


def bayesian_search(init_parameters: Callable[[], Sequence[Sequence[float]]],
                    objective_function: Callable[[np.ndarray], float], gen_params,
                    n_iter: int, batch_size: Optional[int] = None,
                    scale: Optional[float] = None, seed: int = 0,
                    log: Optional[Callable[[str], None]] = None) -> Tuple[np.ndarray, float]:
    """bayesian_search! (src/explore/bayesian.rs:104-244): maximise
    objective_function.  The first pattern passes gen_params, a function of
    the evaluated points returning candidate points; the second passes the
    number of parameters and then batch_size and scale, and the candidates
    are generate_samples(batch_size, scale, num_of_params).  Every iteration
    evaluates the candidate with the highest expected improvement and adds
    it to the Gaussian process.  Returns (best point, best value).  With
    flock_objective the evaluations are flock runs on the device."""
    rng = np.random.default_rng(seed)
    x_init = [np.asarray(x, np.float64) for x in init_parameters()]
    y_init = [float(objective_function(x)) for x in x_init]
    k = int(np.argmax(y_init))
    x_max, y_max = x_init[k].copy(), y_init[k]
    gp = GaussianProcess(np.vstack(x_init), y_init)
    for i in range(int(n_iter)):
        if callable(gen_params):
            samples = np.asarray(gen_params(x_init), np.float64)
        else:
            samples = generate_samples(batch_size, scale, int(gen_params), rng)
        x_next = acquisition_function(np.vstack(x_init), samples, gp)
        y_next = float(objective_function(x_next))
        if log is not None:
            log(f"iteration {i}: point {x_next.tolist()}, f(x) = {y_next}, "
                f"predicted {gp.predict(x_next)}")
        gp.add_samples(x_next[None, :], [y_next])
        x_init.append(x_next)
        if y_next > y_max:
            x_max, y_max = x_next.copy(), y_next
    return x_max, y_max


def flock_objective(base: FlockerConfig, names: Sequence[str],
                    value_of: Callable[[List[dict]], float], step: int, reps: int = 1,
                    init_seed: int = 0, device: int = 0) -> Callable[[np.ndarray], float]:
    """An objective for bayesian_search whose evaluation is a flock run on
    the device: point x sets the configuration fields names[i] = x[i]; the
    point's reps runs go as one batch for step steps, and value_of receives
    their observables (the OUTPUTS of explore).  Run k of the whole search
    starts from Philox(init_seed + k)."""
    counter = [0]

    def f(x) -> float:
        cfg = base
        for nm, v in zip(names, np.asarray(x, np.float64).tolist()):
            cfg = _apply(cfg, nm, float(v))
        reps_list = []
        for _ in range(int(reps)):
            reps_list.append(_replica(cfg, init_seed + counter[0]))
            counter[0] += 1
        mom = _run_batch(reps_list, int(step), device)
        return float(value_of([_observables(mom[r]) for r in range(int(reps))]))

    return f


# ------------------------------------------------------------ sweep inputs
def gen_param(kind, minimum, maximum, n: int = 1,
              rng: Optional[np.random.Generator] = None) -> list:
    """gen_param! (src/lib.rs:1823-1852): n values uniform over [min, max) of
    type kind (int or float), for parameter sweeps.  As the macro does, a
    reversed range is swapped and an empty one widened by 1; n = 0 gives no
    value (the macro takes its argument n, not the adjusted count).  A seeded
    generator stands in for rand::rng()."""
    rng = rng if rng is not None else np.random.default_rng()
    lo, hi = kind(minimum), kind(maximum)
    if lo > hi:
        lo, hi = hi, lo
    elif lo == hi:
        hi = hi + kind(1)
    if kind is int:
        return [int(v) for v in rng.integers(lo, hi, int(n))]
    return [kind(v) for v in rng.uniform(lo, hi, int(n))]


def load_csv(path: str, *fields: Tuple[str, type]) -> tuple:
    """load_csv! (src/lib.rs:1854-1890): the columns of a CSV file with a
    header row, one list per (name, type) field taken by position, each value
    parsed as its type."""
    cols = [[] for _ in fields]
    with open(path, newline="") as fh:
        rows = csv.reader(fh)
        next(rows, None)  # the header (csv::Reader reads one by default)
        for rec in rows:
            for i, (_, kind) in enumerate(fields):
                cols[i].append(kind(rec[i]))
    return tuple(cols)
