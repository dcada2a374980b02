"""Generates the committed 1,000-boid fixtures from the oracle.

The flock: 1,000 boids on a 200x200 torus, discretization 10/1.5 (f32), radius 10,
all weights 1.0, jump 0.7, uniform positions and unit headings from
Philox(seed 42), jitter from Philox(seed 42).  Checkpoints of the whole read
buffer (stored order) after 1, 10 and 200 steps, for the relaxed query
(the reference Flockers query path) and the exact query (the in-tree Bird).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import krabmaga_gb300 as kg  # noqa: E402  (host-only generator, no GPU needed)
import oracle  # noqa: E402

SIDE = 200.0
D = float(np.float32(10.0) / np.float32(1.5))
SEED = 42
CHECKPOINTS = [1, 10, 200]


def make(kind: int, name: str) -> None:
    ids0, xy0, dxy0 = kg.gen_uniform(1000, SIDE, SIDE, SEED, 1.0)
    f = oracle.OracleField(SIDE, SIDE, D, True)
    f.set_many(ids0, xy0, dxy0)
    f.lazy_update()
    p = oracle.params(seed=SEED, query_mode=kind)
    out = {"ids0": ids0, "xy0": xy0, "dxy0": dxy0, "seed": np.int64(SEED),
           "checkpoints": np.array(CHECKPOINTS), "kind": np.int64(kind)}
    # neighbour lists of every boid at step 0 (reference visiting order)
    ids, st, _ = f.iter(1)
    counts, lists = f.neighbor_lists(kind, 10.0, st[:, :2])
    out["nb_counts0"], out["nb_ids0"] = counts, lists
    done = 0
    for c in CHECKPOINTS:
        f.flock_run(p, done, c - done)
        done = c
        ids, st, _ = f.iter(1)
        out[f"ids_{c}"], out[f"st_{c}"] = ids, st
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    make(0, "flock1k_relax_strict.npz")
    make(1, "flock1k_exact_strict.npz")
