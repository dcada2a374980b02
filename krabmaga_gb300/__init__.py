"""krabmaga_gb300 -- GB300-native continuous-space agent step for krABMaga.

The compute runs in ``libkrabgpu.so`` (hand-written sm_103a kernels behind the
C ABI of include/krabgpu.h); this package is its Python host binding with the
reference's API names (Field2D, State, Schedule, simulate, Flocker).
"""
from . import _lib
from ._lib import KbError, lib, LIB_PATH, KB_QUERY_RELAX, KB_QUERY_EXACT, KB_ARITH_STRICT, KB_ARITH_FAST
from ._lib import (KB_CELL_WRAP_CLAMP, KB_CELL_WRAP_TORUS, KB_DENSE_AUTO, KB_DENSE_OFF, KB_DENSE_ON,
                   KB_PATH_DENSE, KB_PATH_FUSED, KB_PATH_SEPARATE, KB_PATH_SMALL, KB_PATH_TILED,
                   KB_FLAG_KEY_RANGE, KB_FLAG_REBIN_MISS, KB_FLAG_SPIN_TIMEOUT, KB_FLAG_NONFINITE)
from .field import Bird, Field2D, Real2D
from .batch import Batch, Replica, sweep_replicas
from .serve import Request, Server, request_stream
from .explore import (ExploreMode, FlockerConfig, bayesian_search, build_configurations,
                      evolutionary_search, explore, explore_distributed, flock_objective,
                      gen_param, load_csv, random_search, write_csv)
from .model import (Agent, AgentImpl, FlockParams, Flocker, Schedule, State, gen_clustered,
                    gen_uniform, simulate, simulate_old)

__all__ = [
    "Bird", "Field2D", "Real2D", "FlockParams", "Flocker", "Schedule", "State", "simulate",
    "Agent", "AgentImpl",
    "simulate_old", "gen_uniform", "gen_clustered", "KbError", "lib", "LIB_PATH",
    "KB_QUERY_RELAX", "KB_QUERY_EXACT", "KB_ARITH_STRICT", "KB_ARITH_FAST", "device_count",
    "KB_CELL_WRAP_CLAMP", "KB_CELL_WRAP_TORUS", "KB_DENSE_AUTO", "KB_DENSE_OFF", "KB_DENSE_ON",
    "KB_PATH_SEPARATE", "KB_PATH_FUSED", "KB_PATH_TILED", "KB_PATH_SMALL", "KB_PATH_DENSE",
    "KB_FLAG_KEY_RANGE", "KB_FLAG_REBIN_MISS", "KB_FLAG_SPIN_TIMEOUT", "KB_FLAG_NONFINITE",
    "Batch", "Replica", "sweep_replicas", "Request", "Server", "request_stream",
    "ExploreMode", "FlockerConfig", "build_configurations", "explore", "explore_distributed",
    "random_search",
    "evolutionary_search", "write_csv", "bayesian_search", "flock_objective", "gen_param",
    "load_csv",
]


def device_count() -> int:
    return int(lib.kb_device_count())
