"""ctypes binding of libkrabgpu.so (the C ABI declared in include/krabgpu.h).

The shared library is built in place by ``__graft_entry__.build()`` (or
``make -C krabmaga_gb300``).  There is no fallback: if the library is missing
or cannot load, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkrabgpu.so")

KB_OK = 0
KB_ERR_ARG = 1
KB_ERR_OOM = 2
KB_ERR_CUDA = 3
KB_ERR_TIMEOUT = 4
KB_ERR_DEVICE_FLAG = 5
KB_ERR_STATE = 6
KB_ERR_RANGE = 7
KB_ERR_NO_DEVICE = 8
KB_ERR_BUSY = 9

KB_FLAG_KEY_RANGE = 0x1
KB_FLAG_REBIN_MISS = 0x2
KB_FLAG_SPIN_TIMEOUT = 0x4
KB_FLAG_NONFINITE = 0x8

KB_QUERY_RELAX = 0
KB_QUERY_EXACT = 1
KB_ARITH_STRICT = 0
KB_ARITH_FAST = 1
KB_NOALLOC_MAX_QUERIES = 65536
KB_CELL_WRAP_CLAMP = 0
KB_CELL_WRAP_TORUS = 1
KB_DENSE_AUTO = 0
KB_DENSE_OFF = 1
KB_DENSE_ON = 2
KB_PATH_SEPARATE = 0
KB_PATH_FUSED = 1
KB_PATH_TILED = 2
KB_PATH_SMALL = 3
KB_PATH_DENSE = 4
KB_WITHHOLD_NONE = 0
KB_WITHHOLD_SCAN_PUBLISH = 1
KB_WITHHOLD_GRID_ARRIVAL = 2

STATUS_NAMES = {
    0: "KB_OK", 1: "KB_ERR_ARG", 2: "KB_ERR_OOM", 3: "KB_ERR_CUDA", 4: "KB_ERR_TIMEOUT",
    5: "KB_ERR_DEVICE_FLAG", 6: "KB_ERR_STATE", 7: "KB_ERR_RANGE", 8: "KB_ERR_NO_DEVICE",
    9: "KB_ERR_BUSY",
}


class KbError(RuntimeError):
    """A libkrabgpu call returned a non-zero kb_status."""

    def __init__(self, status: int, func: str, msg: str):
        self.status = status
        super().__init__(f"{func}: {STATUS_NAMES.get(status, status)}: {msg}")


class FieldDesc(C.Structure):
    _fields_ = [
        ("width", C.c_float),
        ("height", C.c_float),
        ("discretization", C.c_float),
        ("toroidal", C.c_int32),
        ("device", C.c_int32),
        ("capacity_hint", C.c_uint32),
        ("cell_wrap", C.c_int32),
    ]


class FlockParamsC(C.Structure):
    _fields_ = [
        ("cohesion", C.c_float),
        ("avoidance", C.c_float),
        ("consistency", C.c_float),
        ("randomness", C.c_float),
        ("momentum", C.c_float),
        ("jump", C.c_float),
        ("neighbor_radius", C.c_float),
        ("query_mode", C.c_int32),
        ("arith", C.c_int32),
        ("_pad", C.c_uint32),
        ("seed", C.c_uint64),
    ]


class ReplicaDesc(C.Structure):
    _fields_ = [
        ("width", C.c_float),
        ("height", C.c_float),
        ("discretization", C.c_float),
        ("toroidal", C.c_int32),
        ("nboids", C.c_uint32),
        ("cell_wrap", C.c_int32),
        ("params", FlockParamsC),
    ]


class ServerDesc(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("max_slots", C.c_uint32),
        ("hbm_budget_bytes", C.c_uint64),
        ("quantum_steps", C.c_uint32),
        ("max_request_boids", C.c_uint32),
        ("max_request_cells", C.c_uint32),
        ("query_mode", C.c_int32),
        ("arith", C.c_int32),
        ("_pad", C.c_uint32),
    ]


class RequestC(C.Structure):
    _fields_ = [
        ("nboids", C.c_uint32),
        ("side", C.c_float),
        ("discretization", C.c_float),
        ("steps", C.c_uint32),
        ("params", FlockParamsC),
        ("init_seed", C.c_uint64),
        ("heading_scale", C.c_float),
        ("_pad", C.c_uint32),
    ]


class ServerReport(C.Structure):
    _fields_ = [
        ("completed", C.c_uint64), ("failed", C.c_uint64), ("queued", C.c_uint64),
        ("running", C.c_uint64), ("p50_s", C.c_double), ("p99_s", C.c_double),
        ("max_s", C.c_double), ("boid_updates", C.c_double), ("wall_s", C.c_double),
        ("busy_s", C.c_double), ("launches", C.c_uint64), ("repacks", C.c_uint64),
        ("max_active", C.c_uint64),
    ]


if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
    )
lib = C.CDLL(LIB_PATH)

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U32 = C.POINTER(C.c_uint32)
_SZ = C.POINTER(C.c_size_t)

_SIGS = {
    "kb_last_error": (C.c_char_p, []),
    "kb_version": (C.c_char_p, []),
    "kb_device_count": (C.c_int32, []),
    "kb_field_create": (C.c_int32, [C.POINTER(FieldDesc), C.POINTER(_P)]),
    "kb_field_destroy": (C.c_int32, [_P]),
    "kb_field_dims": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "kb_field_cuda_stream": (C.c_int32, [_P, C.POINTER(_P)]),
    "kb_field_set_object_location": (C.c_int32, [_P, C.c_uint32, _F, _F, _F]),
    "kb_field_set_locations": (C.c_int32, [_P, C.c_size_t, _U32, _F, _F]),
    "kb_field_remove_object_location": (C.c_int32, [_P, C.c_uint32, _F]),
    "kb_field_remove_ids": (C.c_int32, [_P, C.c_size_t, _U32, _SZ]),
    "kb_field_get_locations": (C.c_int32, [_P, C.c_int32, C.c_size_t, _U32, _F,
                                           C.POINTER(C.c_int32)]),
    "kb_field_lazy_update": (C.c_int32, [_P]),
    "kb_field_num_agents": (C.c_int32, [_P, _SZ]),
    "kb_field_num_objects": (C.c_int32, [_P, _SZ]),
    "kb_field_get_neighbors_within_relax_distance": (
        C.c_int32, [_P, _F, C.c_float, _U32, _F, C.c_size_t, _SZ]),
    "kb_field_get_neighbors_within_distance": (
        C.c_int32, [_P, _F, C.c_float, _U32, _F, C.c_size_t, _SZ]),
    "kb_field_get_objects": (C.c_int32, [_P, _F, _U32, _F, C.c_size_t, _SZ]),
    "kb_field_get_objects_unbuffered": (C.c_int32, [_P, _F, _U32, _F, C.c_size_t, _SZ]),
    "kb_field_num_objects_at_location": (C.c_int32, [_P, _F, _SZ]),
    "kb_field_get_empty_bags": (C.c_int32, [_P, _F, C.c_size_t, _SZ]),
    "kb_field_get_random_empty_bag": (C.c_int32, [_P, C.c_uint64, _F, C.POINTER(C.c_int32)]),
    "kb_field_iter_objects": (C.c_int32, [_P, C.c_int32, _F, _U32, _F, C.c_size_t, _SZ]),
    "kb_flock_compute": (C.c_int32, [_P, C.POINTER(FlockParamsC), C.c_uint64]),
    "kb_flock_compute_agents": (C.c_int32, [_P, C.POINTER(FlockParamsC), C.c_uint64, C.c_size_t,
                                            _U32, _F]),
    # device-resident record exchange: device pointers as void*
    "kb_field_copy_read_buffer": (C.c_int32, [_P, _P, _P, C.c_size_t, _SZ]),
    "kb_field_set_states_device": (C.c_int32, [_P, C.c_size_t, _P, _P]),
    "kb_flock_next_states_device": (C.c_int32, [_P, C.POINTER(FlockParamsC), C.c_uint64,
                                                C.c_size_t, _P, _P, _P]),
    "kb_field_set_step_options": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "kb_field_set_dense_mode": (C.c_int32, [_P, C.c_int32]),
    "kb_field_dense_active": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "kb_field_step_path": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "kb_field_step_stats": (C.c_int32, [_P, _U32]),
    "kb_field_set_kernel_timing": (C.c_int32, [_P, C.c_int32]),
    "kb_field_kernel_times": (C.c_int32, [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "kb_field_phase_clocks": (C.c_int32, [_P, C.c_int32, C.POINTER(C.c_uint64)]),
    "kb_flock_step": (C.c_int32, [_P, C.POINTER(FlockParamsC), C.c_uint64, C.c_uint32]),
    "kb_field_get_state": (C.c_int32, [_P, _U32, _F, C.c_size_t, _SZ]),
    "kb_field_device_flags": (C.c_int32, [_P, _U32, C.c_int32]),
    "kb_field_set_wait_test": (C.c_int32, [_P, C.c_uint32, C.c_int32, C.c_uint32]),
    "kb_field_synchronize": (C.c_int32, [_P]),
    "kb_field_neighbor_lists": (
        C.c_int32, [_P, C.c_int32, C.c_float, C.c_size_t, _F, _U32, _U32, C.c_size_t, _SZ]),
    "kb_field_neighbor_digest": (
        C.c_int32, [_P, C.c_int32, C.c_float, C.c_size_t, _F, _U32, _U32]),
    "kb_field_neighbor_digest_noalloc": (
        C.c_int32, [_P, C.c_int32, C.c_float, C.c_size_t, _F, _U32, _U32]),
    "kb_debug_allocation_counts": (C.c_int32, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "kb_debug_fail_allocations": (C.c_int32, [C.c_uint32]),
    "kb_batch_create": (C.c_int32, [C.c_int32, C.c_uint32, C.POINTER(ReplicaDesc), C.POINTER(_P)]),
    "kb_batch_destroy": (C.c_int32, [_P]),
    "kb_batch_set_replica": (C.c_int32, [_P, C.c_uint32, C.c_size_t, _U32, _F, _F]),
    "kb_batch_commit": (C.c_int32, [_P]),
    "kb_batch_step": (C.c_int32, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]),
    "kb_batch_get_replica": (C.c_int32, [_P, C.c_uint32, _U32, _F, C.c_size_t, _SZ]),
    "kb_batch_synchronize": (C.c_int32, [_P]),
    "kb_batch_moments": (C.c_int32, [_P, C.POINTER(C.c_double)]),
    "kb_batch_add_replica": (C.c_int32, [_P, C.POINTER(ReplicaDesc), _U32, _F, _F, C.c_uint64,
                                         C.POINTER(C.c_uint32)]),
    "kb_batch_remove_replica": (C.c_int32, [_P, C.c_uint32]),
    "kb_field_moments": (C.c_int32, [_P, C.POINTER(C.c_double)]),
    "kb_batch_cuda_stream": (C.c_int32, [_P, C.POINTER(_P)]),
    "kb_batch_set_step_options": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "kb_batch_step_stats": (C.c_int32, [_P, _U32]),
    "kb_batch_device_flags": (C.c_int32, [_P, _U32, C.c_int32]),
    "kb_batch_autotune": (C.c_int32, [_P, C.c_uint64, C.c_uint32, C.POINTER(C.c_int32), C.c_int32,
                                      C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "kb_field_autotune": (C.c_int32, [_P, C.POINTER(FlockParamsC), C.c_uint64, C.c_uint32,
                                      C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_float)]),
    "kb_server_create": (C.c_int32, [C.POINTER(ServerDesc), C.POINTER(_P)]),
    "kb_server_destroy": (C.c_int32, [_P]),
    "kb_server_submit": (C.c_int32, [_P, C.POINTER(RequestC), C.POINTER(C.c_uint64)]),
    "kb_server_poll": (C.c_int32, [_P, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "kb_server_result": (C.c_int32, [_P, C.c_uint64, _U32, _F, C.c_size_t, _SZ]),
    "kb_server_release": (C.c_int32, [_P, C.c_uint64]),
    "kb_server_wait_idle": (C.c_int32, [_P, C.c_double]),
    "kb_server_stats": (C.c_int32, [_P, C.POINTER(ServerReport)]),
    "kb_gen_uniform": (C.c_int32, [C.c_size_t, C.c_float, C.c_float, C.c_uint64, C.c_float,
                                   _U32, _F, _F]),
    "kb_gen_clustered": (C.c_int32, [C.c_size_t, C.c_float, C.c_float, C.c_uint32, C.c_float,
                                     C.c_float, C.c_uint64, _U32, _F, _F]),
}

for _name, (_res, _args) in _SIGS.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def last_error() -> str:
    return (lib.kb_last_error() or b"").decode()


def check(status: int, func: str) -> None:
    if status != KB_OK:
        raise KbError(status, func, last_error())


def call(name: str, *args) -> None:
    check(getattr(lib, name)(*args), name)


def fptr(a):
    return a.ctypes.data_as(_F) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(_U32) if a is not None else None


def allocation_counts():
    """(device allocations, device frees) the library has made in this process."""
    a, f = C.c_uint64(), C.c_uint64()
    call("kb_debug_allocation_counts", C.byref(a), C.byref(f))
    return int(a.value), int(f.value)


def fail_allocations(count: int) -> None:
    """The next `count` device allocations of the library fail as if the device
    were out of memory (testing failure handling); 0 ends it."""
    call("kb_debug_fail_allocations", C.c_uint32(count))
