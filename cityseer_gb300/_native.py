"""ctypes binding of libcsgpu.so, the C-ABI declared in include/cityseer_gb300.h.

The library is built in-tree by ``cityseer_gb300.build``.  There is no CPU fallback: if the
library is missing or a CUDA call fails, the calling API raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

MAX_K = 16
MAX_DEGREE = 32

CS_OK = 0
CS_ERR_ARG = 1
CS_ERR_CAPACITY = 2
CS_ERR_CUDA = 3
CS_ERR_TIMEOUT = 4
CS_ERR_INTERNAL = 5
CS_BATCH_ASYNC = 1

_ptr = C.c_void_p


class PrimalGraph(C.Structure):
    _fields_ = [
        ("n_bound", C.c_int32),
        ("n_edges", C.c_int32),
        ("max_out_degree", C.c_int32),
        ("in_ptr", _ptr),
        ("in_nb", _ptr),
        ("in_w", _ptr),
        ("in_seglen", _ptr),
        ("in_segimp", _ptr),
        ("out_ptr", _ptr),
        ("out_to", _ptr),
        ("out_w", _ptr),
        ("out_cnt", _ptr),
        ("out_seglen", _ptr),
        ("node_w", _ptr),
    ]


class DualGraph(C.Structure):
    _fields_ = [
        ("n_bound", C.c_int32),
        ("n_edges", C.c_int32),
        ("max_out_degree", C.c_int32),
        ("ptr", _ptr),
        ("to", _ptr),
        ("w", _ptr),
        ("ang", _ptr),
        ("len", _ptr),
        ("exit_slot", _ptr),
        ("entry_slot", _ptr),
        ("rptr", _ptr),
        ("rfrom", _ptr),
        ("rid", _ptr),
        ("fwd_pack", _ptr),
        ("rev_pack", _ptr),
    ]


class DataMapArrays(C.Structure):
    """cs_data_map: a data layer's node assignments as device arrays."""

    _fields_ = [
        ("n_entries", C.c_int32), ("n_assign", C.c_int32), ("n_groups", C.c_int32),
        ("node_ptr", _ptr), ("assign_entry", _ptr), ("assign_dist", _ptr), ("assign_node", _ptr),
        ("assign_rank", _ptr), ("entry_group", _ptr), ("entry_class", _ptr), ("group_ptr", _ptr),
        ("group_assign", _ptr),
    ]


class Query(C.Structure):
    _fields_ = [
        ("k", C.c_int32),
        ("distances", C.c_uint32 * MAX_K),
        ("betas", C.c_float * MAX_K),
        ("seconds", C.c_uint32 * MAX_K),
        ("speed_m_s", C.c_float),
        ("tolerance", C.c_float),
        ("angular_scaling_unit", C.c_float),
        ("farness_scaling_offset", C.c_float),
        ("compute_closeness", C.c_int32),
        ("compute_betweenness", C.c_int32),
        ("track_reach", C.c_int32),
        ("n_sources", C.c_int64),
        ("sources", _ptr),
        ("src_wt", _ptr),
        ("eligible", _ptr),
    ]


class Plan(C.Structure):
    _fields_ = [
        ("n_slots", C.c_int32),
        ("cap", C.c_int32),
        ("threads_per_block", C.c_int32),
        ("blocks", C.c_int32),
        ("delta_seconds", C.c_float),
        ("lanes", C.c_int32),
        ("variant", C.c_int32),
        ("max_degree", C.c_int32),
        ("n_bound", C.c_int32),
        ("cta_blocks", C.c_int32),
        ("workspace_bytes", C.c_size_t),
    ]


class BatchJob(C.Structure):
    _fields_ = [
        ("g", PrimalGraph),
        ("mode", C.c_int32),
        ("k", C.c_int32),
        ("distances", C.c_uint32 * MAX_K),
        ("betas", C.c_float * MAX_K),
        ("seconds", C.c_uint32 * MAX_K),
        ("speed_m_s", C.c_float),
        ("tolerance", C.c_float),
        ("delta_seconds", C.c_float),
        ("compute_closeness", C.c_int32),
        ("compute_betweenness", C.c_int32),
        ("n_sources", C.c_int32),
        ("sources", _ptr),
        ("src_wt", _ptr),
        ("eligible", _ptr),
        ("out", _ptr),
        ("bucket", _ptr),
        ("out2", _ptr),
        ("item_begin", C.c_int64),
    ]


class DualBatchJob(C.Structure):
    _fields_ = [
        ("g", DualGraph),
        ("k", C.c_int32),
        ("seconds", C.c_uint32 * MAX_K),
        ("tolerance", C.c_float),
        ("angular_scaling_unit", C.c_float),
        ("farness_scaling_offset", C.c_float),
        ("compute_closeness", C.c_int32),
        ("compute_betweenness", C.c_int32),
        ("n_sources", C.c_int32),
        ("sources", _ptr),
        ("src_wt", _ptr),
        ("eligible", _ptr),
        ("out", _ptr),
        ("bucket", _ptr),
        ("item_begin", C.c_int64),
    ]


class Outputs(C.Structure):
    _fields_ = [("out", _ptr), ("reach", _ptr)]


# every symbol declared in include/cityseer_gb300.h, with its ctypes signature
SIGNATURES = {
    "cs_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "cs_pair_distances_betas_time": (
        C.c_int32,
        [C.c_float, C.c_int32, C.c_int32, _ptr, _ptr, _ptr, C.c_float, _ptr, _ptr, _ptr],
    ),
    "cs_edge_travel_seconds": (
        C.c_int32,
        [C.c_int64, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr, C.c_float, C.c_int32, _ptr],
    ),
    "cs_plan_primal": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.POINTER(Plan)],
    ),
    "cs_plan_dual": (
        C.c_int32,
        [C.POINTER(DualGraph), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.POINTER(Plan)],
    ),
    "cs_workspace_init": (C.c_int32, [C.POINTER(Plan), C.c_int32, _ptr, C.c_size_t, _ptr]),
    "cs_dual_workspace_init": (C.c_int32, [C.POINTER(Plan), C.c_int32, _ptr, C.c_size_t, _ptr]),
    "cs_centrality_shortest": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.POINTER(Query), C.POINTER(Plan), _ptr, C.c_size_t, Outputs, _ptr],
    ),
    "cs_centrality_simplest": (
        C.c_int32,
        [C.POINTER(DualGraph), C.POINTER(Query), C.POINTER(Plan), _ptr, C.c_size_t, Outputs, _ptr],
    ),
    "cs_betweenness_od_shortest": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.POINTER(Query), _ptr, _ptr, _ptr, C.POINTER(Plan), _ptr, C.c_size_t, Outputs,
         _ptr],
    ),
    "cs_segment_centrality": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.POINTER(Query), C.POINTER(Plan), _ptr, C.c_size_t, Outputs, _ptr],
    ),
    "cs_accessibility": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.POINTER(DataMapArrays), C.POINTER(Query), _ptr, C.c_int32, C.POINTER(Plan), _ptr,
         C.c_size_t, _ptr, _ptr, _ptr, _ptr],
    ),
    "cs_tree_shortest": (
        C.c_int32,
        [
            C.POINTER(PrimalGraph), C.c_int32, _ptr, C.c_uint32, C.c_float, C.POINTER(Plan), _ptr, C.c_size_t,
            C.c_int32, _ptr, _ptr, _ptr, _ptr, _ptr,
        ],
    ),
    "cs_tree_simplest": (
        C.c_int32,
        [
            C.POINTER(DualGraph), C.c_int32, _ptr, C.c_uint32, C.c_float, C.POINTER(Plan), _ptr, C.c_size_t,
            C.c_int32, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr,
        ],
    ),
    "cs_plan_dual_tree": (C.c_int32, [C.POINTER(DualGraph), C.c_int32, C.c_int32, C.c_int64, C.POINTER(Plan)]),
    "cs_dual_tree_workspace_init": (C.c_int32, [C.POINTER(Plan), _ptr, C.c_size_t, _ptr]),
    "cs_last_counters": (C.c_int32, [C.POINTER(C.c_int64)] * 4),
    "cs_batch_prepare": (C.c_int32, [C.POINTER(BatchJob), C.c_int32, C.POINTER(C.c_int64)]),
    "cs_batch_plan": (C.c_int32, [C.POINTER(BatchJob), C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.POINTER(Plan)]),
    "cs_batch_run": (
        C.c_int32,
        [C.POINTER(BatchJob), _ptr, C.c_int32, C.POINTER(Plan), _ptr, C.c_size_t, C.c_int32, _ptr],
    ),
    "cs_batch_status": (C.c_int32, [_ptr, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _ptr]),
    "cs_batch_failed": (C.c_int32, [_ptr, C.POINTER(Plan), C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int64),
                                    _ptr]),
    "cs_abi_sizes": (C.c_int32, [_ptr, C.c_int32]),
    "cs_last_retries": (C.c_int32, [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cs_dual_batch_prepare": (C.c_int32, [C.POINTER(DualBatchJob), C.c_int32, C.POINTER(C.c_int64)]),
    "cs_dual_batch_plan": (C.c_int32, [C.POINTER(DualBatchJob), C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                       C.POINTER(Plan)]),
    "cs_dual_batch_run": (C.c_int32, [C.POINTER(DualBatchJob), _ptr, C.c_int32, C.POINTER(Plan), _ptr, C.c_size_t,
                                      C.c_int32, _ptr]),
    "cs_dual_batch_failed": (C.c_int32, [_ptr, C.POINTER(Plan), C.POINTER(C.c_int32), C.c_int32,
                                         C.POINTER(C.c_int64), _ptr]),
    "cs_source_weights": (C.c_int32, [_ptr, C.c_int64, _ptr, C.c_int32, _ptr, _ptr, _ptr]),
    "cs_device_sm_count": (C.c_int32, []),
    "cs_last_phase_cycles": (C.c_int32, [_ptr, C.c_int32]),
    "cs_dual_pack": (C.c_int32, [C.POINTER(DualGraph), _ptr, _ptr, _ptr]),
    "cs_centrality_shortest_noalloc": (
        C.c_int32,
        [C.POINTER(PrimalGraph), C.POINTER(Query), Outputs, _ptr],
    ),
    "cs_debug_seed_exp": (C.c_int32, [_ptr, _ptr, _ptr, _ptr, C.c_int64, _ptr]),
    "cs_workspace_progress": (C.c_int32, [_ptr, C.POINTER(C.c_int64)]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero cs_status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[cs_status {code}] {msg}")
        self.code = code
        self.msg = msg


def lib_path() -> Path:
    return _build.LIB_PATH


def load(auto_build: bool = True) -> C.CDLL:
    """Loads (building first if needed) libcsgpu.so and declares every exported signature."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if auto_build:
            _build.build()
        if not path.exists():
            raise RuntimeError(f"libcsgpu.so not found at {path}; run cityseer_gb300.build.build()")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        sizes = (C.c_int32 * 7)()
        lib.cs_abi_sizes(sizes, 7)
        want = [C.sizeof(t) for t in (PrimalGraph, DualGraph, Query, Plan, Outputs, BatchJob, DualBatchJob)]
        if list(sizes) != want:
            raise RuntimeError(f"libcsgpu.so struct layouts {list(sizes)} differ from the binding's {want}")
        _lib = lib
        return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(4096)
    lib.cs_last_error(buf, 4096)
    return buf.value.decode("utf-8", "replace")


def check(code: int, what: str = "") -> None:
    if code != CS_OK:
        msg = last_error()
        if code == CS_ERR_ARG:
            raise ValueError(msg)
        raise NativeError(code, f"{what}: {msg}" if what else msg)
