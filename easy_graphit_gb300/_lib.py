"""ctypes binding of libgg.so (the C ABI declared in include/gg.h).

The library is loaded from this package directory; there is no fallback: if
libgg.so is missing the import of anything that needs it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libgg.so"

i32, i64, u32, f32 = C.c_int32, C.c_int64, C.c_uint32, C.c_float
P = C.c_void_p
Pi32 = C.POINTER(C.c_int32)

# gg_status values (gg.h)
GG_OK, GG_ERR_INVALID, GG_ERR_CUDA, GG_ERR_OOM, GG_ERR_TIMEOUT = 0, 1, 2, 3, 4
GG_ERR_OVERFLOW, GG_ERR_UNSUPPORTED, GG_ERR_IO, GG_ERR_STATE = 5, 6, 7, 8
STATUS_NAMES = {0: "GG_OK", 1: "GG_ERR_INVALID", 2: "GG_ERR_CUDA", 3: "GG_ERR_OOM",
                4: "GG_ERR_TIMEOUT", 5: "GG_ERR_OVERFLOW", 6: "GG_ERR_UNSUPPORTED",
                7: "GG_ERR_IO", 8: "GG_ERR_STATE"}


class GGError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class gg_schedule(C.Structure):
    _fields_ = [("direction", i32), ("pull_frontier_rep", i32), ("frontier_creation", i32),
                ("deduplication", i32), ("deduplication_strategy", i32), ("load_balancing", i32),
                ("edge_blocking", i32), ("block_size", i32), ("kernel_fusion", i32),
                ("max_cta", i32), ("cta_size", i32)]


class gg_app_schedule(C.Structure):
    _fields_ = [("kind", i32), ("fuse", i32), ("threshold", f32), ("s1", gg_schedule),
                ("s2", gg_schedule), ("selector", P)]


class gg_vertex_data(C.Structure):
    _fields_ = [("parent", P), ("depth", P), ("dist", P), ("ids", P), ("updates", P),
                ("old_rank", P), ("new_rank", P), ("contrib", P), ("num_paths", P),
                ("dependences", P), ("visited", P), ("level", i32), ("src", i32),
                ("damping", f32)]


class gg_batch_tuning(C.Structure):
    _fields_ = [("blocks_per_sm", i32), ("chunk", i32), ("edge_parallel_max", i32), ("bottom_up_div", i32),
                ("per_source_cta", i32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class gg_tune_row(C.Structure):
    _fields_ = [("tuning", gg_batch_tuning), ("ms", f32)]


class gg_stats(C.Structure):
    _fields_ = [("iterations", i32), ("push_iterations", i32), ("pull_iterations", i32),
                ("bucket_advances", i32), ("vertices_reached", i64), ("edges_traversed", i64),
                ("device_ms", f32), ("loop_ms", f32), ("fused", i32), ("launches", i32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes); every symbol include/gg.h declares.
SIGNATURES: dict[str, tuple] = {
    "gg_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "gg_version": (C.c_char_p, []),
    "gg_schedule_init": (None, [C.POINTER(gg_schedule)]),
    "gg_set_default_launch": (None, [i32, i32]),
    "gg_host_graph_rmat": (i32, [i32, i32, f32, f32, f32, i64, i32, i32, i32, C.POINTER(P)]),
    "gg_host_graph_grid": (i32, [i32, i32, i64, i32, i32, C.POINTER(P)]),
    "gg_host_graph_mix_spec": (i32, [i64, i32, P]),
    "gg_host_graph_from_edges": (i32, [i32, i64, P, P, P, i32, C.POINTER(P)]),
    "gg_host_graph_from_csr": (i32, [i32, i64, P, P, P, C.POINTER(P)]),
    "gg_host_graph_load": (i32, [C.c_char_p, i32, C.POINTER(P)]),
    "gg_host_graph_save_bin": (i32, [P, C.c_char_p]),
    "gg_host_graph_save_sg": (i32, [P, C.c_char_p, i32]),
    "gg_host_graph_info": (i32, [P, Pi32, C.POINTER(i64)]),
    "gg_host_graph_pick_sources": (i32, [P, i32, i64, P]),
    "gg_host_graph_offsets": (P, [P]),
    "gg_host_graph_dst": (P, [P]),
    "gg_host_graph_weights": (P, [P]),
    "gg_host_graph_destroy": (None, [P]),
    "gg_graph_create": (i32, [P, P, P, i32, i64, u32, C.POINTER(P)]),
    "gg_graph_destroy": (i32, [P]),
    "gg_graph_info": (i32, [P, Pi32, C.POINTER(i64)]),
    "gg_graph_set_stream": (i32, [P, P]),
    "gg_graph_sync": (i32, [P]),
    "gg_graph_transpose": (i32, [P]),
    "gg_graph_blocked": (i32, [P, i32]),
    "gg_graph_device_arrays": (i32, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "gg_frontier_create": (i32, [P, i32, C.POINTER(P)]),
    "gg_frontier_destroy": (i32, [P]),
    "gg_frontier_add": (i32, [P, i32]),
    "gg_frontier_size": (i32, [P, Pi32]),
    "gg_frontier_clear": (i32, [P]),
    "gg_frontier_format": (i32, [P, Pi32]),
    "gg_frontier_to_sparse": (i32, [P]),
    "gg_frontier_to_bitmap": (i32, [P]),
    "gg_frontier_to_boolmap": (i32, [P]),
    "gg_frontier_dedup": (i32, [P]),
    "gg_frontier_read": (i32, [P, P, i32, Pi32]),
    "gg_edgeset_apply": (i32, [P, C.POINTER(gg_schedule), i32, i32, P, P, i32,
                               C.POINTER(gg_vertex_data)]),
    "gg_vertexset_apply": (i32, [P, P, i32, C.POINTER(gg_vertex_data)]),
    "gg_pq_create": (i32, [P, P, i32, i32, i32, C.POINTER(P)]),
    "gg_pq_destroy": (i32, [P]),
    "gg_pq_finished": (i32, [P, Pi32]),
    "gg_pq_dequeue": (i32, [P, C.POINTER(P)]),
    "gg_edgeset_apply_priority": (i32, [P, C.POINTER(gg_schedule), P, C.POINTER(gg_vertex_data)]),
    "gg_frontier_list_create": (i32, [P, C.POINTER(P)]),
    "gg_frontier_list_destroy": (i32, [P]),
    "gg_frontier_list_insert": (i32, [P, P]),
    "gg_frontier_list_retrieve": (i32, [P, P]),
    "gg_bfs": (i32, [P, C.POINTER(gg_app_schedule), i32, P, P, C.POINTER(gg_stats)]),
    "gg_bfs_collect_directions": (i32, [P, i32, i32, P, P, C.POINTER(i32)]),
    "gg_sssp": (i32, [P, C.POINTER(gg_app_schedule), i32, i32, P, C.POINTER(gg_stats)]),
    "gg_pagerank": (i32, [P, C.POINTER(gg_app_schedule), i32, f32, P, C.POINTER(gg_stats)]),
    "gg_cc": (i32, [P, C.POINTER(gg_app_schedule), P, C.POINTER(gg_stats)]),
    "gg_bc": (i32, [P, C.POINTER(gg_app_schedule), i32, P, C.POINTER(gg_stats)]),
    "gg_debug_barrier_timeout": (i32, [i32]),
    "gg_kernel_launches": (C.c_uint64, []),
    "gg_memory_trim": (i32, [C.c_size_t]),
    "gg_bfs_noalloc": (i32, [P, P, i32, i32, i32, P, P]),
    "gg_bfs_batch": (i32, [P, P, i32, P, C.POINTER(gg_stats)]),
    "gg_bc_batch": (i32, [P, P, i32, P, C.POINTER(gg_stats)]),
    "gg_bfs_multi": (i32, [P, C.POINTER(gg_app_schedule), P, i32, P, P, C.POINTER(gg_stats)]),
    "gg_sssp_multi": (i32, [P, C.POINTER(gg_app_schedule), P, i32, i32, P, C.POINTER(gg_stats)]),
    "gg_host_graph_union": (i32, [P, i32, P, C.POINTER(P)]),
    "gg_batch_plan_create": (i32, [P, i32, P, i32, i32, P, C.POINTER(P)]),
    "gg_batch_plan_run": (i32, [P, C.POINTER(gg_stats)]),
    "gg_batch_plan_destroy": (i32, [P]),
    "gg_batch_set_tuning": (i32, [P, i32, C.POINTER(gg_batch_tuning)]),
    "gg_batch_get_tuning": (i32, [P, i32, C.POINTER(gg_batch_tuning)]),
    "gg_batch_autotune": (i32, [P, i32, P, i32, i32, C.POINTER(gg_batch_tuning), P, i32,
                                C.POINTER(i32)]),
    "gg_selector_create": (i32, [i64, C.POINTER(P)]),
    "gg_selector_destroy": (i32, [P]),
    "gg_selector_num_params": (i32, []),
    "gg_selector_get_params": (i32, [P, P, i32]),
    "gg_selector_set_params": (i32, [P, P, i32]),
    "gg_selector_forward": (i32, [P, P, i32, P]),
    "gg_selector_grad": (i32, [P, P, P, i32, P, P]),
    "gg_selector_train": (i32, [P, P, P, i32, i32, f32, P]),
    "gg_selector_save": (i32, [P, C.c_char_p]),
    "gg_selector_load": (i32, [C.c_char_p, C.POINTER(P)]),
    "gg_selector_collect": (i32, [P, i32, i32, i32, i32, P, P, P]),
    "gg_sssp_batch": (i32, [P, P, i32, i32, P, C.POINTER(gg_stats)]),
    "gg_sssp_parts": (i32, [P, P, i32, P, i32, P, C.POINTER(gg_stats)]),
    "gg_batch_set_selector": (i32, [P, i32, P]),
    "gg_batch_collect": (i32, [P, i32, P, i32, i32, P, P, C.POINTER(i32)]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libgg.so (once) and declares every exported signature."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (the engine has no non-CUDA fallback)")
        L = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib().gg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != GG_OK:
        raise GGError(status, last_error())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
