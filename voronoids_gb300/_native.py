"""Loads ``libvoronoids_gpu.so`` and declares the C ABI (include/voronoids_gpu.h).

There is no CPU fallback: if the library is missing or cannot be loaded the
import of the API fails loudly.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvoronoids_gpu.so")

STATUS = {
    0: "VD_OK", 1: "VD_ERR_ARG", 2: "VD_ERR_CUDA", 3: "VD_ERR_NOMEM", 4: "VD_ERR_DUPLICATE",
    5: "VD_ERR_NONFINITE", 6: "VD_ERR_OUTSIDE", 7: "VD_ERR_PRECISION", 8: "VD_ERR_ROUND_LIMIT",
    9: "VD_ERR_CAVITY", 10: "VD_ERR_WALK", 11: "VD_ERR_INTERNAL", 12: "VD_ERR_DEGENERATE",
    13: "VD_ERR_RANGE",
}
VD_OK = 0
VD_ERR_DUPLICATE = 4

# Every symbol include/voronoids_gpu.h declares.
EXPORTS = [
    "vd_tree_new", "vd_tree_new_on_stream", "vd_tree_free", "vd_super_simplex", "vd_tree_new_device",
    "vd_tree_reset", "vd_tree_reset_device", "vd_delaunay_tree", "vd_delaunay_device", "vd_edges_u32", "vd_insert_points",
    "vd_insert_points_device", "vd_insert_point", "vd_locate", "vd_num_vertices",
    "vd_max_simplex_id", "vd_num_simplices", "vd_simplices", "vd_num_edges", "vd_edges",
    "vd_edges_device", "vd_check_delaunay", "vd_duplicates", "vd_get_stats", "vd_status_str",
    "vd_delaunay", "vd_set_schedule", "vd_set_tuning", "vd_set_graphs", "vd_set_profiling", "vd_profile", "vd_profile_name", "vd_set_trace", "vd_trace", "vd_kernel_launches", "vd_edges_from_simplices_noalloc",
    "vd_batch_delaunay", "vd_batch_delaunay_device", "vd_num_sets", "vd_tree_create",
    "vd_set_launch", "vd_autotune_batch", "vd_locate_points", "vd_set_adjacent", "vd_circumspheres", "vd_set_small_rounds", "vd_set_early_phase", "vd_set_exact_tier", "vd_set_first_block",
    "vd_server_new", "vd_server_submit", "vd_server_poll", "vd_server_result", "vd_server_stats", "vd_server_free",
    "vd_check_triangulation", "vd_voronoi_edges", "vd_voronoi_cells",
]


class VdStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in (
        "rounds", "inserted", "duplicates", "live_simplices", "slots", "created", "killed",
        "max_cavity", "max_facets", "pred_f32", "pred_f64", "pred_exact", "pred_sos",
        "walk_steps", "cavity_tests", "deferred_overflow", "deferred_pool", "candidates",
        "searched", "won_pass0", "won_pass1", "won_pass2", "spilled", "max_search_levels")]


_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (building nothing).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    i64 = ctypes.c_int64
    i64p = ctypes.POINTER(ctypes.c_int64)
    i32p = ctypes.POINTER(ctypes.c_int32)
    ip = ctypes.POINTER(ctypes.c_int)
    sig = {
        "vd_tree_new": ([ctypes.c_int, dp, i64, ip], vp),
        "vd_tree_new_on_stream": ([ctypes.c_int, dp, i64, vp, ip], vp),
        "vd_tree_free": ([vp], None),
        "vd_super_simplex": ([ctypes.c_int, dp, i64, dp, dp], ctypes.c_int),
        "vd_tree_new_device": ([ctypes.c_int, vp, i64, vp, ip], vp),
        "vd_tree_reset": ([vp, dp, i64], ctypes.c_int),
        "vd_tree_reset_device": ([vp, vp, i64], ctypes.c_int),
        "vd_delaunay_tree": ([vp, dp, i64, ctypes.c_uint64, vp, i64, i64p], ctypes.c_int),
        "vd_delaunay_device": ([vp, vp, i64, ctypes.c_uint64, vp, i64, i64p], ctypes.c_int),
        "vd_edges_u32": ([vp, vp, i64, i64p], ctypes.c_int),
        "vd_insert_points": ([vp, dp, i64, ctypes.c_uint64], ctypes.c_int),
        "vd_insert_points_device": ([vp, vp, i64, ctypes.c_uint64], ctypes.c_int),
        "vd_insert_point": ([vp, dp], ctypes.c_int),
        "vd_locate": ([vp, dp, i64p, i64, i64p], ctypes.c_int),
        "vd_num_vertices": ([vp, i64p], ctypes.c_int),
        "vd_max_simplex_id": ([vp, i64p], ctypes.c_int),
        "vd_num_simplices": ([vp, i64p], ctypes.c_int),
        "vd_simplices": ([vp, i32p, i32p, i64, i64p], ctypes.c_int),
        "vd_num_edges": ([vp, i64p], ctypes.c_int),
        "vd_edges": ([vp, i64p, i64, i64p], ctypes.c_int),
        "vd_edges_device": ([vp, vp, i64, i64p], ctypes.c_int),
        "vd_check_delaunay": ([vp, ip, i64p], ctypes.c_int),
        "vd_check_triangulation": ([ctypes.c_int, dp, i64, i32p, i32p, i64, ip, i64p], ctypes.c_int),
        "vd_voronoi_edges": ([vp, i64p, i64, i64p], ctypes.c_int),
        "vd_voronoi_cells": ([vp, i64p, i64p, i64], ctypes.c_int),
        "vd_duplicates": ([vp, i64p, i64, i64p], ctypes.c_int),
        "vd_get_stats": ([vp, ctypes.POINTER(VdStats)], ctypes.c_int),
        "vd_status_str": ([ctypes.c_int], ctypes.c_char_p),
        "vd_delaunay": ([ctypes.c_int, dp, i64, ctypes.c_uint64, i64p, i64, i64p], ctypes.c_int),
        "vd_set_profiling": ([vp, ctypes.c_int], ctypes.c_int),
        "vd_set_schedule": ([vp, i64, ctypes.c_double, ctypes.c_double], ctypes.c_int),
        "vd_set_tuning": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "vd_set_graphs": ([vp, ctypes.c_int], ctypes.c_int),
        "vd_batch_delaunay": ([vp, dp, i64p, ctypes.c_int, ctypes.c_uint64, vp, i64, i64p], ctypes.c_int),
        "vd_batch_delaunay_device": ([vp, vp, i64p, ctypes.c_int, ctypes.c_uint64, vp, i64, i64p], ctypes.c_int),
        "vd_num_sets": ([vp, ip], ctypes.c_int),
        "vd_tree_create": ([ctypes.c_int, vp, ip], vp),
        "vd_set_launch": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "vd_set_adjacent": ([vp, ctypes.c_int], ctypes.c_int),
        "vd_set_small_rounds": ([vp, ctypes.c_int], ctypes.c_int),
        "vd_set_early_phase": ([vp, i64, ctypes.c_int, ctypes.c_double], ctypes.c_int),
        "vd_set_first_block": ([vp, i64], ctypes.c_int),
        "vd_set_exact_tier": ([vp, ctypes.c_int, i64], ctypes.c_int),
        "vd_circumspheres": ([vp, dp, dp, i64, i64p], ctypes.c_int),
        "vd_locate_points": ([vp, dp, i64, i64p, i64p, i64], ctypes.c_int),
        "vd_autotune_batch": ([vp, vp, i64p, ctypes.c_int, i64, i64p], ctypes.c_int),
        "vd_server_new": ([ctypes.c_uint64, ctypes.c_int, i64, ctypes.c_uint64, ip], vp),
        "vd_server_submit": ([vp, ctypes.c_int, dp, i64, i64p], ctypes.c_int),
        "vd_server_poll": ([vp, i64p, i64, i64p, ctypes.c_int], ctypes.c_int),
        "vd_server_result": ([vp, i64, vp, i64, i64p, ip], ctypes.c_int),
        "vd_server_stats": ([vp, i64p], ctypes.c_int),
        "vd_server_free": ([vp], None),
        "vd_profile": ([vp, dp, i64p, ctypes.c_int, ip], ctypes.c_int),
        "vd_profile_name": ([ctypes.c_int], ctypes.c_char_p),
        "vd_set_trace": ([vp, ctypes.c_int], ctypes.c_int),
        "vd_trace": ([vp, i64p, i64, i64p], ctypes.c_int),
        "vd_kernel_launches": ([], ctypes.c_int64),
        "vd_edges_from_simplices_noalloc": ([ctypes.c_int, vp, i64, i64, vp, i64, i64p, vp], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L
