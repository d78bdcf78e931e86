"""ctypes binding of ``libcelltree_gb300.so`` (declared in include/celltree_gb300.h).

The library is the product's compute path; there is no fallback.  Loading it
fails loudly when it is missing or was built for another ABI version.
"""

from __future__ import annotations

import ctypes
import pathlib

from . import build as _build

LIB_PATH = _build.LIB_PATH
ABI_VERSION = 3

CT_OK = 0
CT_ERR_CUDA = 1
CT_ERR_ARG = 2
CT_ERR_WORKSPACE = 3
CT_ERR_DEVICE = 4

CT_MODE_FP64 = 0
CT_MODE_FP32 = 1

DEVERR_STACK = 1
DEVERR_BUCKET = 2
DEVERR_CLIP = 4
DEVERR_CAPACITY = 8
DEVERR_LOOP = 16
DEVERR_NONFINITE = 32

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_D = ctypes.c_double
_SZ = ctypes.c_size_t


class CtTree(ctypes.Structure):
    """Mirror of ``struct ct_tree`` in include/celltree_gb300.h."""

    _fields_ = [
        ("elements", _P),
        ("vertices", _P),
        ("bb_indices", _P),
        ("bb_coords", _P),
        ("node_child", _P),
        ("node_Lmax", _P),
        ("node_Rmin", _P),
        ("node_ptr", _P),
        ("node_size", _P),
        ("node_dim", _P),
        ("n_elements", _I64),
        ("n_vertices", _I64),
        ("n_nodes", _I64),
        ("n_max_vert", _I32),
        ("max_depth", _I32),
        ("bbox", _D * 4),
        ("nodes_f32", _P),
        ("nodes_f64", _P),
        ("poly_f64", _P),
        ("poly_f32", _P),
        ("poly_len", _P),
        ("poly_len32", _P),
        ("origin", _D * 2),
        ("vmax", ctypes.c_float),
        ("abs_eps", ctypes.c_float),
        ("error_word", _P),
        ("grid_start", _P),
        ("grid_nx", _I32),
        ("grid_ny", _I32),
        ("grid_x0", ctypes.c_float),
        ("grid_y0", ctypes.c_float),
        ("grid_sx", ctypes.c_float),
        ("grid_sy", ctypes.c_float),
        ("cand_off", _P),
        ("cand_idx", _P),
        ("cand_lbox", _P),
        ("cand_box", _P),
        ("cand_n", _I64),
        ("cand_tol", _D),
        ("bounds_finite", _I32),
        ("bb_leaf", _P),
        ("node_box", _P),
        ("leaf_start", _P),
        ("tune_cells_bpsm", _I32),
        ("tune_fast_bpsm", _I32),
        ("tune_query_threads", _I32),
        ("tune_fp64_stack", _I32),
        ("node_parent", _P),
        ("bb_leaf32", _P),
    ]


class CtForestPlan(ctypes.Structure):
    """Mirror of ``struct ct_forest_plan``."""

    _fields_ = [
        ("n_points", _I64),
        ("n_trees", _I32),
        ("kt", _I32),
        ("stack", _I32),
        ("morton_bits", _I32),
        ("error_word", _P),
        ("max_tree_points", _I64),
        ("tune_cells_bpsm", _I32),
        ("tune_fast_bpsm", _I32),
    ]


class CtForestIndex(ctypes.Structure):
    """Mirror of ``struct ct_forest_index``."""

    _fields_ = [(n, _P) for n in (
        "vertices", "faces", "face_off", "poly32_off", "tree_K", "bb_coords", "tree_off", "node_off", "max_depth",
        "node_child", "node_Lmax", "node_Rmin", "node_ptr", "node_size", "node_dim", "bb_indices", "grid_start",
        "grid_off", "grid_nx", "grid_ny")] + [
        ("n_total", _I64),
        ("node_capacity", _I64),
        ("grid_cells", _I64),
        ("n_trees", _I32),
        ("k_max", _I32),
        ("stack", _I32),
        ("pad_", _I32),
        ("tolerance", _D),
    ] + [(n, _P) for n in ("nodes_f32", "nodes_f64", "poly_f64", "poly_f32", "poly_len", "poly_len32", "summary",
                           "error_word", "cand_count", "cand_off", "cand_box", "cand_idx", "cand_lbox",
                           "cand_scan_ws")] + [
        ("cand_scan_bytes", _SZ),
        ("cand_capacity", _I64),
    ]


# name -> (restype, argtypes)
SIGNATURES = {
    "ct_abi_version": (ctypes.c_int, []),
    "ct_last_error_message": (ctypes.c_char_p, []),
    "ct_validate_elements": (ctypes.c_int, [_P, _I64, _I32, _I32, _I64, ctypes.POINTER(_I32), _P]),
    "ct_counter_clockwise": (ctypes.c_int, [_P, _P, _I64, _I32, _P]),
    "ct_face_bboxes": (ctypes.c_int, [_P, _P, _I64, _I32, _P, _P]),
    "ct_edge_bboxes": (ctypes.c_int, [_P, _P, _I64, _D, _P, _P]),
    "ct_bbox_summary": (ctypes.c_int, [_P, _I64, _P, ctypes.POINTER(_D), _P]),
    "ct_vertex_extent": (ctypes.c_int, [_P, _I64, ctypes.POINTER(_D), _P]),
    "ct_pessimistic_n_nodes": (_I64, [_I64]),
    "ct_grid_shape": (ctypes.c_int, [_I64, _D, _D, _D, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "ct_build_forest_workspace_size": (_SZ, [_I64, _I32, _I32, _I32]),
    "ct_build_forest": (ctypes.c_int, [_P, _I64, ctypes.POINTER(_I64), _I32, _I32, _I64, _I32, _P, _SZ,
                                       ctypes.POINTER(_I64), ctypes.POINTER(_I32), _P]),
    "ct_build_forest_async": (ctypes.c_int, [_P, _I64, ctypes.POINTER(_I64), _P, _I32, _I32, _I64, _I32, _P, _SZ,
                                             _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ct_build_forest_emit": (ctypes.c_int, [_P, _I64, _I32, _I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ct_forest_locate_workspace_size": (_SZ, [_I64, _I32]),
    "ct_forest_locate_prepare": (ctypes.c_int, [_P, _I32, ctypes.POINTER(_D), ctypes.POINTER(_I64), _I64,
                                                _P, _P, _SZ, _P]),
    "ct_forest_locate": (ctypes.c_int, [_P, _P, _P, _P, _SZ, _P]),
    "ct_forest_index_prepare": (ctypes.c_int, [ctypes.POINTER(CtForestIndex), ctypes.POINTER(_I64), _I64, _P, _P,
                                               _SZ, _P]),
    "ct_forest_index_build": (ctypes.c_int, [ctypes.POINTER(CtForestIndex), _P, _P, _SZ, _P]),
    "ct_pack_grid": (ctypes.c_int, [_P, _P]),
    "ct_cand_scratch_size": (_SZ, [_P]),
    "ct_cand_count": (ctypes.c_int, [_P, _D, _P, _SZ, ctypes.POINTER(_I64), _P]),
    "ct_cand_fill": (ctypes.c_int, [_P, _P, _SZ, _P]),
    "ct_build_workspace_size": (_SZ, [_I64, _I32, _I32]),
    "ct_build_tree": (
        ctypes.c_int,
        [_P, _I64, _I32, _I64, _I32, _P, _SZ, ctypes.POINTER(_I64), ctypes.POINTER(_I32), _P],
    ),
    "ct_build_emit": (ctypes.c_int, [_P, _I64, _I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ct_build_tree_noalloc": (
        ctypes.c_int,
        [_P, _I64, _I32, _I64, _P, _P, _P, _P, _P, _P, _I64, _P, ctypes.POINTER(_I64), ctypes.POINTER(_I32), _P],
    ),
    "ct_pack_tree": (ctypes.c_int, [ctypes.POINTER(CtTree), _P]),
    "ct_poly32_stride": (ctypes.c_int, [_I32]),
    "ct_abi_sizeof": (_SZ, [_I32]),
    "ct_host_register": (ctypes.c_int, [_P, _SZ, _I32]),
    "ct_host_unregister": (ctypes.c_int, [_P]),
    "ct_locate_points": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _D, _I32, _P, _P]),
    "ct_locate_points_on_edge": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _D, _P, _P]),
    "ct_locate_workspace_size": (_SZ, [_I64, _I32]),
    "ct_locate_points_batched": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _D, _I32, _P, _P, _SZ, _P]),
    "ct_locate_bin": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _I32, _P, _SZ, _P]),
    "ct_locate_fast": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _D, _I32, _P, _P, _SZ, _P]),
    "ct_locate_exact": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _D, _I32, _P, _P, _SZ, _P]),
    "ct_locate_deferred_count": (ctypes.c_int, [_P, _I64, _I32, ctypes.POINTER(_I64), _P]),
    "ct_scan_workspace_size": (_SZ, [_I64]),
    "ct_exclusive_scan": (ctypes.c_int, [_P, _I64, _P, _P, _SZ, ctypes.POINTER(_I64), _P]),
    "ct_box_index_scratch_size": (_SZ, [ctypes.POINTER(CtTree)]),
    "ct_pack_box_index": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _SZ, _P]),
    "ct_count_boxes": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _P, _P, _P]),
    "ct_write_boxes": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _P, _P, _P, _P, _P]),
    "ct_sort_workspace_size": (_SZ, [_I64]),
    "ct_sort_intersections": (ctypes.c_int, [_P, _I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _SZ, _P]),
    "ct_polygons_intersect": (ctypes.c_int, [_P, _P, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P]),
    "ct_area_of_intersection": (ctypes.c_int, [_P, _P, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P, _P]),
    "ct_box_area_of_intersection": (ctypes.c_int, [_P, _P, _P, _I32, _P, _P, _I64, _P, _P, _P]),
    "ct_area_of_intersection_ordered": (ctypes.c_int, [_P, _P, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P, _P, _P]),
    "ct_box_area_of_intersection_ordered": (ctypes.c_int, [_P, _P, _P, _I32, _P, _P, _I64, _P, _P, _P, _P]),
    "ct_pair_order_workspace_size": (_SZ, [_I64]),
    "ct_pair_order": (ctypes.c_int, [_P, _I32, _P, _P, _I32, _P, _I64, _P, _P, _SZ, _P]),
    "ct_liang_barsky_line_box_clip": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _P, _P]),
    "ct_points_in_triangles": (ctypes.c_int, [_P, _P, _I64, _P, _I32, _I64, _P, _D, _P, _P, _P]),
    "ct_csr_workspace_size": (_SZ, [_I64]),
    "ct_work_order_workspace_size": (_SZ, [_I64]),
    "ct_count_edge_candidates": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _P, _P]),
    "ct_write_edge_candidates": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _P, _P, _P, _P]),
    "ct_write_boxes_workspace_size": (ctypes.c_size_t, [_I64, _I32]),
    "ct_write_boxes_ws": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _P, _P, _I64, _I32, _P, _P, _P,
                                         ctypes.c_size_t, _P]),
    "ct_count_boxes_spec": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _P, _P, _P, _I32, _P]),
    "ct_write_boxes_spec": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _I64, _P, _P, _P, _P, _I32, _I64, _I32, _P, _P,
                                           _P, ctypes.c_size_t, _P]),
    "ct_count_edge_candidates_spec": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _P, _P, _I32, _P]),
    "ct_write_edge_candidates_spec": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _P, _P, _P, _I32, _P,
                                                     _P, _P]),
    "ct_cs_certificates": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _P, _P, _I64, _P, _P]),
    "ct_count_edge_items": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _I32, _P, _P]),
    "ct_write_edge_items": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _I64, _P, _I32, _P, _P, _P, _P]),
    "ct_count_item_candidates": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _P, _P, _I64, _P, _P]),
    "ct_write_item_candidates": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "ct_segment_candidate_ranges": (ctypes.c_int, [_P, _P, _I64, _P, _P, _I64, _P, _P, _P]),
    "ct_test_edge_candidates": (ctypes.c_int, [ctypes.POINTER(CtTree), _I32, _P, _P, _P, _I64, _P, _P, _P]),
    "ct_compact_edge_hits": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P, _P,
                                            _P, _P, _P, _P]),
    "ct_work_order": (ctypes.c_int, [_P, _I64, _I32, _D, _P, _P, _SZ, _P]),
    "ct_radix_pass_workspace_size": (_SZ, []),
    "ct_radix_pass": (ctypes.c_int, [_P, _P, _I64, _I32, _P, _P, _P, _SZ, _P]),
    "ct_csr_row_ptr": (ctypes.c_int, [_P, _I64, _I64, _P, _P, _SZ, _P, _P]),
    "ct_csr_weighted_mean": (ctypes.c_int, [_P, _P, _P, _I64, _I64, _P, _P, _P, _P, _P]),
    "ct_area_of_intersection_grad": (ctypes.c_int, [_P, _P, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P, _P, _P, _P]),
    "ct_barycentric_weights_grad": (ctypes.c_int, [_P, _P, _I64, _P, _P, _I32, _I32, _D, _P, _P, _P, _P]),
    "ct_compact_workspace_size": (_SZ, [_I64]),
    "ct_compact_pairs": (ctypes.c_int, [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _SZ, ctypes.POINTER(_I64), _P]),
    "ct_barycentric_weights": (ctypes.c_int, [ctypes.POINTER(CtTree), _P, _P, _I64, _D, _P, _P]),
    "ct_node_bounds": (ctypes.c_int, [_P, _P, _P, _P, _I64, ctypes.POINTER(_D), _P, _P, _P]),
    "ct_validate_node_bounds": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _P, _P, _P]),
}

_lib = None


class CellTreeError(RuntimeError):
    """A call into libcelltree_gb300 failed."""


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = pathlib.Path(LIB_PATH)
    if not path.exists() and build_if_missing:
        _build.build()
    if not path.exists():
        raise ImportError(f"libcelltree_gb300.so not found at {path}; run numba_celltree_gb300.build.build()")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    v = lib.ct_abi_version()
    if v != ABI_VERSION:
        raise ImportError(f"libcelltree_gb300 ABI {v} != expected {ABI_VERSION}")
    _lib = lib
    return lib


def device_error_text(err: int) -> str:
    """The CT_DEVERR_* bits of a device error word, in words."""
    names = [(DEVERR_STACK, "traversal stack overflow"), (DEVERR_BUCKET, "centroid outside every bucket"),
             (DEVERR_CLIP, "clip polygon overflow"), (DEVERR_CAPACITY, "output capacity exceeded"),
             (DEVERR_LOOP, "bounded loop gave up"), (DEVERR_NONFINITE, "non-finite coordinate")]
    return ", ".join(text for bit, text in names if err & bit) or f"{err:#x}"


def check(status: int, what: str = "") -> None:
    if status == CT_OK:
        return
    msg = load().ct_last_error_message().decode(errors="replace")
    if status == CT_ERR_ARG:
        raise ValueError(f"{what}: {msg}" if what else msg)
    raise CellTreeError(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")
