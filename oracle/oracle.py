"""CPU parity oracle: a ctypes front-end over ``celltree_oracle.c``.

TEST INFRASTRUCTURE ONLY.  The test-suite, ``__graft_entry__.smoke()`` and
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) use this
module as the checker and as the timed host-core baseline.  The product
package ``numba_celltree_gb300`` never imports it.

``OracleCellTree2d`` and ``OracleEdgeCellTree2d`` restate the upstream classes
``CellTree2d`` (celltree.py:37-351) and ``EdgeCellTree2d``
(edge_celltree.py:25-146) on top of the C restatement, with the same casting
(cast.py:14-54), tolerance defaults (celltree_base.py:20-52) and outputs.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
from typing import NamedTuple, Optional

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libcelltree_oracle.so"

MIN_TOLERANCE = 1e-15  # constants.py:146
TOLERANCE_FACTOR = 1e-12  # constants.py:147
MAX_N_VERTEX = 32  # constants.py:134
FILL_VALUE = -1  # constants.py:135

NodeDType = np.dtype(  # constants.py:92-106
    [
        ("child", np.intp),
        ("Lmax", np.float64),
        ("Rmin", np.float64),
        ("ptr", np.intp),
        ("size", np.intp),
        ("dim", bool),
    ]
)

_lib = None


def build() -> pathlib.Path:
    """Compile the oracle shared library (make, gcc)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int64
_D = ctypes.c_double


class _Pt(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class _Box(ctypes.Structure):
    _fields_ = [
        ("xmin", ctypes.c_double),
        ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double),
        ("ymax", ctypes.c_double),
    ]


class _Tree(ctypes.Structure):
    _fields_ = [
        ("elements", _P),
        ("n_max_vert", _I),
        ("vertices", _P),
        ("child", _P),
        ("Lmax", _P),
        ("Rmin", _P),
        ("ptr", _P),
        ("size", _P),
        ("dim", _P),
        ("n_nodes", _I),
        ("bb_indices", _P),
        ("bb_coords", _P),
        ("bbox", _P),
    ]


def _declare(L):
    sigs = {
        "cto_pessimistic_n_nodes": (_I, [_I]),
        "cto_counter_clockwise": (None, [_P, _P, _I, _I]),
        "cto_build_face_bboxes": (None, [_P, _I, _I, _P, _P]),
        "cto_build_edge_bboxes": (None, [_P, _I, _P, _D, _P]),
        "cto_build_tree": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
        "cto_locate_points": (None, [_P, _P, _I, _D, _P]),
        "cto_locate_points_on_edge": (None, [_P, _P, _I, _D, _P]),
        "cto_count_boxes": (None, [_P, _P, _I, _P]),
        "cto_write_boxes": (None, [_P, _P, _I, _P, _P, _P]),
        "cto_count_edges": (None, [ctypes.c_int, _P, _P, _I, _P]),
        "cto_write_edges": (None, [ctypes.c_int, _P, _P, _I, _P, _P, _P, _P]),
        "cto_sort_intersections": (None, [_P, _P, _I, _P, _P]),
        "cto_polygons_intersect": (None, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P]),
        "cto_area_of_intersection": (None, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P]),
        "cto_box_area_of_intersection": (None, [_P, _P, _P, _I, _P, _P, _I, _P]),
        "cto_barycentric_triangle": (None, [_P, _P, _P, _I, _P, _I, _P]),
        "cto_barycentric_wachspress": (None, [_P, _P, _P, _I, _P, _I, _D, _P]),
        "cto_collect_node_bounds": (None, [_P, _P]),
        "cto_validate_node_bounds": (None, [_P, _P, _P]),
        "cto_cohen_sutherland": (ctypes.c_int, [_Pt, _Pt, _Box, ctypes.POINTER(_Pt), ctypes.POINTER(_Pt)]),
        "cto_liang_barsky": (ctypes.c_int, [_Pt, _Pt, _Box, ctypes.POINTER(_Pt), ctypes.POINTER(_Pt)]),
        "cto_cyrus_beck": (ctypes.c_int, [_Pt, _Pt, _P, _I, _D, ctypes.POINTER(_Pt), ctypes.POINTER(_Pt)]),
        "cto_separating_axes": (ctypes.c_int, [_P, _I, _P, _I]),
        "cto_polygon_polygon_clip_area": (_D, [_P, _I, _P, _I]),
        "cto_polygon_area": (_D, [_P, _I]),
        "cto_wachspress_weights": (None, [_P, _I, _D, _D, _P, _I, _D]),
        "cto_points_in_triangles": (None, [_P, _P, _P, _I, _P, _I, _D, _P]),
        "cto_num_threads": (ctypes.c_int, []),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _f64(a, shape_last=None) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


# --------------------------------------------------------------------------
# casting: cast.py:14-54 and celltree_base.py:20-52
# --------------------------------------------------------------------------


def cast_vertices(vertices, copy=False):
    if isinstance(vertices, np.ndarray):
        vertices = vertices.astype(np.float64, copy=copy)
    else:
        vertices = np.ascontiguousarray(vertices, dtype=np.float64)
    if vertices.ndim != 2 or vertices.shape[1] != 2:
        raise ValueError("vertices must have shape (n_points, 2)")
    return np.ascontiguousarray(vertices)


def cast_faces(faces, fill_value):
    if isinstance(faces, np.ndarray):
        faces = faces.astype(np.intp, copy=True)
    else:
        faces = np.ascontiguousarray(faces, dtype=np.intp)
    if faces.ndim != 2:
        raise ValueError("faces must have shape (n_face, n_max_vert)")
    if faces.shape[1] > MAX_N_VERTEX:
        raise ValueError("faces contains too many vertices for a single face")
    if fill_value != FILL_VALUE:
        faces[faces == fill_value] = FILL_VALUE
    return np.ascontiguousarray(faces)


def cast_bboxes(bbox_coords):
    bbox_coords = np.ascontiguousarray(bbox_coords, dtype=np.float64)
    if bbox_coords.ndim != 2 or bbox_coords.shape[1] != 4:
        raise ValueError("bbox_coords must have shape (n_box, 4)")
    return bbox_coords


def cast_edges(edges):
    edges = np.ascontiguousarray(edges, dtype=np.float64)
    if edges.ndim != 3 or edges.shape[1] != 2 or edges.shape[2] != 2:
        raise ValueError("edges must have shape (n_edge, 2, 2)")
    return edges


def bbox_tree(bb_coords):
    return np.array(
        [bb_coords[:, 0].min(), bb_coords[:, 1].max(), bb_coords[:, 2].min(), bb_coords[:, 3].max()],
        dtype=np.float64,
    )


def bbox_distances(bb_coords):
    d = np.empty((bb_coords.shape[0], 3), dtype=np.float64)
    d[:, 0] = bb_coords[:, 1] - bb_coords[:, 0]
    d[:, 1] = bb_coords[:, 3] - bb_coords[:, 2]
    d[:, 2] = np.sqrt(d[:, 0] ** 2 + d[:, 1] ** 2)
    return d


def default_tolerance(bb_diagonal):
    return max(MIN_TOLERANCE, TOLERANCE_FACTOR * max(bb_diagonal))


# --------------------------------------------------------------------------
# building blocks
# --------------------------------------------------------------------------


def counter_clockwise(vertices, faces):
    """In place, like geometry_utils.py:541-561."""
    assert faces.dtype == np.int64 and faces.flags.c_contiguous
    vertices = _f64(vertices)
    lib().cto_counter_clockwise(_ptr(vertices), _ptr(faces), faces.shape[0], faces.shape[1])


def build_face_bboxes(faces, vertices):
    faces = _i64(faces)
    vertices = _f64(vertices)
    out = np.empty((faces.shape[0], 4), dtype=np.float64)
    lib().cto_build_face_bboxes(_ptr(faces), faces.shape[0], faces.shape[1], _ptr(vertices), _ptr(out))
    return out


def build_edge_bboxes(edges, vertices, tolerance):
    edges = _i64(edges)
    vertices = _f64(vertices)
    out = np.empty((edges.shape[0], 4), dtype=np.float64)
    lib().cto_build_edge_bboxes(_ptr(edges), edges.shape[0], _ptr(vertices), float(tolerance), _ptr(out))
    return out


def build_tree(bb_coords, n_buckets=4, cells_per_leaf=2):
    """initialize creation.py:384-413 -> (nodes[NodeDType], bb_indices)."""
    bb_coords = _f64(bb_coords)
    n = bb_coords.shape[0]
    cap = lib().cto_pessimistic_n_nodes(n)
    child = np.empty(cap, np.int64)
    Lmax = np.empty(cap, np.float64)
    Rmin = np.empty(cap, np.float64)
    ptr = np.empty(cap, np.int64)
    size = np.empty(cap, np.int64)
    dim = np.empty(cap, np.uint8)
    bbi = np.empty(n, np.int64)
    n_nodes = lib().cto_build_tree(
        _ptr(bb_coords), n, int(n_buckets), int(cells_per_leaf),
        _ptr(child), _ptr(Lmax), _ptr(Rmin), _ptr(ptr), _ptr(size), _ptr(dim), _ptr(bbi),
    )
    if n_nodes < 0:
        raise RuntimeError("tree construction failed: a centroid fell outside every bucket")
    nodes = np.empty(n_nodes, dtype=NodeDType)
    nodes["child"] = child[:n_nodes]
    nodes["Lmax"] = Lmax[:n_nodes]
    nodes["Rmin"] = Rmin[:n_nodes]
    nodes["ptr"] = ptr[:n_nodes]
    nodes["size"] = size[:n_nodes]
    nodes["dim"] = dim[:n_nodes].astype(bool)
    return nodes, bbi


class _TreeArrays:
    """Keeps the numpy arrays alive behind the ctypes tree descriptor."""

    def __init__(self, elements, vertices, nodes, bb_indices, bb_coords, bbox):
        self.elements = _i64(elements)
        self.vertices = _f64(vertices)
        self.child = np.ascontiguousarray(nodes["child"], dtype=np.int64)
        self.Lmax = np.ascontiguousarray(nodes["Lmax"], dtype=np.float64)
        self.Rmin = np.ascontiguousarray(nodes["Rmin"], dtype=np.float64)
        self.ptr = np.ascontiguousarray(nodes["ptr"], dtype=np.int64)
        self.size = np.ascontiguousarray(nodes["size"], dtype=np.int64)
        self.dim = np.ascontiguousarray(nodes["dim"], dtype=np.uint8)
        self.bb_indices = _i64(bb_indices)
        self.bb_coords = _f64(bb_coords)
        self.bbox = _f64(bbox)
        self.desc = _Tree(
            _ptr(self.elements), self.elements.shape[1], _ptr(self.vertices),
            _ptr(self.child), _ptr(self.Lmax), _ptr(self.Rmin), _ptr(self.ptr), _ptr(self.size), _ptr(self.dim),
            len(self.child), _ptr(self.bb_indices), _ptr(self.bb_coords), _ptr(self.bbox),
        )


class CellTreeData(NamedTuple):  # constants.py:82-89
    elements: np.ndarray
    vertices: np.ndarray
    nodes: np.ndarray
    bb_indices: np.ndarray
    bb_coords: np.ndarray
    bbox: np.ndarray
    cells_per_leaf: int


class _OracleBase:
    def _arrays(self):
        # Rebuilt on every call so that edits to ``nodes`` (as the upstream
        # node-validity test does) are seen.
        return _TreeArrays(self._elements, self.vertices, self.nodes, self.bb_indices, self.bb_coords, self.bbox)

    @property
    def node_bounds(self):
        t = self._arrays()
        out = np.empty((len(self.nodes), 4), dtype=np.float64)
        lib().cto_collect_node_bounds(ctypes.byref(t.desc), _ptr(out))
        return out

    def validate_node_bounds(self):
        t = self._arrays()
        nb = self.node_bounds
        out = np.empty(len(self.nodes), dtype=np.uint8)
        lib().cto_validate_node_bounds(ctypes.byref(t.desc), _ptr(nb), _ptr(out))
        return out.astype(bool)

    def to_dict_of_lists(self):
        d = {}
        for i, c in enumerate(self.nodes["child"]):
            d[i] = [] if c == -1 else [int(c), int(c) + 1]
        return d

    def _multi(self, mode, edge_coords):
        t = self._arrays()
        n = edge_coords.shape[0]
        counts = np.empty(n, np.int64)
        lib().cto_count_edges(mode, ctypes.byref(t.desc), _ptr(edge_coords), n, _ptr(counts))
        offsets = np.zeros(n, np.int64)
        if n:
            offsets[1:] = np.cumsum(counts)[:-1]
        total = int(counts.sum())
        ii = np.empty(total, np.int64)
        jj = np.empty(total, np.int64)
        xy = np.empty((total, 2, 2), np.float64)
        lib().cto_write_edges(mode, ctypes.byref(t.desc), _ptr(edge_coords), n, _ptr(offsets), _ptr(ii), _ptr(jj), _ptr(xy))
        order = np.empty(total, np.int64)
        lib().cto_sort_intersections(_ptr(ii), _ptr(xy), total, _ptr(edge_coords), _ptr(order))
        return ii[order], jj[order], xy[order]


class OracleCellTree2d(_OracleBase):
    """CPU restatement of CellTree2d (celltree.py:37-351)."""

    def __init__(self, vertices, faces, fill_value, n_buckets: int = 4, cells_per_leaf: int = 2):
        if n_buckets < 2:
            raise ValueError("n_buckets must be >= 2")
        if cells_per_leaf < 1:
            raise ValueError("cells_per_leaf must be >= 1")
        vertices = cast_vertices(vertices, copy=True)
        faces = cast_faces(faces, fill_value)
        counter_clockwise(vertices, faces)
        bb_coords = build_face_bboxes(faces, vertices)
        nodes, bb_indices = build_tree(bb_coords, n_buckets, cells_per_leaf)
        self.vertices = vertices
        self.faces = faces
        self._elements = faces
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self.nodes = nodes
        self.bb_indices = bb_indices
        self.bb_coords = bb_coords
        self.bbox = bbox_tree(bb_coords)
        self.bb_distances = bbox_distances(bb_coords)
        self.celltree_data = CellTreeData(faces, vertices, nodes, bb_indices, bb_coords, self.bbox, cells_per_leaf)

    def locate_points(self, points, tolerance: Optional[float] = None):
        if tolerance is None:
            tolerance = default_tolerance(self.bb_distances[:, 2])
        points = cast_vertices(points)
        t = self._arrays()
        out = np.empty(len(points), np.int64)
        lib().cto_locate_points(ctypes.byref(t.desc), _ptr(points), len(points), float(tolerance), _ptr(out))
        return out

    def locate_boxes(self, bbox_coords):
        bbox_coords = cast_bboxes(bbox_coords)
        t = self._arrays()
        n = bbox_coords.shape[0]
        counts = np.empty(n, np.int64)
        lib().cto_count_boxes(ctypes.byref(t.desc), _ptr(bbox_coords), n, _ptr(counts))
        offsets = np.zeros(n, np.int64)
        if n:
            offsets[1:] = np.cumsum(counts)[:-1]
        total = int(counts.sum())
        ii = np.empty(total, np.int64)
        jj = np.empty(total, np.int64)
        lib().cto_write_boxes(ctypes.byref(t.desc), _ptr(bbox_coords), n, _ptr(offsets), _ptr(ii), _ptr(jj))
        return ii, jj

    def intersect_boxes(self, bbox_coords):
        bbox_coords = cast_bboxes(bbox_coords)
        i, j = self.locate_boxes(bbox_coords)
        area = np.empty(len(i), np.float64)
        lib().cto_box_area_of_intersection(
            _ptr(bbox_coords), _ptr(self.vertices), _ptr(self.faces), self.faces.shape[1], _ptr(i), _ptr(j), len(i), _ptr(area)
        )
        actual = area > 0
        return i[actual], j[actual], area[actual]

    def locate_faces(self, vertices, faces):
        counter_clockwise(vertices, faces)
        bbox_coords = build_face_bboxes(faces, vertices)
        si, sj = self.locate_boxes(bbox_coords)
        out = np.empty(len(si), np.uint8)
        lib().cto_polygons_intersect(
            _ptr(_f64(vertices)), _ptr(self.vertices), _ptr(faces), faces.shape[1], _ptr(self.faces), self.faces.shape[1],
            _ptr(si), _ptr(sj), len(si), _ptr(out),
        )
        keep = out.astype(bool)
        return si[keep], sj[keep]

    def intersect_faces(self, vertices, faces, fill_value):
        vertices = cast_vertices(vertices)
        faces = cast_faces(faces, fill_value)
        i, j = self.locate_faces(vertices, faces)
        area = np.empty(len(i), np.float64)
        lib().cto_area_of_intersection(
            _ptr(vertices), _ptr(self.vertices), _ptr(faces), faces.shape[1], _ptr(self.faces), self.faces.shape[1],
            _ptr(i), _ptr(j), len(i), _ptr(area),
        )
        actual = area > 0
        return i[actual], j[actual], area[actual]

    def intersect_edges(self, edge_coords):
        edge_coords = cast_edges(edge_coords)
        return self._multi(1, edge_coords)

    def compute_barycentric_weights(self, points, tolerance: Optional[float] = None):
        if tolerance is None:
            tolerance = default_tolerance(self.bb_distances[:, 2])
        points = cast_vertices(points)
        face_indices = self.locate_points(points, tolerance)
        K = self.faces.shape[1]
        n = len(points)
        if K > 3:
            w = np.empty((n, K), np.float64)
            lib().cto_barycentric_wachspress(
                _ptr(points), _ptr(face_indices), _ptr(self.faces), K, _ptr(self.vertices), n, float(tolerance), _ptr(w)
            )
        else:
            w = np.empty((n, 3), np.float64)
            lib().cto_barycentric_triangle(
                _ptr(points), _ptr(face_indices), _ptr(self.faces), K, _ptr(self.vertices), n, _ptr(w)
            )
        return face_indices, w


class OracleEdgeCellTree2d(_OracleBase):
    """CPU restatement of EdgeCellTree2d (edge_celltree.py:25-146)."""

    def __init__(self, vertices, edges, n_buckets: int = 4, cells_per_leaf: int = 2):
        if n_buckets < 2:
            raise ValueError("n_buckets must be >= 2")
        if cells_per_leaf < 1:
            raise ValueError("cells_per_leaf must be >= 1")
        vertices = cast_vertices(vertices, copy=True)
        x, y = vertices.T
        dx = x.max() - x.min()
        dy = y.max() - y.min()
        tol = max(MIN_TOLERANCE, TOLERANCE_FACTOR * max(dx, dy))
        edges_i = _i64(edges)
        bb_coords = build_edge_bboxes(edges_i, vertices, tol)
        nodes, bb_indices = build_tree(bb_coords, n_buckets, cells_per_leaf)
        self.vertices = vertices
        self.edges = edges
        self._elements = edges_i
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self.nodes = nodes
        self.bb_indices = bb_indices
        self.bb_coords = bb_coords
        self.bbox = bbox_tree(bb_coords)
        self.bb_distances = bbox_distances(bb_coords)
        self.celltree_data = CellTreeData(edges, vertices, nodes, bb_indices, bb_coords, self.bbox, cells_per_leaf)

    def locate_points(self, points, tolerance: Optional[float] = None):
        if tolerance is None:
            tolerance = default_tolerance(self.bb_distances[:, 2])
        points = cast_vertices(points)
        t = self._arrays()
        out = np.empty(len(points), np.int64)
        lib().cto_locate_points_on_edge(ctypes.byref(t.desc), _ptr(points), len(points), float(tolerance), _ptr(out))
        return out

    def intersect_edges(self, edge_coords):
        edge_coords = cast_edges(edge_coords)
        ii, jj, xy = self._multi(0, edge_coords)
        return ii, jj, np.ascontiguousarray(xy[:, 0])


# --------------------------------------------------------------------------
# single-call helpers (unit-level golden checks)
# --------------------------------------------------------------------------


def _pt(p):
    return _Pt(float(p[0]), float(p[1]))


def cohen_sutherland_line_box_clip(a, b, box):
    c, d = _Pt(), _Pt()
    r = lib().cto_cohen_sutherland(_pt(a), _pt(b), _Box(*map(float, box)), ctypes.byref(c), ctypes.byref(d))
    return bool(r == 1), (c.x, c.y), (d.x, d.y)


def liang_barsky_line_box_clip(a, b, box):
    c, d = _Pt(), _Pt()
    r = lib().cto_liang_barsky(_pt(a), _pt(b), _Box(*map(float, box)), ctypes.byref(c), ctypes.byref(d))
    return bool(r == 1), (c.x, c.y), (d.x, d.y)


def cyrus_beck_line_polygon_clip(a, b, poly, tolerance):
    poly = _f64(poly)
    c, d = _Pt(), _Pt()
    r = lib().cto_cyrus_beck(_pt(a), _pt(b), _ptr(poly), len(poly), float(tolerance), ctypes.byref(c), ctypes.byref(d))
    return bool(r == 1), (c.x, c.y), (d.x, d.y)


def separating_axes(a, b):
    a = _f64(a)
    b = _f64(b)
    return bool(lib().cto_separating_axes(_ptr(a), len(a), _ptr(b), len(b)))


def polygon_polygon_clip_area(polygon, clipper):
    polygon = _f64(polygon)
    clipper = _f64(clipper)
    return lib().cto_polygon_polygon_clip_area(_ptr(polygon), len(polygon), _ptr(clipper), len(clipper))


def polygon_area(polygon):
    polygon = _f64(polygon)
    return lib().cto_polygon_area(_ptr(polygon), len(polygon))


def wachspress_weights(polygon, p, n_weights, tolerance):
    polygon = _f64(polygon)
    w = np.zeros(n_weights, np.float64)
    lib().cto_wachspress_weights(_ptr(polygon), len(polygon), float(p[0]), float(p[1]), _ptr(w), n_weights, float(tolerance))
    return w


def points_in_triangles(points, face_indices, faces, vertices, tolerance):
    points = _f64(points)
    face_indices = _i64(face_indices)
    faces = _i64(faces)
    vertices = _f64(vertices)
    out = np.empty(len(points), np.uint8)
    lib().cto_points_in_triangles(
        _ptr(points), _ptr(face_indices), _ptr(faces), faces.shape[1], _ptr(vertices), len(points), float(tolerance), _ptr(out)
    )
    return out.astype(bool)


def num_threads() -> int:
    return int(lib().cto_num_threads())


if __name__ == "__main__":  # pragma: no cover
    print(build())
