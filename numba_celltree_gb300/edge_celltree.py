"""EdgeCellTree2d on the GPU -- drop-in for numba_celltree.EdgeCellTree2d
(edge_celltree.py:25-146 upstream)."""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _device, _lib
from .cast import cast_edges, cast_vertices, is_cuda_tensor
from .celltree_base import CellTree2dBase, _GpuTree, _validate_params, prebuilt_from_nodes, validate_elements
from .constants import MIN_TOLERANCE, TOLERANCE_FACTOR


def _edge_boxes(v_d, e_d):
    """Edge boxes widened by the global tolerance of the vertex extent
    (edge_celltree.py:59-64, build_edge_bboxes geometry_utils.py:474-487)."""
    torch = _device.torch()
    lib = _lib.load()
    st = _device.stream()
    ext = (ctypes.c_double * 4)()
    _lib.check(lib.ct_vertex_extent(_device.ptr(v_d), int(v_d.shape[0]), ext, st), "vertex_extent")
    dx = ext[1] - ext[0]
    dy = ext[3] - ext[2]
    global_tolerance = max(MIN_TOLERANCE, TOLERANCE_FACTOR * max(dx, dy))
    n = int(e_d.shape[0])
    bb = _device.empty((n, 4), torch.float64, v_d.device)
    _lib.check(lib.ct_edge_bboxes(_device.ptr(v_d), _device.ptr(e_d), n, global_tolerance, _device.ptr(bb), st),
               "edge_bboxes")
    return bb


class EdgeCellTree2d(CellTree2dBase):
    """
    Construct a cell tree from 2D vertices and an edges indexing array.

    Parameters
    ----------
    vertices: ndarray of floats with shape ``(n_point, 2)``
    edges: ndarray of integers with shape ``(n_edge, 2)``
    n_buckets: int, optional, default: 4
    cells_per_leaf: int, optional, default: 2
    """

    _elements_name = "edges"

    def __init__(self, vertices, edges, n_buckets: int = 4, cells_per_leaf: int = 2):
        _validate_params(n_buckets, cells_per_leaf)
        device = _device.require_cuda()
        torch = _device.torch()
        vertices = cast_vertices(vertices, copy=True)
        v_d = _device.to_device(vertices, torch.float64, device)
        e_d = _device.to_device(edges, torch.int64, device)
        if e_d.ndim != 2 or e_d.shape[1] != 2:
            raise ValueError("edges must have shape (n_edge, 2)")
        if e_d.shape[0] == 0:
            raise ValueError("zero-size array to reduction operation minimum which has no identity")
        validate_elements(e_d, int(v_d.shape[0]), 2, "edges")
        bb = _edge_boxes(v_d, e_d)
        self._tree = _GpuTree(device, e_d, v_d, bb, n_buckets, cells_per_leaf, candidate_lists=False)
        self._host = {}
        self._edges_in = edges
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf

    # -- serialisation (no upstream counterpart) -------------------------------
    def save(self, path) -> None:
        """Write the tree to an ``.npz`` file: vertices, edges, nodes
        (NodeDType), bb_indices and the build parameters.  ``load`` restores
        it without rebuilding."""
        edges = self.edges
        edges = edges.cpu().numpy() if is_cuda_tensor(edges) else np.asarray(edges)
        np.savez(path, format="numba_celltree_gb300.EdgeCellTree2d", version=1, vertices=self.vertices,
                 edges=edges, nodes=self.nodes, bb_indices=self.bb_indices, n_buckets=self.n_buckets,
                 cells_per_leaf=self.cells_per_leaf)

    @classmethod
    def load(cls, path) -> "EdgeCellTree2d":
        """A tree written by ``save``."""
        with np.load(path, allow_pickle=False) as z:
            if str(z["format"]) != "numba_celltree_gb300.EdgeCellTree2d":
                raise ValueError("not an EdgeCellTree2d file")
            return cls._from_arrays(z["vertices"], z["edges"], z["nodes"], z["bb_indices"], int(z["n_buckets"]),
                                    int(z["cells_per_leaf"]))

    @classmethod
    def from_celltree_data(cls, data, n_buckets: int = 4) -> "EdgeCellTree2d":
        """A tree from upstream's ``CellTreeData`` of an edge tree
        (``numba_celltree.EdgeCellTree2d(...).celltree_data``), without
        rebuilding; ``n_buckets`` only sets the returned object's attribute."""
        return cls._from_arrays(data.vertices, data.elements, data.nodes, data.bb_indices, n_buckets,
                                int(data.cells_per_leaf))

    @classmethod
    def _from_arrays(cls, vertices, edges, nodes, bb_indices, n_buckets: int, cells_per_leaf: int):
        _validate_params(n_buckets, cells_per_leaf)
        device = _device.require_cuda()
        torch = _device.torch()
        vertices = cast_vertices(vertices, copy=True)
        edges = np.ascontiguousarray(edges, dtype=np.int64)
        if edges.ndim != 2 or edges.shape[0] == 0 or edges.shape[1] != 2:
            raise ValueError("edges must have shape (n_edge >= 1, 2)")
        v_d = _device.to_device(vertices, torch.float64, device)
        e_d = _device.to_device(edges, torch.int64, device)
        validate_elements(e_d, int(v_d.shape[0]), 2, "edges")
        pre = prebuilt_from_nodes(nodes, bb_indices, int(edges.shape[0]), device)
        tree = cls.__new__(cls)
        tree._tree = _GpuTree(device, e_d, v_d, _edge_boxes(v_d, e_d), n_buckets, cells_per_leaf,
                              candidate_lists=False, prebuilt=pre)
        tree._host = {}
        tree._edges_in = edges
        tree.n_buckets = n_buckets
        tree.cells_per_leaf = cells_per_leaf
        return tree

    @property
    def edges(self):
        return self._edges_in

    def locate_points(self, points, tolerance: Optional[float] = None):
        """Index of an edge each point lies on, -1 if none (query.py:167-174)."""
        tol = self._tolerance(tolerance)
        cuda_in = is_cuda_tensor(points)
        points = cast_vertices(points)
        t = self._tree
        torch = _device.torch()
        p_d = _device.to_device(points, torch.float64, t.device)
        n = int(p_d.shape[0])
        out = _device.empty((n,), torch.int64, t.device)
        t.reset_error()
        _lib.check(
            _lib.load().ct_locate_points_on_edge(
                ctypes.byref(t.desc), _device.ptr(p_d), n, tol, _device.ptr(out), _device.stream()
            ),
            "locate_points",
        )
        t.raise_on_device_error()
        return out if cuda_in else out.cpu().numpy()

    def intersect_edges(self, edge_coords):
        """
        Find the tree edges intersected by each edge (edge_celltree.py:114-146):
        ``(edge_indices, tree_edge_indices, intersection_xy)``, each edge's
        results ordered by distance along it.
        """
        cuda_in = is_cuda_tensor(edge_coords)
        e = cast_edges(edge_coords)
        t = self._tree
        e_d = _device.to_device(e, _device.torch().float64, t.device)
        ii, jj, xy = t.locate_edges(e_d, 0)
        xy0 = xy[:, 0].contiguous()
        if cuda_in:
            return ii, jj, xy0
        return ii.cpu().numpy(), jj.cpu().numpy(), xy0.cpu().numpy()
