"""CellTree2d on the GPU -- drop-in for numba_celltree.CellTree2d
(celltree.py:37-351 upstream)."""

from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import _device, _pipeline, _lib
from .cast import cast_bboxes, cast_edges, cast_faces, cast_vertices, is_cuda_tensor
from .celltree_base import CellTree2dBase, _GpuTree, _validate_params, prebuilt_from_nodes, validate_elements


def _as_output(t, like_cuda: bool):
    return t if like_cuda else t.cpu().numpy()


class CellTree2d(CellTree2dBase):
    """
    Construct a cell tree from 2D vertices and a faces indexing array.

    Parameters
    ----------
    vertices: ndarray of floats with shape ``(n_point, 2)``
        Corner coordinates (x, y) of the cells.  A CUDA tensor is used in place.
    faces: ndarray of integers with shape ``(n_face, n_max_vert)``
        For every face the indices of its corner nodes; shorter faces are
        padded with ``fill_value``.
    fill_value: int
        Fill value marking empty nodes in ``faces``.
    n_buckets: int, optional, default: 4
        Buckets used in tree construction, 2 <= n_buckets <= 32.
    cells_per_leaf: int, optional, default: 2
        Number of cells in the leaf nodes.

    Results are identical to the upstream package: the same ``nodes`` and
    ``bb_indices`` arrays, the same cells for every query.  Queries given numpy
    arrays return numpy arrays; queries given CUDA tensors return CUDA tensors.
    ``precision`` selects the point-location form, all returning identical
    indices: ``"fp32"`` (default: queries sorted for coherence, per-grid-cell
    candidate lists and a float32 traversal with exact float32 filters, a
    float64 pass over the queries the filters could not decide),
    ``"fp32-inline"`` (one float32 kernel with in-line float64 fallbacks) or
    ``"fp64"`` (plain float64).
    """

    _elements_name = "faces"

    def __init__(self, vertices, faces, fill_value: int, n_buckets: int = 4, cells_per_leaf: int = 2):
        _validate_params(n_buckets, cells_per_leaf)
        device = _device.require_cuda()
        torch = _device.torch()
        vertices = cast_vertices(vertices, copy=True)
        faces = cast_faces(faces, fill_value)
        v_d = _device.to_device(vertices, torch.float64, device)
        f_d = _device.to_device(faces, torch.int64, device)
        if f_d.shape[1] < 3 and f_d.shape[0] > 0:
            raise ValueError("faces must have at least 3 columns")
        if f_d.shape[0] == 0:
            raise ValueError("zero-size array to reduction operation minimum which has no identity")
        validate_elements(f_d, int(v_d.shape[0]), 3, "faces")
        lib = _lib.load()
        st = _device.stream()
        n, K = int(f_d.shape[0]), int(f_d.shape[1])
        # counter_clockwise geometry_utils.py:541-561, build_face_bboxes 443-456
        _lib.check(lib.ct_counter_clockwise(_device.ptr(v_d), _device.ptr(f_d), n, K, st), "counter_clockwise")
        bb = _device.empty((n, 4), torch.float64, device)
        _lib.check(lib.ct_face_bboxes(_device.ptr(v_d), _device.ptr(f_d), n, K, _device.ptr(bb), st), "face_bboxes")
        self._tree = _GpuTree(device, f_d, v_d, bb, n_buckets, cells_per_leaf)
        self._host = {}
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self.precision = "fp32"

    # -- serialisation (no upstream counterpart) -------------------------------
    def save(self, path) -> None:
        """Write the tree to an ``.npz`` file: vertices, oriented faces, nodes
        (NodeDType), bb_indices and the build parameters.  ``load`` restores
        it without rebuilding."""
        np.savez(path, format="numba_celltree_gb300.CellTree2d", version=1, vertices=self.vertices,
                 faces=self.faces, nodes=self.nodes, bb_indices=self.bb_indices,
                 n_buckets=self.n_buckets, cells_per_leaf=self.cells_per_leaf)

    @classmethod
    def load(cls, path) -> "CellTree2d":
        """A tree written by ``save``."""
        with np.load(path, allow_pickle=False) as z:
            if str(z["format"]) != "numba_celltree_gb300.CellTree2d":
                raise ValueError("not a CellTree2d file")
            return cls._from_arrays(z["vertices"], z["faces"], z["nodes"], z["bb_indices"], int(z["n_buckets"]),
                                    int(z["cells_per_leaf"]))

    @classmethod
    def from_celltree_data(cls, data, n_buckets: int = 4) -> "CellTree2d":
        """A tree from upstream's ``CellTreeData`` (constants.py:82-89: elements,
        vertices, nodes, bb_indices, bb_coords, bbox, cells_per_leaf), e.g.
        ``numba_celltree.CellTree2d(...).celltree_data``, without rebuilding.
        ``n_buckets`` is not part of ``CellTreeData``; it only matters for
        ``n_buckets`` of the returned object."""
        return cls._from_arrays(data.vertices, data.elements, data.nodes, data.bb_indices, n_buckets,
                                int(data.cells_per_leaf))

    @classmethod
    def _from_arrays(cls, vertices, faces, nodes, bb_indices, n_buckets: int, cells_per_leaf: int):
        _validate_params(n_buckets, cells_per_leaf)
        device = _device.require_cuda()
        torch = _device.torch()
        vertices = cast_vertices(vertices, copy=True)
        faces = np.ascontiguousarray(faces, dtype=np.int64)
        if faces.ndim != 2 or faces.shape[0] == 0 or faces.shape[1] < 3:
            raise ValueError("faces must have shape (n_face >= 1, n_max_vert >= 3)")
        n = faces.shape[0]
        v_d = _device.to_device(vertices, torch.float64, device)
        f_d = _device.to_device(faces, torch.int64, device)
        validate_elements(f_d, int(v_d.shape[0]), 3, "faces")
        pre = prebuilt_from_nodes(nodes, bb_indices, n, device)
        lib = _lib.load()
        st = _device.stream()
        K = int(f_d.shape[1])
        bb = _device.empty((n, 4), torch.float64, device)
        _lib.check(lib.ct_face_bboxes(_device.ptr(v_d), _device.ptr(f_d), n, K, _device.ptr(bb), st), "face_bboxes")
        tree = cls.__new__(cls)
        tree._tree = _GpuTree(device, f_d, v_d, bb, n_buckets, cells_per_leaf, prebuilt=pre)
        tree._host = {}
        tree.n_buckets = n_buckets
        tree.cells_per_leaf = cells_per_leaf
        tree.precision = "fp32"
        return tree

    @property
    def faces(self) -> np.ndarray:
        return self._cached("faces", lambda: self._tree.elements.cpu().numpy())

    def default_tolerance(self) -> float:
        return self._tolerance(None)

    def launch_locate(self, points_dev, out_dev, tolerance: float, precision: str = "fp32") -> None:
        """Enqueue locate_points on the current stream for device-resident
        float64 points (n, 2) and an int64 output (n,); no synchronisation and
        no error-word check (for pipelines and timing loops)."""
        self._tree.locate(points_dev, out_dev, tolerance, precision)

    def locate_points(self, points, tolerance: Optional[float] = None):
        """
        Find the index of a face that contains a point (query.py:110-117).

        Points that are very close near an edge of a face will also be
        identified as falling within that face.  Returns -1 for points that
        fall in no face.
        """
        tol = self._tolerance(tolerance)
        cuda_in = is_cuda_tensor(points)
        points = cast_vertices(points)
        t = self._tree
        torch = _device.torch()
        n = int(points.shape[0])
        # first use of a batch size class: tune the launch shape (autotune.py)
        t.maybe_tune_locate(points, tol, self.precision, n if cuda_in else min(n, _pipeline.CHUNK_POINTS))
        t.reset_error()
        if not cuda_in:
            # host batch: chunked upload / query / download, result in pinned memory
            res = _pipeline.stream_points(
                points, t.device, lambda p_d, o_d, slot: t.locate(p_d, o_d, tol, self.precision, slot=slot),
                torch.int64,
            )
            t.raise_on_device_error()
            return res
        p_d = _device.to_device(points, torch.float64, t.device)
        out = _device.empty((int(p_d.shape[0]),), torch.int64, t.device)
        t.locate(p_d, out, tol, self.precision)
        t.raise_on_device_error()
        return out

    # -- launch-shape tuning (no upstream counterpart) --------------------------
    def autotune(self, points=None, boxes=None, edges=None, tolerance: Optional[float] = None,
                 index: bool = False) -> dict:
        """Time the launch shapes of this tree's kernels on sample queries and
        keep the fastest (autotune.py: per GPU and problem size class, cached
        on disk).  ``points``: point location for batches of that size (and,
        with ``index=True``, the density of the start-node grid and candidate
        lists, rebuilt for each candidate); ``boxes`` / ``edges``: the box and
        segment traversals.  Results never change, only speed.  Returns
        {kind: cache entry}."""
        from . import autotune as at

        t = self._tree
        torch = _device.torch()
        out = {}
        tol = self._tolerance(tolerance)
        if points is not None:
            p_d = _device.to_device(cast_vertices(points), torch.float64, t.device)
            n = int(p_d.shape[0])
            if index:
                o = _device.empty((n,), torch.int64, t.device)
                timed = []
                for dens in at.SPACE["index"]["grid_density"]:
                    t.rebuild_index(dens)
                    cfg = {"grid_density": dens}
                    timed.append((cfg, at.time_gpu(lambda: t.locate(p_d, o, tol, "fp32"))))
                best, ms = at.pick(timed)
                key = t.tune_key("index", 0)
                entry = {"config": best, "ms": round(ms, 4), "candidates": len(timed), "sample": n}
                at.cache().put(key, entry)
                t._tuned[key] = dict(best)
                t.rebuild_index(best["grid_density"])
                out["index"] = entry
            out["locate"] = t.tune_locate(p_d, tol, "fp32")
        if boxes is not None:
            b_d = _device.to_device(cast_bboxes(boxes), torch.float64, t.device)
            key = t.tune_key("boxes", int(b_d.shape[0]))
            t._tuned[key] = t.tune("boxes", key, lambda c: t.locate_boxes(b_d, c), int(b_d.shape[0]))
            out["boxes"] = at.cache().get(key)
        if edges is not None:
            e_d = _device.to_device(cast_edges(edges), torch.float64, t.device)
            key = t.tune_key("segments", int(e_d.shape[0]))
            t._tuned[key] = t.tune("segments", key, lambda c: t.locate_edges(e_d, 1, c), int(e_d.shape[0]))
            out["segments"] = at.cache().get(key)
        return out

    # -- box queries -----------------------------------------------------------
    # bytes a result of a multi-result query occupies on the device while it
    # is produced (pairs, temporaries of the count / write / compact passes)
    BYTES_PER_BOX_PAIR = 64
    BYTES_PER_EDGE_CANDIDATE = 160

    def _chunks(self, q_d, count, run, budget: int, cuda_out: bool, counts=None):
        """Ranges of the device queries q_d whose results fit `budget`, run one
        after another; yields each range's results (global query indices) as
        CUDA tensors or, with cuda_out False, numpy arrays (so that the device
        holds one range's results at a time).  `counts`: the per-query counts
        when already known."""
        t = self._tree
        counts = (count(q_d) if counts is None else counts).cpu().numpy()
        for s, e in t.chunk_ranges(counts, budget):
            res = run(q_d[s:e])
            res = (res[0] + s,) + tuple(res[1:])
            yield tuple(_as_output(x, cuda_out) for x in res)

    def _iter(self, q, cast, count, run, per_result: int, max_results):
        cuda_in = is_cuda_tensor(q)
        t = self._tree
        q_d = _device.to_device(cast(q), _device.torch().float64, t.device)
        budget = int(max_results) if max_results is not None else t.device_budget(per_result)
        return self._chunks(q_d, count, run, budget, cuda_in)

    @staticmethod
    def _concat(chunks):
        chunks = list(chunks)
        return tuple(np.concatenate([c[k] for c in chunks]) for k in range(len(chunks[0])))

    def iter_locate_boxes(self, bbox_coords, max_pairs: Optional[int] = None):
        """locate_boxes in ranges of boxes whose pairs stay within max_pairs
        (default: what fits the free device memory): yields
        ``(bbox_indices, tree_face_indices)`` per range, box-major; their
        concatenation is locate_boxes' result."""
        t = self._tree
        return self._iter(bbox_coords, cast_bboxes, t.count_boxes, t.locate_boxes, self.BYTES_PER_BOX_PAIR,
                          max_pairs)

    def iter_intersect_boxes(self, bbox_coords, max_pairs: Optional[int] = None):
        """intersect_boxes in ranges of boxes (see iter_locate_boxes)."""
        t = self._tree
        return self._iter(bbox_coords, cast_bboxes, t.count_boxes, self._intersect_boxes_dev,
                          self.BYTES_PER_BOX_PAIR, max_pairs)

    def iter_intersect_edges(self, edge_coords, max_candidates: Optional[int] = None):
        """intersect_edges in ranges of segments whose candidate cells (an
        upper bound of their results) stay within max_candidates (default:
        what fits the free device memory); the concatenation of the ranges'
        results is intersect_edges' result.  Segments crossing much of a big
        mesh produce billions of results: this keeps the device memory
        bounded while they stream to the host."""
        t = self._tree
        return self._iter(edge_coords, cast_edges, lambda q: t.count_edge_candidates(q, 1),
                          lambda q: t.locate_edges(q, 1), self.BYTES_PER_EDGE_CANDIDATE, max_candidates)

    def locate_boxes(self, bbox_coords):
        """
        Find the index of a face intersecting with a bounding box
        (celltree.py:130-148, query.py:177-289).

        Returns ``(bbox_indices, tree_face_indices)``, box-major, in the
        upstream order.  Host (numpy) batches whose pairs exceed the free
        device memory run in ranges of boxes (iter_locate_boxes).
        """
        cuda_in = is_cuda_tensor(bbox_coords)
        b = cast_bboxes(bbox_coords)
        t = self._tree
        b_d = _device.to_device(b, _device.torch().float64, t.device)
        budget = None if cuda_in else t.device_budget(self.BYTES_PER_BOX_PAIR)
        res = t.locate_boxes(b_d, budget=budget)
        if res is None:  # more pairs than the device holds: ranges of boxes
            return self._concat(self._chunks(b_d, None, t.locate_boxes, budget, False, counts=t.last_counts))
        ii, jj = res
        return _as_output(ii, cuda_in), _as_output(jj, cuda_in)

    def intersect_boxes(self, bbox_coords):
        """
        Boxes, intersecting faces and the area of intersection
        (celltree.py:150-184); only pairs with area > 0 are kept.  Host
        batches run in ranges when their pairs exceed the device memory.
        """
        cuda_in = is_cuda_tensor(bbox_coords)
        t = self._tree
        b_d = _device.to_device(cast_bboxes(bbox_coords), _device.torch().float64, t.device)
        budget = None if cuda_in else t.device_budget(self.BYTES_PER_BOX_PAIR)
        res = self._intersect_boxes_dev(b_d, budget)
        if res is None:  # more pairs than the device holds: ranges of boxes
            return self._concat(self._chunks(b_d, None, self._intersect_boxes_dev, budget, False,
                                             counts=t.last_counts))
        return tuple(_as_output(x, cuda_in) for x in res)

    def _intersect_boxes_dev(self, b_d, budget=None):
        t = self._tree
        torch = _device.torch()
        res = t.locate_boxes(b_d, budget=budget)
        if res is None:
            return None
        ii, jj = res
        n = int(ii.shape[0])
        area = _device.empty((n,), torch.float64, t.device)
        t.reset_error()
        order = t.pair_order(None, 4, ii, t.elements, t.K, jj)
        _lib.check(
            _lib.load().ct_box_area_of_intersection_ordered(
                _device.ptr(b_d), _device.ptr(t.vertices), _device.ptr(t.elements), t.K, _device.ptr(ii),
                _device.ptr(jj), n, _device.ptr(order), _device.ptr(area), _device.ptr(t.error_word),
                _device.stream(),
            ),
            "intersect_boxes",
        )
        del order
        t.stage_error()
        out = t.compact(ii, jj, area=area)  # synchronises (pair count)
        t.raise_on_staged_error()
        return out

    # -- face queries ----------------------------------------------------------
    def _faces_on_device(self, vertices, faces):
        torch = _device.torch()
        t = self._tree
        v_d = _device.to_device(vertices, torch.float64, t.device)
        f_d = _device.to_device(faces, torch.int64, t.device)
        if v_d.ndim != 2 or v_d.shape[1] != 2:
            raise ValueError("vertices must have shape (n_points, 2)")
        if f_d.ndim != 2:
            raise ValueError("faces must have shape (n_face, n_max_vert)")
        if f_d is faces:
            f_d = f_d.clone()
        if f_d.shape[0] > 0:
            if f_d.shape[1] < 3:
                raise ValueError("faces must have at least 3 columns")
            validate_elements(f_d, int(v_d.shape[0]), 3, "faces")
        return v_d, f_d

    def _locate_faces_dev(self, v_d, f_d):
        torch = _device.torch()
        t = self._tree
        lib = _lib.load()
        st = _device.stream()
        n, K = int(f_d.shape[0]), int(f_d.shape[1])
        # counter_clockwise + build_face_bboxes of the query faces (celltree.py:212-213)
        _lib.check(lib.ct_counter_clockwise(_device.ptr(v_d), _device.ptr(f_d), n, K, st), "counter_clockwise")
        bb = _device.empty((n, 4), torch.float64, t.device)
        _lib.check(lib.ct_face_bboxes(_device.ptr(v_d), _device.ptr(f_d), n, K, _device.ptr(bb), st), "face_bboxes")
        si, sj = t.locate_boxes(bb)
        m = int(si.shape[0])
        flag = _device.empty((m,), torch.uint8, t.device)
        _lib.check(
            lib.ct_polygons_intersect(
                _device.ptr(v_d), _device.ptr(f_d), K, _device.ptr(t.vertices), _device.ptr(t.elements), t.K,
                _device.ptr(si), _device.ptr(sj), m, _device.ptr(flag), st,
            ),
            "polygons_intersect",
        )
        return t.compact(si, sj, flag=flag)

    def locate_faces(self, vertices, faces):
        """
        Find the index of a face intersecting with another face
        (celltree.py:186-226).  Like upstream, a numpy ``faces`` argument is
        reoriented counter-clockwise in place.
        """
        cuda_in = is_cuda_tensor(faces)
        v_d, f_d = self._faces_on_device(vertices, faces)
        if f_d.shape[0] == 0:
            e = _device.empty((0,), _device.torch().int64, self._tree.device)
            return _as_output(e, cuda_in), _as_output(e, cuda_in)
        i, j = self._locate_faces_dev(v_d, f_d)
        if isinstance(faces, np.ndarray):
            faces[...] = f_d.cpu().numpy().astype(faces.dtype, copy=False)
        elif cuda_in:
            faces.copy_(f_d.to(faces.dtype))
        return _as_output(i, cuda_in), _as_output(j, cuda_in)

    def intersect_faces(self, vertices, faces, fill_value: int):
        """
        Faces of another mesh, intersecting tree faces and the area of
        intersection (celltree.py:228-269); only pairs with area > 0 are kept.
        """
        cuda_in = is_cuda_tensor(faces)
        vertices = cast_vertices(vertices)
        faces = cast_faces(faces, fill_value)
        v_d, f_d = self._faces_on_device(vertices, faces)
        t = self._tree
        torch = _device.torch()
        if f_d.shape[0] == 0:
            e = _device.empty((0,), torch.int64, t.device)
            return _as_output(e, cuda_in), _as_output(e, cuda_in), _as_output(e.double(), cuda_in)
        i, j = self._locate_faces_dev(v_d, f_d)
        n = int(i.shape[0])
        area = _device.empty((n,), torch.float64, t.device)
        t.reset_error()
        order = t.pair_order(f_d, int(f_d.shape[1]), i, t.elements, t.K, j)
        _lib.check(
            _lib.load().ct_area_of_intersection_ordered(
                _device.ptr(v_d), _device.ptr(f_d), int(f_d.shape[1]), _device.ptr(t.vertices),
                _device.ptr(t.elements), t.K, _device.ptr(i), _device.ptr(j), n, _device.ptr(order),
                _device.ptr(area), _device.ptr(t.error_word), _device.stream(),
            ),
            "area_of_intersection",
        )
        del order
        t.stage_error()
        i2, j2, a2 = t.compact(i, j, area=area)  # synchronises (pair count)
        t.raise_on_staged_error()
        return _as_output(i2, cuda_in), _as_output(j2, cuda_in), _as_output(a2, cuda_in)

    # -- segments --------------------------------------------------------------
    def intersect_edges(self, edge_coords):
        """
        Find the faces intersected by each edge and the clipped edge
        (celltree.py:271-304); results of each edge are ordered by distance
        along it.  Returns ``(edge_indices, tree_face_indices, xy)`` with xy of
        shape ``(n_found, 2, 2)``.
        """
        cuda_in = is_cuda_tensor(edge_coords)
        e = cast_edges(edge_coords)
        t = self._tree
        e_d = _device.to_device(e, _device.torch().float64, t.device)
        budget = None if cuda_in else t.device_budget(self.BYTES_PER_EDGE_CANDIDATE)
        res = t.locate_edges(e_d, 1, budget=budget)
        if res is None:  # more candidates than the device holds: ranges of segments
            return self._concat(self._chunks(e_d, None, lambda q: t.locate_edges(q, 1), budget, False,
                                             counts=t.last_counts))
        ii, jj, xy = res
        return _as_output(ii, cuda_in), _as_output(jj, cuda_in), _as_output(xy, cuda_in)

    # -- barycentric -----------------------------------------------------------
    def compute_barycentric_weights(self, points, tolerance: Optional[float] = None):
        """
        Locate points and compute barycentric weights of their face's vertices
        (celltree.py:306-351): triangle weights when faces have at most 3
        vertices, else Wachspress weights.  Rows of points not found are zero.
        """
        tol = self._tolerance(tolerance)
        cuda_in = is_cuda_tensor(points)
        points = cast_vertices(points)
        t = self._tree
        torch = _device.torch()
        p_d = _device.to_device(points, torch.float64, t.device)
        n = int(p_d.shape[0])
        idx = _device.empty((n,), torch.int64, t.device)
        t.reset_error()
        self.launch_locate(p_d, idx, tol, self.precision)
        K = t.K
        w = _device.empty((n, K if K > 3 else 3), torch.float64, t.device)
        _lib.check(
            _lib.load().ct_barycentric_weights(
                ctypes.byref(t.desc), _device.ptr(p_d), _device.ptr(idx), n, tol, _device.ptr(w), _device.stream()
            ),
            "barycentric",
        )
        t.raise_on_device_error()
        return _as_output(idx, cuda_in), _as_output(w, cuda_in)
