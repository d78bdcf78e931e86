"""A batch of face trees built together and queried together (no upstream
counterpart; upstream builds and queries one ``CellTree2d`` at a time).

``CellTreeBatch(meshes)`` builds every mesh's tree in one forest build
(``ct_build_forest``: all roots start the level-synchronous builder together,
so the batch costs one host synchronisation per tree level instead of one per
level per mesh) and exposes each mesh as an ordinary ``CellTree2d`` with the
upstream ``nodes`` / ``bb_indices`` (bit-identical to building it alone).

``locate_points`` runs the points of all meshes through one batched pipeline
(``ct_forest_locate``: queries sorted by (mesh, Morton key), the tree looked up
per query).  ``plan_locate`` + ``LocatePlan.launch`` split it into a one-time
upload and a launch-only part that can be captured in a CUDA graph.
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np

from . import _device, _lib
from .cast import cast_faces, cast_vertices, is_cuda_tensor
from .celltree import CellTree2d
from .celltree_base import _GpuTree, _validate_params, validate_elements


class LocatePlan:
    """Point counts per mesh and tolerances, uploaded once; ``launch`` only
    enqueues kernels (graph-capturable)."""

    def __init__(self, batch: "CellTreeBatch", counts: Sequence[int], tolerances: Sequence[float]):
        torch = _device.torch()
        lib = _lib.load()
        trees = batch.trees
        n_trees = len(trees)
        if len(counts) != n_trees or len(tolerances) != n_trees:
            raise ValueError("one point count and one tolerance per mesh")
        off = np.zeros(n_trees + 1, dtype=np.int64)
        off[1:] = np.cumsum(np.asarray(counts, dtype=np.int64))
        self.offsets = off
        self.n_points = int(off[-1])
        self.tolerances = np.asarray(tolerances, dtype=np.float64)
        descs = (_lib.CtTree * n_trees)()
        for i, t in enumerate(trees):
            descs[i] = t._tree.desc
        self._descs = descs
        nbytes = int(lib.ct_forest_locate_workspace_size(self.n_points, n_trees))
        self.workspace = _device.empty((max(nbytes, 1),), torch.uint8, batch.device)
        self.plan = _lib.CtForestPlan()
        off_c = (ctypes.c_int64 * (n_trees + 1))(*off.tolist())
        tol_c = (ctypes.c_double * n_trees)(*self.tolerances.tolist())
        _lib.check(
            lib.ct_forest_locate_prepare(
                ctypes.cast(descs, ctypes.c_void_p), n_trees, tol_c, off_c, self.n_points, ctypes.byref(self.plan),
                _device.ptr(self.workspace), int(self.workspace.numel()), _device.stream(),
            ),
            "forest locate prepare",
        )
        self.batch = batch

    def launch(self, points_d, out_d) -> None:
        """Enqueue the batched locate of ``points_d`` (n_points x 2 float64,
        mesh i's points at rows offsets[i]:offsets[i+1]) into ``out_d``
        (n_points int64) on the current stream: kernels only."""
        _lib.check(
            _lib.load().ct_forest_locate(
                ctypes.byref(self.plan), _device.ptr(points_d), _device.ptr(out_d), _device.ptr(self.workspace),
                int(self.workspace.numel()), _device.stream(),
            ),
            "forest locate",
        )


class CellTreeBatch:
    """
    Build the cell trees of several meshes at once.

    Parameters
    ----------
    meshes: sequence of ``(vertices, faces)`` pairs (numpy arrays or CUDA
        tensors), each as for ``CellTree2d``.
    fill_value, n_buckets, cells_per_leaf: as for ``CellTree2d``, shared by
        all meshes.

    ``batch[i]`` is mesh i's ``CellTree2d``.
    """

    def __init__(self, meshes: Sequence, fill_value: int = -1, n_buckets: int = 4, cells_per_leaf: int = 2):
        _validate_params(n_buckets, cells_per_leaf)
        if len(meshes) == 0:
            raise ValueError("need at least one mesh")
        device = _device.require_cuda()
        self.device = device
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        prepared = []
        for vertices, faces in meshes:
            v = cast_vertices(vertices, copy=True)
            f = cast_faces(faces, fill_value)
            v_d = _device.to_device(v, torch.float64, device)
            f_d = _device.to_device(f, torch.int64, device)
            if f_d is faces:
                f_d = f_d.clone()
            if f_d.shape[0] == 0:
                raise ValueError("every mesh needs at least one face")
            if f_d.shape[1] < 3:
                raise ValueError("faces must have at least 3 columns")
            validate_elements(f_d, int(v_d.shape[0]), 3, "faces")
            prepared.append((v_d, f_d))
        sizes = np.array([int(f.shape[0]) for _, f in prepared], dtype=np.int64)
        tree_off = np.zeros(len(prepared) + 1, dtype=np.int64)
        tree_off[1:] = np.cumsum(sizes)
        n_total = int(tree_off[-1])
        bb_all = _device.empty((n_total, 4), torch.float64, device)
        for (v_d, f_d), a in zip(prepared, tree_off[:-1]):
            n, K = int(f_d.shape[0]), int(f_d.shape[1])
            # counter_clockwise geometry_utils.py:541-561, build_face_bboxes 443-456
            _lib.check(lib.ct_counter_clockwise(_device.ptr(v_d), _device.ptr(f_d), n, K, st), "counter_clockwise")
            _lib.check(lib.ct_face_bboxes(_device.ptr(v_d), _device.ptr(f_d), n, K, _device.ptr(bb_all[a:a + n]),
                                          st), "face_bboxes")
        n_trees = len(prepared)
        off_c = (ctypes.c_int64 * (n_trees + 1))(*tree_off.tolist())
        n_nodes = (ctypes.c_int64 * n_trees)()
        depth = (ctypes.c_int32 * n_trees)()
        factor = 1
        while True:
            wsz = int(lib.ct_build_forest_workspace_size(n_total, n_trees, n_buckets, factor))
            ws = _device.empty((max(wsz, 1),), torch.uint8, device)
            status = lib.ct_build_forest(_device.ptr(bb_all), n_total, off_c, n_trees, n_buckets, cells_per_leaf,
                                         factor, _device.ptr(ws), wsz, n_nodes, depth, st)
            if status == _lib.CT_ERR_WORKSPACE and factor < 4096:
                factor *= 8
                del ws
                continue
            _lib.check(status, "forest build")
            break
        nn = np.array(n_nodes[:], dtype=np.int64)
        node_off = np.zeros(n_trees + 1, dtype=np.int64)
        node_off[1:] = np.cumsum(nn)
        total = int(node_off[-1])
        child = _device.empty((total,), torch.int64, device)
        Lmax = _device.empty((total,), torch.float64, device)
        Rmin = _device.empty((total,), torch.float64, device)
        ptr = _device.empty((total,), torch.int64, device)
        size = _device.empty((total,), torch.int64, device)
        dim = _device.empty((total,), torch.uint8, device)
        bbi = _device.empty((n_total,), torch.int64, device)
        node_off_d = torch.as_tensor(node_off, device=device)
        _lib.check(
            lib.ct_build_forest_emit(
                _device.ptr(ws), n_total, n_trees, n_buckets, factor, _device.ptr(node_off_d),
                _device.ptr(child), _device.ptr(Lmax), _device.ptr(Rmin), _device.ptr(ptr), _device.ptr(size),
                _device.ptr(dim), _device.ptr(bbi), st,
            ),
            "forest emit",
        )
        del ws
        self.trees: List[CellTree2d] = []
        for i, (v_d, f_d) in enumerate(prepared):
            a, b = int(node_off[i]), int(node_off[i + 1])
            e0, e1 = int(tree_off[i]), int(tree_off[i + 1])
            pre = (child[a:b], Lmax[a:b], Rmin[a:b], ptr[a:b], size[a:b], dim[a:b], bbi[e0:e1], int(depth[i]))
            tree = CellTree2d.__new__(CellTree2d)
            tree._tree = _GpuTree(device, f_d, v_d, bb_all[e0:e1], n_buckets, cells_per_leaf, prebuilt=pre)
            tree._host = {}
            tree.n_buckets = n_buckets
            tree.cells_per_leaf = cells_per_leaf
            tree.precision = "fp32"
            self.trees.append(tree)
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self._plan = None

    def __len__(self) -> int:
        return len(self.trees)

    def __getitem__(self, i) -> CellTree2d:
        return self.trees[i]

    def plan_locate(self, counts: Sequence[int], tolerance: Optional[float] = None) -> LocatePlan:
        """Upload the batch's tree records for ``counts[i]`` points of mesh i
        (tolerance: one value for all meshes, default each mesh's own)."""
        tols = [t._tolerance(tolerance) for t in self.trees]
        return LocatePlan(self, [int(c) for c in counts], tols)

    def locate_points(self, points: Sequence, tolerance: Optional[float] = None) -> list:
        """``locate_points`` (query.py:110-117) of ``points[i]`` in mesh i, all
        meshes in one batched pipeline; returns one index array per mesh
        (CUDA tensors for CUDA inputs, numpy arrays otherwise)."""
        torch = _device.torch()
        if len(points) != len(self.trees):
            raise ValueError("one point array per mesh")
        cuda_in = [is_cuda_tensor(p) for p in points]
        parts = [cast_vertices(p) for p in points]
        counts = [int(p.shape[0]) for p in parts]
        key = (tuple(counts), tolerance)
        if self._plan is None or self._plan[0] != key:
            self._plan = (key, self.plan_locate(counts, tolerance))
        plan = self._plan[1]
        pts_d = torch.cat([_device.to_device(p, torch.float64, self.device) for p in parts]) if parts else None
        out = _device.empty((plan.n_points,), torch.int64, self.device)
        for t in self.trees:
            t._tree.reset_error()
        plan.launch(pts_d, out)
        for t in self.trees:
            t._tree.raise_on_device_error()
        res = []
        for i, c in enumerate(cuda_in):
            o = out[int(plan.offsets[i]):int(plan.offsets[i + 1])]
            res.append(o if c else o.cpu().numpy())
        return res
