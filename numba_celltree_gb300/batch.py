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


class ForestBuild:
    """The tree build of a batch of meshes of fixed cell counts, enqueued with
    no host synchronisation (``ct_build_forest_async``: every tree level runs
    on the device), so ``launch`` can be captured in a CUDA graph and replayed
    when the meshes' coordinates change.  Node arrays are sized for the
    pessimistic node count of every tree; ``node_off`` / ``n_nodes`` /
    ``max_depth`` / ``status`` stay on the device until ``result`` reads them."""

    def __init__(self, cell_counts: Sequence[int], device, n_buckets: int = 4, cells_per_leaf: int = 2,
                 capacity_factor: int = 1):
        torch = _device.torch()
        lib = _lib.load()
        counts = np.asarray(cell_counts, dtype=np.int64)
        if counts.size == 0 or np.any(counts < 1):
            raise ValueError("every mesh needs at least one face")
        self.n_trees = int(counts.size)
        self.tree_off = np.zeros(self.n_trees + 1, dtype=np.int64)
        self.tree_off[1:] = np.cumsum(counts)
        self.n_total = int(self.tree_off[-1])
        self.n_buckets, self.cells_per_leaf, self.factor = n_buckets, cells_per_leaf, capacity_factor
        self.device = device
        self.capacity = int(sum(int(lib.ct_pessimistic_n_nodes(int(c))) for c in counts))
        wsz = int(lib.ct_build_forest_workspace_size(self.n_total, self.n_trees, n_buckets, capacity_factor))
        self.workspace = _device.empty((max(wsz, 1),), torch.uint8, device)
        E = lambda n, dt: _device.empty((n,), dt, device)
        cap = self.capacity
        self.child, self.Lmax, self.Rmin = E(cap, torch.int64), E(cap, torch.float64), E(cap, torch.float64)
        self.ptr, self.size, self.dim = E(cap, torch.int64), E(cap, torch.int64), E(cap, torch.uint8)
        self.bb_indices = E(self.n_total, torch.int64)
        self.n_nodes = E(self.n_trees, torch.int64)
        self.node_off = E(self.n_trees + 1, torch.int64)
        self.max_depth = E(self.n_trees, torch.int32)
        self.status = torch.zeros((1,), dtype=torch.int32, device=device)
        self.tree_off_d = torch.as_tensor(self.tree_off, device=device)
        self._off_c = (ctypes.c_int64 * (self.n_trees + 1))(*self.tree_off.tolist())

    def launch(self, bb_all) -> None:
        """Enqueue the build of all trees from ``bb_all`` (n_total x 4 boxes,
        tree i at rows tree_off[i]:tree_off[i+1]) on the current stream."""
        P = _device.ptr
        _lib.check(
            _lib.load().ct_build_forest_async(
                P(bb_all), self.n_total, self._off_c, P(self.tree_off_d), self.n_trees, self.n_buckets,
                self.cells_per_leaf, self.factor, P(self.workspace), int(self.workspace.numel()), self.capacity,
                P(self.child), P(self.Lmax), P(self.Rmin), P(self.ptr), P(self.size), P(self.dim),
                P(self.bb_indices), P(self.n_nodes), P(self.node_off), P(self.max_depth), P(self.status),
                _device.stream(),
            ),
            "forest build",
        )

    def result(self):
        """(node_off, max_depth) on the host after the enqueued build, or
        raise if the device reported a problem."""
        st = int(self.status.item())
        if st:
            raise _lib.CellTreeError(f"device-driven forest build reported status {st:#x}")
        return self.node_off.cpu().numpy(), self.max_depth.cpu().numpy()


def k_runs(Ks: Sequence[int], tree_off, face_off) -> list:
    """Runs of consecutive meshes with the same number of columns K, one
    launch each for the face orientation and boxes: (first face row, rows,
    K, first int64 of the run's faces)."""
    runs = []
    i, n = 0, len(Ks)
    while i < n:
        j = i
        while j + 1 < n and Ks[j + 1] == Ks[i]:
            j += 1
        runs.append((int(tree_off[i]), int(tree_off[j + 1] - tree_off[i]), int(Ks[i]), int(face_off[i])))
        i = j + 1
    return runs


class ForestPipeline:
    """Build and point location of a batch of meshes with fixed topology, as
    one sequence of launches with no host synchronisation: per replay the
    faces are reoriented and boxed (``ct_counter_clockwise``,
    ``ct_face_bboxes``), every tree is built (``ct_build_forest_async``),
    indexed (``ct_forest_index_build``: bbox, tolerance, float32 frame,
    packed nodes and cells, start-node grid) and queried
    (``ct_forest_locate``).  ``capture`` records the sequence in a CUDA graph;
    ``run`` writes new vertices and points into the pipeline's buffers,
    replays it and returns the cell index of every point.

    meshes: ``(vertices, faces)`` pairs as for ``CellTree2d`` (the faces fix
    the topology; the vertex coordinates may change between runs).
    point_counts: points per mesh (fixed).  tolerance: one value for all
    meshes, default each mesh's own (default_tolerance of each build).
    Results equal ``CellTree2d(vertices_i, faces_i).locate_points(points_i)``.

    The traversal stack is sized from the first build's deepest tree plus
    ``stack_headroom`` levels (at most 126 levels); a replay whose trees grow
    deeper than that, or whose build overflows the node capacity, raises in
    ``check``.  Each build also gets candidate lists (for each mesh's query
    tolerance) of up to ``candidate_entries_per_cell`` entries per cell in
    total; a build with more entries locates without them (same results).
    """

    def __init__(self, meshes: Sequence, point_counts: Sequence[int], fill_value: int = -1, n_buckets: int = 4,
                 cells_per_leaf: int = 2, tolerance: Optional[float] = None, stack_headroom: int = 8,
                 grid_density: float = 1.0, candidate_entries_per_cell: float = 8.0):
        _validate_params(n_buckets, cells_per_leaf)
        if len(meshes) == 0:
            raise ValueError("need at least one mesh")
        if len(point_counts) != len(meshes):
            raise ValueError("one point count per mesh")
        torch = _device.torch()
        lib = _lib.load()
        device = _device.require_cuda()
        self.device = device
        st = _device.stream()
        n_trees = len(meshes)
        verts, faces, Ks, sizes, nverts = [], [], [], [], []
        for vertices, f in meshes:
            v = cast_vertices(vertices)
            fa = cast_faces(f, fill_value)
            v_h = v.cpu().numpy() if is_cuda_tensor(v) else v
            f_h = fa.cpu().numpy() if is_cuda_tensor(fa) else fa
            if f_h.shape[0] == 0:
                raise ValueError("every mesh needs at least one face")
            if f_h.shape[1] < 3:
                raise ValueError("faces must have at least 3 columns")
            validate_elements(_device.to_device(f_h, torch.int64, device), int(v_h.shape[0]), 3, "faces")
            verts.append(v_h)
            faces.append(f_h)
            Ks.append(int(f_h.shape[1]))
            sizes.append(int(f_h.shape[0]))
            nverts.append(int(v_h.shape[0]))
        self.n_trees = n_trees
        self.vert_off = np.zeros(n_trees + 1, dtype=np.int64)
        self.vert_off[1:] = np.cumsum(nverts)
        sizes_a = np.asarray(sizes, dtype=np.int64)
        Ks_a = np.asarray(Ks, dtype=np.int64)
        self.tree_off = np.zeros(n_trees + 1, dtype=np.int64)
        self.tree_off[1:] = np.cumsum(sizes_a)
        face_off = np.zeros(n_trees + 1, dtype=np.int64)
        face_off[1:] = np.cumsum(sizes_a * Ks_a)
        s4 = np.asarray([int(lib.ct_poly32_stride(k)) for k in Ks], dtype=np.int64)
        poly32_off = np.zeros(n_trees + 1, dtype=np.int64)
        poly32_off[1:] = np.cumsum(sizes_a * s4)
        flat = np.concatenate([np.where(f >= 0, f + self.vert_off[i], -1).ravel() for i, f in enumerate(faces)])
        self.faces = torch.as_tensor(flat, dtype=torch.int64, device=device)
        self.vertices = torch.as_tensor(np.concatenate(verts), dtype=torch.float64, device=device)
        self._runs = k_runs(Ks, self.tree_off, face_off)
        n_total = int(self.tree_off[-1])
        self.bb = _device.empty((n_total, 4), torch.float64, device)
        # start-node grid shapes from the first geometry's bboxes
        gnx, gny = np.zeros(n_trees, dtype=np.int32), np.zeros(n_trees, dtype=np.int32)
        for i, (v_h, f_h) in enumerate(zip(verts, faces)):
            used = v_h[f_h[f_h >= 0]]
            w, h = float(used[:, 0].max() - used[:, 0].min()), float(used[:, 1].max() - used[:, 1].min())
            a, b = ctypes.c_int32(0), ctypes.c_int32(0)
            _lib.check(lib.ct_grid_shape(sizes[i], w, h, float(grid_density), ctypes.byref(a), ctypes.byref(b)),
                       "grid shape")
            gnx[i], gny[i] = a.value, b.value
        grid_off = np.zeros(n_trees + 1, dtype=np.int64)
        grid_off[1:] = np.cumsum(gnx.astype(np.int64) * gny.astype(np.int64))
        # the build; the first one runs now and sizes the traversal stack
        factor = 1
        while True:
            self.build = ForestBuild(sizes, device, n_buckets, cells_per_leaf, factor)
            self._enqueue_build()
            status = int(self.build.status.item())
            if status & _lib.DEVERR_CAPACITY and factor < 4096:
                factor *= 8
                continue
            break
        _, depth = self.build.result()
        self.stack = min(128, int(depth.max()) + 2 + int(stack_headroom))
        if int(depth.max()) + 2 > 128:
            raise _lib.CellTreeError("a tree deeper than 126 levels: use CellTree2d for this mesh")
        T = lambda a: torch.as_tensor(a, device=device)
        self._keep = dict(face_off=T(face_off[:-1].copy()), poly32_off=T(poly32_off[:-1].copy()),
                          tree_K=T(Ks_a.astype(np.int32)), grid_off=T(grid_off), grid_nx=T(gnx), grid_ny=T(gny))
        cap = self.build.capacity
        E = lambda n, dt: _device.empty((max(int(n), 1),), dt, device)
        self.grid_start = E(grid_off[-1], torch.int32)
        self.nodes_f32 = E(4 * cap, torch.float32)
        self.nodes_f64 = E(2 * cap, torch.float64)
        self.poly_f64 = E(2 * face_off[-1], torch.float64)
        self.poly_f32 = E(4 * poly32_off[-1], torch.float32)
        self.poly_len = E(n_total, torch.uint8)
        self.poly_len32 = E(n_total, torch.uint8)
        self.summary = E(16 * n_trees, torch.int64)
        grid_cells = int(grid_off[-1])
        self.cand_capacity = int(candidate_entries_per_cell * n_total) if grid_cells > 0 else 0
        self.cand_count = E(grid_cells + 1, torch.int64)
        self.cand_off = E(grid_cells + 1, torch.int64)
        self.cand_box = E(4 * n_total, torch.float32)
        self.cand_idx = E(self.cand_capacity, torch.int32)
        self.cand_lbox = E(4 * self.cand_capacity, torch.float32)
        scan_bytes = int(lib.ct_scan_workspace_size(grid_cells + 1))
        self.cand_scan = E(scan_bytes, torch.uint8)
        self.error_word = torch.zeros((1,), dtype=torch.int32, device=device)
        P = _device.ptr
        fb = self.build
        X = _lib.CtForestIndex()
        X.vertices, X.faces, X.bb_coords = P(self.vertices), P(self.faces), P(self.bb)
        X.face_off, X.poly32_off, X.tree_K = P(self._keep["face_off"]), P(self._keep["poly32_off"]), P(self._keep["tree_K"])
        X.tree_off, X.node_off, X.max_depth = P(fb.tree_off_d), P(fb.node_off), P(fb.max_depth)
        X.node_child, X.node_Lmax, X.node_Rmin = P(fb.child), P(fb.Lmax), P(fb.Rmin)
        X.node_ptr, X.node_size, X.node_dim, X.bb_indices = P(fb.ptr), P(fb.size), P(fb.dim), P(fb.bb_indices)
        X.grid_start, X.grid_off = P(self.grid_start), P(self._keep["grid_off"])
        X.grid_nx, X.grid_ny = P(self._keep["grid_nx"]), P(self._keep["grid_ny"])
        X.n_total, X.node_capacity, X.grid_cells = n_total, cap, int(grid_off[-1])
        X.n_trees, X.k_max, X.stack = n_trees, int(Ks_a.max()), self.stack
        X.tolerance = float(tolerance) if tolerance is not None else 0.0
        X.nodes_f32, X.nodes_f64, X.poly_f64, X.poly_f32 = (P(self.nodes_f32), P(self.nodes_f64), P(self.poly_f64),
                                                            P(self.poly_f32))
        X.poly_len, X.poly_len32, X.summary, X.error_word = (P(self.poly_len), P(self.poly_len32), P(self.summary),
                                                             P(self.error_word))
        X.cand_count, X.cand_off, X.cand_box = P(self.cand_count), P(self.cand_off), P(self.cand_box)
        X.cand_idx, X.cand_lbox, X.cand_scan_ws = P(self.cand_idx), P(self.cand_lbox), P(self.cand_scan)
        X.cand_scan_bytes, X.cand_capacity = scan_bytes, self.cand_capacity
        if tolerance is not None and not float(tolerance) > 0.0:
            raise ValueError("tolerance must be > 0")
        self.index = X
        counts = np.asarray([int(c) for c in point_counts], dtype=np.int64)
        if np.any(counts < 0):
            raise ValueError("point counts must be >= 0")
        self.offsets = np.zeros(n_trees + 1, dtype=np.int64)
        self.offsets[1:] = np.cumsum(counts)
        self.n_points = int(self.offsets[-1])
        nbytes = int(lib.ct_forest_locate_workspace_size(self.n_points, n_trees))
        self.workspace = _device.empty((max(nbytes, 1),), torch.uint8, device)
        self.plan = _lib.CtForestPlan()
        off_c = (ctypes.c_int64 * (n_trees + 1))(*self.offsets.tolist())
        _lib.check(lib.ct_forest_index_prepare(ctypes.byref(X), off_c, self.n_points, ctypes.byref(self.plan),
                                               P(self.workspace), int(self.workspace.numel()), st),
                   "forest index prepare")
        self.points = torch.zeros((max(self.n_points, 1), 2), dtype=torch.float64, device=device)
        self.out = _device.empty((max(self.n_points, 1),), torch.int64, device)
        self.graph = None

    def _enqueue_build(self) -> None:
        lib = _lib.load()
        st = _device.stream()
        P = _device.ptr
        v, f, bb = P(self.vertices), P(self.faces), P(self.bb)
        for r0, n, K, e0 in self._runs:
            # counter_clockwise geometry_utils.py:541-561, build_face_bboxes 443-456
            _lib.check(lib.ct_counter_clockwise(v, f + 8 * e0, n, K, st), "counter_clockwise")
            _lib.check(lib.ct_face_bboxes(v, f + 8 * e0, n, K, bb + 32 * r0, st), "face_bboxes")
        self.build.launch(self.bb)

    def launch(self) -> None:
        """Enqueue one build + index + locate of the current ``vertices`` and
        ``points`` buffers on the current stream (kernels and memsets only)."""
        lib = _lib.load()
        st = _device.stream()
        P = _device.ptr
        self._enqueue_build()
        nbytes = int(self.workspace.numel())
        _lib.check(lib.ct_forest_index_build(ctypes.byref(self.index), ctypes.byref(self.plan), P(self.workspace),
                                             nbytes, st), "forest index")
        _lib.check(lib.ct_forest_locate(ctypes.byref(self.plan), P(self.points), P(self.out), P(self.workspace),
                                        nbytes, st), "forest locate")

    def capture(self):
        """Record ``launch`` in a CUDA graph (after one warm-up launch)."""
        torch = _device.torch()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.launch()
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g
        return g

    def check(self) -> None:
        """Raise if the last build or index reported a problem (reads two
        device words)."""
        st = int(self.build.status.item())
        if st:
            raise _lib.CellTreeError("forest build: " + _lib.device_error_text(st))
        err = int(self.error_word.item())
        if err:
            raise _lib.CellTreeError("forest index: " + _lib.device_error_text(err))

    def run(self, vertices=None, points=None):
        """Copy new vertex coordinates (all meshes, rows ``vert_off[i]`` ..
        for mesh i) and points (rows ``offsets[i]`` .. for mesh i) into the
        buffers, replay the graph (or launch when none is captured), check
        and return the results (a view of ``out``)."""
        torch = _device.torch()
        if vertices is not None:
            self.vertices.copy_(torch.as_tensor(vertices, dtype=torch.float64).reshape(self.vertices.shape))
        if points is not None and self.n_points:
            self.points[:self.n_points].copy_(torch.as_tensor(points, dtype=torch.float64).reshape(self.n_points, 2))
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        self.check()
        return self.out[:self.n_points]

    def candidate_entries(self) -> int:
        """Entries of the last build's candidate lists (above cand_capacity
        the lists were off for that build)."""
        return int(self.cand_off[-1].item()) if self.cand_capacity else 0

    def result(self, i: int):
        """Cell indices of mesh i's points after the last run."""
        return self.out[int(self.offsets[i]):int(self.offsets[i + 1])]


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

    def __init__(self, meshes: Sequence, fill_value: int = -1, n_buckets: int = 4, cells_per_leaf: int = 2,
                 device_levels: bool = True):
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
        self.forest = None
        if device_levels:
            # every level on the device; one synchronisation at the end
            fb = ForestBuild(sizes, device, n_buckets, cells_per_leaf)
            fb.launch(bb_all)
            if int(fb.status.item()) == 0:
                self.forest = fb
        if self.forest is not None:
            fb = self.forest
            node_off, depth_h = fb.result()
            self.trees: List[CellTree2d] = []
            for i, (v_d, f_d) in enumerate(prepared):
                a, b = int(node_off[i]), int(node_off[i + 1])
                e0, e1 = int(tree_off[i]), int(tree_off[i + 1])
                pre = (fb.child[a:b], fb.Lmax[a:b], fb.Rmin[a:b], fb.ptr[a:b], fb.size[a:b], fb.dim[a:b],
                       fb.bb_indices[e0:e1], int(depth_h[i]))
                self.trees.append(self._tree_of(device, f_d, v_d, bb_all[e0:e1], n_buckets, cells_per_leaf, pre))
            self.n_buckets = n_buckets
            self.cells_per_leaf = cells_per_leaf
            self._plan = None
            return
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
            self.trees.append(self._tree_of(device, f_d, v_d, bb_all[e0:e1], n_buckets, cells_per_leaf, pre))
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self._plan = None

    @staticmethod
    def _tree_of(device, f_d, v_d, bb, n_buckets, cells_per_leaf, pre) -> CellTree2d:
        tree = CellTree2d.__new__(CellTree2d)
        tree._tree = _GpuTree(device, f_d, v_d, bb, n_buckets, cells_per_leaf, prebuilt=pre)
        tree._host = {}
        tree.n_buckets = n_buckets
        tree.cells_per_leaf = cells_per_leaf
        tree.precision = "fp32"
        return tree

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
