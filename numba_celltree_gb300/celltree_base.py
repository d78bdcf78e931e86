"""Shared machinery of the GPU cell trees (celltree_base.py:1-114 upstream).

A tree lives on the GPU: the reference-layout arrays (faces/edges, vertices,
nodes as NodeDType fields, bb_indices, bb_coords) plus the packed traversal
arrays of ``ct_tree``.  The public numpy attributes of the upstream classes
(``vertices``, ``faces``, ``nodes``, ``bb_indices``, ``bb_coords``,
``bb_distances``, ``celltree_data``) are host copies made on first access.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _device
from . import _lib
from . import autotune
from .constants import MAX_N_BUCKETS, MIN_TOLERANCE, TOLERANCE_FACTOR, CellTreeData, NodeDType


def default_tolerance(max_bb_diagonal: float) -> float:
    """default_tolerance celltree_base.py:51-52 (given the maximum diagonal)."""
    return max(MIN_TOLERANCE, TOLERANCE_FACTOR * max_bb_diagonal)


class _GpuTree:
    """Device arrays of one tree and the ``ct_tree`` descriptor over them."""

    # query tolerances up to this multiple of the default one use the
    # candidate lists (widening 2 * 1e-6 of the largest cell diagonal)
    CAND_TOL_FACTOR = 1.0e6
    # grid cells (start-node grid and candidate lists) per mesh cell
    GRID_CELLS_PER_ELEMENT = 1.0

    def __init__(self, device, elements, vertices, bb_coords, n_buckets: int, cells_per_leaf: int,
                 candidate_lists: bool = True, prebuilt=None):
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        self.device = device
        self.elements = elements
        self.vertices = vertices
        self.bb_coords = bb_coords
        n = int(elements.shape[0])
        K = int(elements.shape[1])
        self.n = n
        self.K = K
        # bbox_tree / bbox_distances / default tolerance (celltree_base.py:20-52)
        self.bb_distances = _device.empty((n, 3), torch.float64, device)
        summ = (ctypes.c_double * 5)()
        _lib.check(lib.ct_bbox_summary(_device.ptr(bb_coords), n, _device.ptr(self.bb_distances), summ, st), "bbox")
        self.bbox = np.array(summ[:4], dtype=np.float64)
        self.max_diagonal = float(summ[4]) if n > 0 else 0.0
        if prebuilt is not None:
            # nodes and bb_indices built elsewhere (a batched forest build)
            (self.node_child, self.node_Lmax, self.node_Rmin, self.node_ptr, self.node_size, self.node_dim,
             self.bb_indices, self.max_depth) = prebuilt
            nn = int(self.node_child.shape[0])
            self.n_nodes = nn
        else:
            nn = self._build(lib, st, device, bb_coords, n, n_buckets, cells_per_leaf)
        # packed traversal arrays
        self.nodes_f32 = _device.empty((max(nn, 1), 4), torch.float32, device)
        self.nodes_f64 = _device.empty((max(nn, 1), 2), torch.float64, device)
        self.poly_f64 = _device.empty((max(n, 1), K, 2), torch.float64, device)
        self.poly_f32 = _device.empty((max(n, 1), lib.ct_poly32_stride(K), 4), torch.float32, device)
        self.poly_len = _device.empty((max(n, 1),), torch.uint8, device)
        self.poly_len32 = _device.empty((max(n, 1),), torch.uint8, device)
        # node parents: trees deeper than the traversal stacks are walked through them
        self.node_parent = _device.empty((max(nn, 1),), torch.int32, device)
        self.error_word = torch.zeros((1,), dtype=torch.int32, device=device)
        self.grid_start = None
        self.desc = _lib.CtTree()
        self._fill_desc()
        self._gpu = None
        self._tuned = {}
        self.candidate_lists = candidate_lists
        _lib.check(lib.ct_pack_tree(ctypes.byref(self.desc), st), "pack")
        self.grid_density = self.GRID_CELLS_PER_ELEMENT
        if candidate_lists and n > 0:
            # a density tuned for trees of this size class (autotune(index=True)), if any
            self.grid_density = float(self.cached("index", 0).get("grid_density") or self.grid_density)
        self._build_index(self.grid_density)

    def _build_index(self, density: float):
        """Start-node grid and candidate lists of the batched float32 locate,
        about `density` grid cells per mesh cell."""
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        n = self.n
        bb = self.desc.bbox
        gx, gy = ctypes.c_int32(0), ctypes.c_int32(0)
        _lib.check(lib.ct_grid_shape(n, bb[1] - bb[0], bb[3] - bb[2], float(density),
                                     ctypes.byref(gx), ctypes.byref(gy)), "grid shape")
        self.grid_start = _device.empty((gx.value * gy.value,), torch.int32, self.device)
        self.desc.grid_start = _device.ptr(self.grid_start)
        self.desc.grid_nx, self.desc.grid_ny = gx.value, gy.value
        _lib.check(lib.ct_pack_grid(ctypes.byref(self.desc), st), "pack_grid")
        self.cand_off = self.cand_box = self.cand_idx = self.cand_lbox = None
        d = self.desc
        d.cand_off = d.cand_box = d.cand_idx = d.cand_lbox = None
        d.cand_n, d.cand_tol = 0, 0.0
        self.grid_density = float(density)
        if self.candidate_lists and int(self.desc.grid_nx) > 0 and n > 0:
            self._build_candidate_lists(lib, st)

    def _build(self, lib, st, device, bb_coords, n, n_buckets, cells_per_leaf) -> int:
        """build (creation.py:384-413) into node_* and bb_indices; returns n_nodes."""
        torch = _device.torch()
        factor = 1
        while True:
            wsz = lib.ct_build_workspace_size(n, n_buckets, factor)
            ws = _device.empty((max(int(wsz), 1),), torch.uint8, device)
            n_nodes = ctypes.c_int64(0)
            depth = ctypes.c_int32(0)
            status = lib.ct_build_tree(
                _device.ptr(bb_coords), n, n_buckets, cells_per_leaf, factor,
                _device.ptr(ws), wsz, ctypes.byref(n_nodes), ctypes.byref(depth), st,
            )
            if status == _lib.CT_ERR_WORKSPACE and factor < 4096:
                factor *= 8
                del ws
                continue
            _lib.check(status, "build")
            break
        nn = int(n_nodes.value)
        self.n_nodes = nn
        self.max_depth = int(depth.value)
        self.node_child = _device.empty((nn,), torch.int64, device)
        self.node_Lmax = _device.empty((nn,), torch.float64, device)
        self.node_Rmin = _device.empty((nn,), torch.float64, device)
        self.node_ptr = _device.empty((nn,), torch.int64, device)
        self.node_size = _device.empty((nn,), torch.int64, device)
        self.node_dim = _device.empty((nn,), torch.uint8, device)
        self.bb_indices = _device.empty((n,), torch.int64, device)
        _lib.check(
            lib.ct_build_emit(
                _device.ptr(ws), n, n_buckets, factor,
                _device.ptr(self.node_child), _device.ptr(self.node_Lmax), _device.ptr(self.node_Rmin),
                _device.ptr(self.node_ptr), _device.ptr(self.node_size), _device.ptr(self.node_dim),
                _device.ptr(self.bb_indices), st,
            ),
            "build_emit",
        )
        del ws
        return nn

    def _build_candidate_lists(self, lib, st):
        """Per-grid-cell candidate lists of the batched float32 locate."""
        torch = _device.torch()
        d = self.desc
        cells = int(d.grid_nx) * int(d.grid_ny)
        self.cand_off = _device.empty((cells + 1,), torch.int64, self.device)
        self.cand_box = _device.empty((self.n, 4), torch.float32, self.device)
        d.cand_off = _device.ptr(self.cand_off)
        d.cand_box = _device.ptr(self.cand_box)
        nbytes = int(lib.ct_cand_scratch_size(ctypes.byref(d)))
        scratch = _device.empty((nbytes,), torch.uint8, self.device)
        total = ctypes.c_int64(0)
        cover = default_tolerance(self.max_diagonal) * self.CAND_TOL_FACTOR
        _lib.check(lib.ct_cand_count(ctypes.byref(d), cover, _device.ptr(scratch), nbytes, ctypes.byref(total), st),
                   "candidate lists")
        if d.cand_tol <= 0.0:
            self.cand_off = self.cand_box = None
            d.cand_off = d.cand_box = None
            return
        m = max(int(total.value), 1)
        self.cand_idx = _device.empty((m,), torch.int32, self.device)
        self.cand_lbox = _device.empty((m, 4), torch.float32, self.device)
        d.cand_idx = _device.ptr(self.cand_idx)
        d.cand_lbox = _device.ptr(self.cand_lbox)
        _lib.check(lib.ct_cand_fill(ctypes.byref(d), _device.ptr(scratch), nbytes, st), "candidate lists")
        self.raise_on_device_error()  # the filling pass never writes past a grid cell's count

    def _fill_desc(self):
        d = self.desc
        P = _device.ptr
        d.elements = P(self.elements)
        d.vertices = P(self.vertices)
        d.bb_indices = P(self.bb_indices)
        d.bb_coords = P(self.bb_coords)
        d.node_child = P(self.node_child)
        d.node_Lmax = P(self.node_Lmax)
        d.node_Rmin = P(self.node_Rmin)
        d.node_ptr = P(self.node_ptr)
        d.node_size = P(self.node_size)
        d.node_dim = P(self.node_dim)
        d.n_elements = self.n
        d.n_vertices = int(self.vertices.shape[0])
        d.n_nodes = self.n_nodes
        d.n_max_vert = self.K
        d.max_depth = self.max_depth
        for k in range(4):
            d.bbox[k] = float(self.bbox[k])
        d.nodes_f32 = P(self.nodes_f32)
        d.nodes_f64 = P(self.nodes_f64)
        d.poly_f64 = P(self.poly_f64)
        d.poly_f32 = P(self.poly_f32)
        d.poly_len = P(self.poly_len)
        d.poly_len32 = P(self.poly_len32)
        d.error_word = P(self.error_word)
        d.node_parent = P(self.node_parent)
        d.grid_start = P(self.grid_start) if self.grid_start is not None else None

    def reset_error(self):
        self.error_word.zero_()

    def raise_on_device_error(self):
        err = int(self.error_word.item())
        if err:
            raise _lib.CellTreeError("device error: " + _lib.device_error_text(err))

    def stage_error(self):
        """Enqueue a copy of the error word into pinned host memory, to be read
        by raise_on_staged_error after a synchronisation the query makes anyway
        (a result count): one host round trip instead of two."""
        torch = _device.torch()
        if getattr(self, "_err_host", None) is None:
            self._err_host = torch.zeros((1,), dtype=torch.int32, pin_memory=True)
            self._err_event = torch.cuda.Event()
        self._err_host.copy_(self.error_word, non_blocking=True)
        self._err_event.record()

    def raise_on_staged_error(self):
        self._err_event.synchronize()  # complete already after the query's own synchronisation
        err = int(self._err_host.numpy()[0])
        if err:
            raise _lib.CellTreeError("device error: " + _lib.device_error_text(err))

    # -- point location ---------------------------------------------------------
    @staticmethod
    def auto_sort_bits(n_points: int) -> int:
        """Bits of the 24-bit Morton key the batched float32 form sorts the
        queries by: none for small batches (the sort costs more than the
        divergence it removes), else 16 (a 256 x 256 grid: with the candidate
        lists a finer order saves less in the query kernels than its third
        radix pass costs)."""
        return 0 if n_points < (1 << 16) else 16

    # deepest tree (levels + 2) the batched float32 locate takes
    BATCHED_MAX_STACK = 128

    # largest batch one library call takes (the entry points index queries
    # with 32-bit integers); larger batches are located slice by slice
    MAX_CALL_POINTS = 1 << 29

    # -- launch shapes (autotune.py) ------------------------------------------
    def gpu(self) -> str:
        if self._gpu is None:
            self._gpu = autotune.gpu_name(self.device)
        return self._gpu

    def tune_key(self, kind: str, n_queries: int) -> str:
        return autotune.cache_key(kind, self.gpu(), self.n, n_queries, K=self.K)

    def cached(self, kind: str, n_queries: int) -> dict:
        """Launch shape of `kind` for a batch of n_queries: tuned in this
        process, else from the cache file, else the library defaults."""
        key = self.tune_key(kind, n_queries)
        if key not in self._tuned:
            self._tuned[key] = autotune.lookup(kind, key)
        return self._tuned[key]

    def _apply(self, kind: str, cfg: dict) -> None:
        d = self.desc
        if kind == "locate":
            d.tune_cells_bpsm = int(cfg.get("cells_bpsm") or 0)
            d.tune_fast_bpsm = int(cfg.get("fast_bpsm") or 0)
        elif kind == "fp64":
            d.tune_fp64_stack = int(cfg.get("stack") or 0)
        elif kind in ("boxes", "segments"):
            d.tune_query_threads = int(cfg.get("threads") or 0)

    @staticmethod
    def _capturing() -> bool:
        torch = _device.torch()
        try:
            return bool(torch.cuda.is_current_stream_capturing())
        except Exception:  # pragma: no cover
            return False

    def maybe_tune(self, kind: str, n_queries: int, run, sample_n: int) -> dict:
        """The launch shape for a batch of n_queries; tunes it first (timing
        `run(cfg)` on a sample of sample_n queries) when autotuning is on,
        the batch is large enough, nothing is cached for its bucket and no
        stream capture is running."""
        key = self.tune_key(kind, n_queries)
        if key in self._tuned:
            return self._tuned[key]
        cached_entry = autotune.cache().get(key)
        if (cached_entry is None and autotune.enabled() and n_queries >= autotune.TUNE_MIN[kind]
                and not self._capturing()):
            self._tuned[key] = self.tune(kind, key, run, sample_n)
        return self.cached(kind, n_queries)

    def tune(self, kind: str, key: str, run, sample_n: int) -> dict:
        """Coordinate descent over the knobs of `kind` (one knob at a time,
        the others at their best so far), timing run(cfg) on the sample;
        stores the best in the cache and returns it merged over the defaults."""
        cfg = dict(autotune.DEFAULTS[kind])
        if kind == "locate":
            cfg["sort_bits"] = self.auto_sort_bits(sample_n)
        default = dict(cfg)
        entries = []
        for knob in sorted(autotune.SPACE[kind]):
            cands = [dict(cfg, **{knob: v}) for v in autotune.SPACE[kind][knob]]
            e = autotune.tune(kind, key, run, cands, store=False, default=default)
            entries.append(e)
            cfg = dict(e["config"])
        best_ms = min(e["ms"] for e in entries)
        d_ms = next((e["default_ms"] for e in entries if e["default_ms"] is not None), None)
        entry = {"config": cfg, "ms": best_ms, "default_ms": d_ms, "candidates": sum(e["candidates"] for e in entries),
                 "sample": int(sample_n)}
        autotune.cache().put(key, entry)
        merged = dict(autotune.DEFAULTS[kind])
        merged.update(cfg)
        return merged

    def locate(self, points_d, out_d, tolerance: float, precision: str, sort_bits=None, config=None,
               slot: int = 0) -> None:
        """Enqueue point location on the current stream (no synchronisation).
        `config`: launch shape (autotune.DEFAULTS["locate"] keys), else the
        cached one for this batch size.  `slot`: workspace of the batched
        form; calls that may run at the same time (other streams) use
        different slots."""
        lib = _lib.load()
        n = int(points_d.shape[0])
        if n > self.MAX_CALL_POINTS:
            for s in range(0, n, self.MAX_CALL_POINTS):
                e = min(s + self.MAX_CALL_POINTS, n)
                self.locate(points_d[s:e], out_d[s:e], tolerance, precision, sort_bits, config, slot)
            return
        if precision == "fp32" and self.max_depth + 2 > self.BATCHED_MAX_STACK:
            precision = "fp64"  # the batched form's stacks hold 126 levels; deeper trees take the float64 walk
        if precision == "fp32":
            cfg = config if config is not None else self.cached("locate", n)
            self._apply("locate", cfg)
            if sort_bits is None:
                sort_bits = cfg.get("sort_bits")
            g = self.auto_sort_bits(n) if sort_bits is None else int(sort_bits)
            need = int(lib.ct_locate_workspace_size(n, g))
            name = "_locate_ws" if slot == 0 else f"_locate_ws{slot}"
            ws = getattr(self, name, None)
            if ws is None or ws.numel() < need:
                torch = _device.torch()
                ws = _device.empty((need,), torch.uint8, self.device)
                setattr(self, name, ws)
            _lib.check(
                lib.ct_locate_points_batched(
                    ctypes.byref(self.desc), _device.ptr(points_d), n, float(tolerance), g, _device.ptr(out_d),
                    _device.ptr(ws), int(ws.numel()), _device.stream(),
                ),
                "locate_points",
            )
            return
        mode = _lib.CT_MODE_FP64 if precision == "fp64" else _lib.CT_MODE_FP32
        self._apply("fp64", config if config is not None else self.cached("fp64", n))
        _lib.check(
            lib.ct_locate_points(ctypes.byref(self.desc), _device.ptr(points_d), n, float(tolerance), mode,
                                 _device.ptr(out_d), _device.stream()),
            "locate_points",
        )

    def tune_locate(self, points_d, tolerance: float, precision: str = "fp32", n_call: Optional[int] = None) -> dict:
        """Tune the launch shape of point location now, timing calls on the
        device points `points_d`, for batches of n_call points (default: as
        many as points_d holds); returns the cache entry (config, ms,
        default_ms)."""
        torch = _device.torch()
        n = int(points_d.shape[0])
        out = _device.empty((n,), torch.int64, self.device)
        kind = "locate" if precision == "fp32" else "fp64"
        key = self.tune_key(kind, n if n_call is None else n_call)
        self._tuned[key] = self.tune(kind, key, lambda c: self.locate(points_d, out, tolerance, precision, config=c), n)
        return autotune.cache().get(key) or {"config": self._tuned[key]}

    def maybe_tune_locate(self, points, tolerance: float, precision: str, n_call: int) -> None:
        """First-use tuning of point location for batches of n_call points
        (host or device `points`; a strided sample of at most one call's
        size is timed on the device)."""
        kind = "locate" if precision == "fp32" else "fp64"
        key = self.tune_key(kind, n_call)
        if self.max_depth + 2 > self.BATCHED_MAX_STACK:
            return
        if (key in self._tuned or not autotune.enabled() or n_call < autotune.TUNE_MIN[kind] or self._capturing()
                or autotune.cache().get(key) is not None):
            return
        torch = _device.torch()
        m = min(int(points.shape[0]), n_call if kind == "locate" else autotune.SAMPLE_MAX[kind])
        step = max(1, int(points.shape[0]) // max(m, 1))
        if isinstance(points, torch.Tensor):
            sample = points[::step][:m].contiguous()
        else:
            sample = torch.as_tensor(np.ascontiguousarray(points[::step][:m]), device=self.device)
        self.tune_locate(sample, tolerance, precision, n_call=n_call)

    def rebuild_index(self, density: float) -> None:
        """Rebuild the start-node grid and candidate lists at `density` grid
        cells per mesh cell (speed only; results never change)."""
        self._build_index(density)

    # -- multi-result helpers ------------------------------------------------
    def scan(self, counts):
        """Exclusive scan of int64 counts on the device -> (offsets, total)."""
        torch = _device.torch()
        lib = _lib.load()
        n = int(counts.shape[0])
        wsz = lib.ct_scan_workspace_size(n)
        ws = _device.empty((max(int(wsz), 8),), torch.uint8, self.device)
        offsets = _device.empty((n,), torch.int64, self.device)
        total = ctypes.c_int64(0)
        _lib.check(
            lib.ct_exclusive_scan(_device.ptr(counts), n, _device.ptr(offsets), _device.ptr(ws), wsz,
                                  ctypes.byref(total), _device.stream()),
            "scan",
        )
        return offsets, int(total.value)

    # queries per batch from which box / segment queries run in work order
    # (below it the ordering's fixed cost outweighs the better warp balance)
    WORK_ORDER_MIN = 65536

    def work_order(self, q_d, kind: int, force=None):
        """Permutation grouping box (kind 0) / segment (kind 1) queries of
        similar size, or None for small batches (`force` True / False
        overrides the size rule)."""
        n = int(q_d.shape[0])
        if force is False or (force is None and n < self.WORK_ORDER_MIN):
            return None
        torch = _device.torch()
        lib = _lib.load()
        nbytes = int(lib.ct_work_order_workspace_size(n))
        ws = _device.empty((nbytes,), torch.uint8, self.device)
        order = _device.empty((n,), torch.int32, self.device)
        cell = max(self.max_diagonal, 1e-300)
        _lib.check(lib.ct_work_order(_device.ptr(q_d), n, kind, cell, _device.ptr(order), _device.ptr(ws), nbytes,
                                     _device.stream()), "work order")
        return order

    def ensure_box_index(self):
        """Build the box index of the multi-result queries on first use (cell
        boxes in leaf order, also in the float32 frame, node bounding boxes
        and leaf ranges)."""
        if self.desc.node_box or not self.desc.bounds_finite or self.n == 0:
            return
        torch = _device.torch()
        lib = _lib.load()
        self.bb_leaf = _device.empty((self.n, 4), torch.float64, self.device)
        self.bb_leaf32 = _device.empty((self.n, 4), torch.float32, self.device)
        self.node_box = _device.empty((self.n_nodes, 8), torch.int32, self.device)
        self.leaf_start = _device.empty((self.n,), torch.int32, self.device)
        d = self.desc
        d.bb_leaf = _device.ptr(self.bb_leaf)
        d.bb_leaf32 = _device.ptr(self.bb_leaf32)
        d.node_box = _device.ptr(self.node_box)
        d.leaf_start = _device.ptr(self.leaf_start)
        nbytes = int(lib.ct_box_index_scratch_size(ctypes.byref(d)))
        scratch = _device.empty((max(nbytes, 1),), torch.uint8, self.device)
        status = lib.ct_pack_box_index(ctypes.byref(d), _device.ptr(scratch), nbytes, _device.stream())
        if status != _lib.CT_OK:
            d.bb_leaf = d.bb_leaf32 = d.node_box = d.leaf_start = None
            _lib.check(status, "box index")

    # -- output-budgeted chunks of multi-result queries ------------------------
    def count_boxes(self, boxes_d):
        """Result pairs of every box query (device int64)."""
        torch = _device.torch()
        n = int(boxes_d.shape[0])
        counts = _device.empty((n,), torch.int64, self.device)
        self.ensure_box_index()
        _lib.check(_lib.load().ct_count_boxes(ctypes.byref(self.desc), _device.ptr(boxes_d), n, None,
                                              _device.ptr(counts), _device.stream()), "count_boxes")
        return counts

    def count_edge_candidates(self, segs_d, mode: int):
        """Candidate cells of every segment (device int64): an upper bound of
        its results."""
        n = int(segs_d.shape[0])
        self.ensure_box_index()
        cfg = self.cached("segments", n)
        self._apply("segments", cfg)
        _, ccnt, _, _ = self.edge_candidate_ranges(segs_d, mode, None, self.edge_cut(cfg, n))
        return ccnt

    # cells under a work item of the split segment traversal (the default)
    SPLIT_CELLS = 1024
    # work items from which their memory is checked against the free memory
    ITEMS_CHECK_MIN = 1 << 20

    # batches from which segment traversals run uncut by default (enough
    # segments to fill the GPU; the split then only adds its item pass)
    SPLIT_MAX_SEGMENTS = 1 << 17

    def edge_cut(self, cfg: dict, n_segments: int = 0):
        """Depth at which segment traversals are cut into work items (about
        cfg["split"] cells under each; by default SPLIT_CELLS for batches
        below SPLIT_MAX_SEGMENTS, else uncut), or None for the uncut
        traversal (no split asked, a tree too small to split or too deep for
        the stacked traversal)."""
        split = cfg.get("split")
        if split is None:
            split = self.SPLIT_CELLS if n_segments < self.SPLIT_MAX_SEGMENTS else 0
        split = int(split or 0)
        if split <= 0 or self.n <= split or self.max_depth + 2 > self.BATCHED_MAX_STACK:
            return None
        return max(1, min(self.max_depth, int(np.ceil(np.log2(self.n / split)))))

    # uncut batches up to this many segments keep each segment's first
    # SEG_SPEC_CAP candidates in the counting pass (one traversal for most;
    # halved until the scratch fits SEG_SPEC_MAX_BYTES, none below 8)
    SPEC_MAX_SEGMENTS = 1 << 22
    SEG_SPEC_CAP = 128
    SEG_SPEC_MAX_BYTES = 1 << 31

    def edge_candidate_ranges(self, segs_d, mode: int, order, cut, keep: bool = False):
        """Every segment's candidate offset and count (device int64) and the
        candidate total, and what the writing pass uses: (coff, ccnt, total,
        items) -- items None (traverse again), ("spec", scratch, cap) with
        `keep` (the counting pass kept each segment's first `cap`
        candidates), or with a
        cut the work items (item_seg, item_node, n_items, item offsets)."""
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        P = _device.ptr
        n = int(segs_d.shape[0])
        d = ctypes.byref(self.desc)
        if cut is None:
            ccnt = _device.empty((n,), torch.int64, self.device)
            cap = int(self.SEG_SPEC_CAP)
            while cap >= 8 and n * cap * 4 > self.SEG_SPEC_MAX_BYTES:
                cap //= 2
            if keep and 0 < n <= self.SPEC_MAX_SEGMENTS and cap >= 1 and (cap >= 8 or cap == self.SEG_SPEC_CAP):
                spec = _device.empty((n, cap), torch.int32, self.device)
                _lib.check(lib.ct_count_edge_candidates_spec(d, mode, P(segs_d), n, P(order), P(ccnt), P(spec),
                                                             cap, st), "intersect_edges")
                coff, nc = self.scan(ccnt)
                return coff, ccnt, nc, ("spec", spec, cap)
            _lib.check(lib.ct_count_edge_candidates(d, mode, P(segs_d), n, P(order), P(ccnt), st), "intersect_edges")
            coff, nc = self.scan(ccnt)
            return coff, ccnt, nc, None
        icnt = _device.empty((n,), torch.int64, self.device)
        while True:
            _lib.check(lib.ct_count_edge_items(d, mode, P(segs_d), n, P(order), cut, P(icnt), st),
                       "intersect_edges")
            ioff, ni = self.scan(icnt)
            # items take 24 bytes each in flight: a coarser cut when they
            # would not fit (a level less about halves them)
            if ni <= self.ITEMS_CHECK_MIN or cut <= 1:
                break
            room = self.device_budget(24)
            if ni <= room:
                break
            cut = max(1, cut - int(np.ceil(np.log2(ni / room))))
        iseg = _device.empty((max(ni, 1),), torch.int32, self.device)
        inode = _device.empty((max(ni, 1),), torch.int32, self.device)
        _lib.check(lib.ct_write_edge_items(d, mode, P(segs_d), n, P(order), cut, P(ioff), P(iseg), P(inode), st),
                   "intersect_edges")
        iccnt = _device.empty((max(ni, 1),), torch.int64, self.device)
        _lib.check(lib.ct_count_item_candidates(d, mode, P(segs_d), P(iseg), P(inode), ni, P(iccnt), st),
                   "intersect_edges")
        icoff, nc = self.scan(iccnt[:ni]) if ni > 0 else (iccnt[:0], 0)
        coff = _device.empty((n,), torch.int64, self.device)
        ccnt = _device.empty((n,), torch.int64, self.device)
        _lib.check(lib.ct_segment_candidate_ranges(P(ioff), P(icnt), n, P(icoff), P(iccnt), ni, P(coff), P(ccnt),
                                                   st), "intersect_edges")
        return coff, ccnt, nc, (iseg, inode, ni, icoff)

    @staticmethod
    def chunk_ranges(counts: np.ndarray, max_results: int):
        """Contiguous query ranges [s, e) whose summed counts stay within
        max_results (a single query above it forms a range of its own)."""
        n = int(counts.shape[0])
        if n == 0:
            return [(0, 0)]
        cum = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
        out, s = [], 0
        while s < n:
            e = int(np.searchsorted(cum, cum[s] + max(int(max_results), 1), side="right")) - 1
            e = min(max(e, s + 1), n)
            out.append((s, e))
            s = e
        return out

    def device_budget(self, bytes_per_result: int) -> int:
        """Results one device pass may produce: a quarter of the free device
        memory over the bytes a result needs in flight."""
        torch = _device.torch()
        free, _ = torch.cuda.mem_get_info(self.device)
        return max(1 << 20, int(free // 4 // max(bytes_per_result, 1)))

    # pairs from which subtrees inside a box are written by a warp each after
    # the traversal (below, the extra launch costs more than it saves)
    BOX_JOBS_MIN_PAIRS = 1 << 20
    # the counting pass keeps each box's first SPEC_CAP pairs (batches up to
    # SPEC_MAX_BOXES boxes; SPEC_CAP_LARGE beyond, scratch up to
    # SPEC_MAX_BYTES), so boxes whose pairs fit are traversed once;
    # SPEC_MAX_BOXES = 0 switches it off
    SPEC_MAX_BOXES = 1 << 16
    SPEC_CAP = 64
    SPEC_CAP_LARGE = 16
    SPEC_MAX_BYTES = 1 << 30

    def locate_boxes(self, boxes_d, config=None, budget=None):
        """Pairs (box, cell) of every box query, box-major in upstream order;
        with `budget`, returns None instead when the pairs would exceed it
        (the per-box counts are left in self.last_counts)."""
        n = int(boxes_d.shape[0])
        if config is None:
            m = min(n, autotune.SAMPLE_MAX["boxes"])
            step = max(1, n // max(m, 1))
            config = self.maybe_tune("boxes", n, lambda c: self.locate_boxes(boxes_d[::step][:m].contiguous(), c), m)
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        counts = _device.empty((n,), torch.int64, self.device)
        self.reset_error()
        self.ensure_box_index()
        self._apply("boxes", config)
        order = self.work_order(boxes_d, 0, config.get("work_order"))
        spec = None
        cap = self.SPEC_CAP if n <= self.SPEC_MAX_BOXES else self.SPEC_CAP_LARGE
        if self.SPEC_MAX_BOXES > 0 and 0 < n and n * cap * 4 <= self.SPEC_MAX_BYTES:
            # one traversal: the counting pass also keeps each box's first pairs
            spec = _device.empty((n, cap), torch.int32, self.device)
            _lib.check(lib.ct_count_boxes_spec(ctypes.byref(self.desc), _device.ptr(boxes_d), n, _device.ptr(order),
                                               _device.ptr(counts), _device.ptr(spec), cap, st),
                       "locate_boxes")
        else:
            _lib.check(lib.ct_count_boxes(ctypes.byref(self.desc), _device.ptr(boxes_d), n, _device.ptr(order),
                                          _device.ptr(counts), st), "locate_boxes")
        self.stage_error()
        offsets, total = self.scan(counts)
        self.raise_on_staged_error()
        if budget is not None and total > budget:
            self.last_counts = counts
            return None
        ii = _device.empty((total,), torch.int64, self.device)
        jj = _device.empty((total,), torch.int64, self.device)
        # the writing pass repeats the counting pass's traversal: a condition
        # it could report has been reported by the count
        if spec is not None:
            jm = int(config.get("job_cells") or 0)
            wsz = int(lib.ct_write_boxes_workspace_size(total, jm))
            ws = _device.empty((wsz,), torch.uint8, self.device)
            _lib.check(
                lib.ct_write_boxes_spec(ctypes.byref(self.desc), _device.ptr(boxes_d), n, _device.ptr(order),
                                        _device.ptr(counts), _device.ptr(offsets), _device.ptr(spec), cap,
                                        total, jm, _device.ptr(ii), _device.ptr(jj), _device.ptr(ws), wsz, st),
                "locate_boxes",
            )
            return ii, jj
        if total < self.BOX_JOBS_MIN_PAIRS:
            _lib.check(
                lib.ct_write_boxes(ctypes.byref(self.desc), _device.ptr(boxes_d), n, _device.ptr(order),
                                   _device.ptr(offsets), _device.ptr(ii), _device.ptr(jj), st),
                "locate_boxes",
            )
            return ii, jj
        jm = int(config.get("job_cells") or 0)
        wsz = int(lib.ct_write_boxes_workspace_size(total, jm))
        ws = _device.empty((wsz,), torch.uint8, self.device)
        _lib.check(
            lib.ct_write_boxes_ws(ctypes.byref(self.desc), _device.ptr(boxes_d), n, _device.ptr(order),
                                  _device.ptr(offsets), total, jm, _device.ptr(ii), _device.ptr(jj),
                                  _device.ptr(ws), wsz, st),
            "locate_boxes",
        )
        return ii, jj

    def locate_edges(self, segs_d, mode: int, config=None, budget=None):
        """Candidates (traversal) -> float64 cell test per candidate -> hits
        in candidate order -> per-segment sort by t; returns ii, jj, xy (R, 2, 2).
        With `budget`, returns None instead when the candidates would exceed
        it (the per-segment candidate counts are left in self.last_counts)."""
        n = int(segs_d.shape[0])
        if config is None:
            m = min(n, autotune.SAMPLE_MAX["segments"])
            step = max(1, n // max(m, 1))
            config = self.maybe_tune("segments", n,
                                     lambda c: self.locate_edges(segs_d[::step][:m].contiguous(), mode, c), m)
        torch = _device.torch()
        lib = _lib.load()
        st = _device.stream()
        self.reset_error()
        self.ensure_box_index()
        self._apply("segments", config)
        order = self.work_order(segs_d, 1, config.get("work_order"))
        P = _device.ptr
        coff, ccnt, nc, items = self.edge_candidate_ranges(segs_d, mode, order, self.edge_cut(config, n), keep=True)
        if budget is not None and nc > budget:
            self.last_counts = ccnt
            return None
        cseg = _device.empty((max(nc, 1),), torch.int32, self.device)
        cpos = _device.empty((max(nc, 1),), torch.int32, self.device)
        if items is None:
            _lib.check(lib.ct_write_edge_candidates(ctypes.byref(self.desc), mode, P(segs_d), n, P(order), P(coff),
                                                    P(cseg), P(cpos), st), "intersect_edges")
        elif isinstance(items[0], str):
            _lib.check(lib.ct_write_edge_candidates_spec(ctypes.byref(self.desc), mode, P(segs_d), n, P(order),
                                                         P(ccnt), P(coff), P(items[1]), items[2], P(cseg),
                                                         P(cpos), st), "intersect_edges")
            del items
        else:
            iseg, inode, ni, icoff = items
            _lib.check(lib.ct_write_item_candidates(ctypes.byref(self.desc), mode, P(segs_d), P(iseg), P(inode), ni,
                                                    P(icoff), P(cseg), P(cpos), st), "intersect_edges")
            del items, iseg, inode, icoff
        keep = _device.empty((max(nc, 1),), torch.int64, self.device)
        xy_c = _device.empty((max(nc, 1), 2, 2), torch.float64, self.device)
        _lib.check(lib.ct_test_edge_candidates(ctypes.byref(self.desc), mode, P(segs_d), P(cseg), P(cpos), nc,
                                               P(keep), P(xy_c), st), "intersect_edges")
        self.stage_error()
        pos, total = self.scan(keep[:nc]) if nc > 0 else (keep[:0], 0)
        self.raise_on_staged_error()
        ii = _device.empty((total,), torch.int64, self.device)
        jj = _device.empty((total,), torch.int64, self.device)
        xy = _device.empty((total, 2, 2), torch.float64, self.device)
        offsets = _device.empty((n,), torch.int64, self.device)
        counts = _device.empty((n,), torch.int64, self.device)
        _lib.check(lib.ct_compact_edge_hits(ctypes.byref(self.desc), P(keep), P(pos), nc, P(cseg), P(cpos), P(xy_c),
                                            P(coff), P(ccnt), n, P(ii), P(jj), P(xy), P(offsets), P(counts), st),
                   "intersect_edges")
        del cseg, cpos, keep, xy_c, pos
        if total > 0:
            jj2 = _device.empty((total,), torch.int64, self.device)
            xy2 = _device.empty((total, 2, 2), torch.float64, self.device)
            wsz = lib.ct_sort_workspace_size(total)
            ws = _device.empty((int(wsz),), torch.uint8, self.device)
            _lib.check(
                lib.ct_sort_intersections(
                    P(segs_d), n, P(offsets), P(counts), P(ii), P(jj), P(xy), total, P(jj2), P(xy2), P(ws), wsz, st,
                ),
                "sort_intersections",
            )
            jj, xy = jj2, xy2
        return ii, jj, xy

    # pairs from which the per-pair kernels run grouped by polygon lengths
    PAIR_ORDER_MIN = 65536

    def pair_order(self, fa, Ka: int, ia, fb, Kb: int, ib):
        """Processing order of the per-pair kernels (pairs of equal polygon
        lengths side by side), or None when every pair has the same lengths
        or the batch is small."""
        n = int(ib.shape[0])
        uniform = Kb <= 3 and (fa is None or Ka <= 3)  # boxes have 4 vertices, triangles 3
        if n < self.PAIR_ORDER_MIN or uniform:
            return None
        torch = _device.torch()
        lib = _lib.load()
        nbytes = int(lib.ct_pair_order_workspace_size(n))
        ws = _device.empty((nbytes,), torch.uint8, self.device)
        order = _device.empty((n,), torch.int32, self.device)
        _lib.check(lib.ct_pair_order(_device.ptr(fa), Ka, _device.ptr(ia), _device.ptr(fb), Kb, _device.ptr(ib), n,
                                     _device.ptr(order), _device.ptr(ws), nbytes, _device.stream()), "pair order")
        return order

    def compact(self, ii, jj, area=None, flag=None):
        """Keep pairs with area > 0 (or flag != 0)."""
        torch = _device.torch()
        lib = _lib.load()
        n = int(ii.shape[0])
        ii_o = _device.empty((n,), torch.int64, self.device)
        jj_o = _device.empty((n,), torch.int64, self.device)
        a_o = _device.empty((n,), torch.float64, self.device) if area is not None else None
        wsz = lib.ct_compact_workspace_size(n)
        ws = _device.empty((int(wsz),), torch.uint8, self.device)
        total = ctypes.c_int64(0)
        _lib.check(
            lib.ct_compact_pairs(
                _device.ptr(area), _device.ptr(flag), n, _device.ptr(ii), _device.ptr(jj), _device.ptr(ii_o),
                _device.ptr(jj_o), _device.ptr(a_o), _device.ptr(ws), wsz, ctypes.byref(total), _device.stream(),
            ),
            "compact",
        )
        m = int(total.value)
        out = (ii_o[:m], jj_o[:m])
        if a_o is not None:
            out = out + (a_o[:m],)
        return out

    def node_bounds(self, nodes_host=None):
        """collect_node_bounds query.py:568-622 on the device."""
        torch = _device.torch()
        lib = _lib.load()
        child, Lmax, Rmin, dim = self.node_child, self.node_Lmax, self.node_Rmin, self.node_dim
        if nodes_host is not None:
            child = torch.as_tensor(np.ascontiguousarray(nodes_host["child"], dtype=np.int64), device=self.device)
            Lmax = torch.as_tensor(np.ascontiguousarray(nodes_host["Lmax"]), device=self.device)
            Rmin = torch.as_tensor(np.ascontiguousarray(nodes_host["Rmin"]), device=self.device)
            dim = torch.as_tensor(np.ascontiguousarray(nodes_host["dim"], dtype=np.uint8), device=self.device)
        n = int(child.shape[0])
        parent = _device.empty((max(n, 1),), torch.int64, self.device)
        out = _device.empty((n, 4), torch.float64, self.device)
        bbox = (ctypes.c_double * 4)(*[float(x) for x in self.bbox])
        _lib.check(
            lib.ct_node_bounds(_device.ptr(child), _device.ptr(Lmax), _device.ptr(Rmin), _device.ptr(dim), n, bbox,
                               _device.ptr(parent), _device.ptr(out), _device.stream()),
            "node_bounds",
        )
        return out, (child, Lmax, Rmin, dim)

    def validate_node_bounds(self, nodes_host=None):
        torch = _device.torch()
        lib = _lib.load()
        nbnd, (child, _, _, _) = self.node_bounds(nodes_host)
        ptr, size = self.node_ptr, self.node_size
        if nodes_host is not None:
            ptr = torch.as_tensor(np.ascontiguousarray(nodes_host["ptr"], dtype=np.int64), device=self.device)
            size = torch.as_tensor(np.ascontiguousarray(nodes_host["size"], dtype=np.int64), device=self.device)
        n = int(child.shape[0])
        valid = _device.empty((n,), torch.uint8, self.device)
        _lib.check(
            lib.ct_validate_node_bounds(_device.ptr(child), _device.ptr(ptr), _device.ptr(size), n,
                                        _device.ptr(self.bb_indices), _device.ptr(self.bb_coords),
                                        _device.ptr(nbnd), _device.ptr(valid), _device.stream()),
            "validate_node_bounds",
        )
        return valid

    def host_nodes(self) -> np.ndarray:
        nodes = np.empty(self.n_nodes, dtype=NodeDType)
        nodes["child"] = self.node_child.cpu().numpy()
        nodes["Lmax"] = self.node_Lmax.cpu().numpy()
        nodes["Rmin"] = self.node_Rmin.cpu().numpy()
        nodes["ptr"] = self.node_ptr.cpu().numpy()
        nodes["size"] = self.node_size.cpu().numpy()
        nodes["dim"] = self.node_dim.cpu().numpy().astype(bool)
        return nodes


def validate_elements(elements, n_vertices: int, min_len: int, what: str) -> None:
    """Reject element arrays that index outside the vertex array (a GPU kernel
    must never read through an invalid index)."""
    lib = _lib.load()
    bad = ctypes.c_int32(0)
    n, K = int(elements.shape[0]), int(elements.shape[1])
    _lib.check(
        lib.ct_validate_elements(_device.ptr(elements), n, K, min_len, n_vertices, ctypes.byref(bad), _device.stream()),
        "validate",
    )
    if bad.value:
        raise ValueError(f"{what} contain indices outside [0, n_vertices)")


def prebuilt_from_nodes(nodes, bb_indices, n: int, device):
    """Device copies of upstream ``nodes`` (NodeDType) and ``bb_indices`` of a
    tree of n elements, checked for the structure the queries rely on
    (children after their parent and inside the array, bb_indices a
    permutation), plus the tree's depth: the ``prebuilt`` argument of
    _GpuTree."""
    torch = _device.torch()
    nodes = np.asarray(nodes)
    bb_indices = np.ascontiguousarray(bb_indices, dtype=np.int64)
    for name in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        if nodes.dtype.names is None or name not in nodes.dtype.names:
            raise ValueError(f"nodes must be a NodeDType array (missing {name})")
    if bb_indices.shape != (n,) or not np.array_equal(np.sort(bb_indices), np.arange(n)):
        raise ValueError("bb_indices must be a permutation of the element indices")
    nn = nodes.shape[0]
    child = np.ascontiguousarray(nodes["child"], dtype=np.int64)
    # depth of every node (children are numbered after their parent)
    internal = child >= 0
    if np.any(child[internal] <= np.nonzero(internal)[0]) or np.any(child[internal] + 1 >= nn):
        raise ValueError("nodes: children must follow their parent and lie inside the array")
    depth = np.zeros(nn, dtype=np.int64)
    frontier, level = np.array([0], dtype=np.int64), 0
    while frontier.size and level <= nn:
        c = child[frontier]
        c = c[c >= 0]
        frontier = np.concatenate([c, c + 1])
        level += 1
        depth[frontier] = level
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), device=device).to(dt)
    return (dev(child, torch.int64), dev(nodes["Lmax"], torch.float64), dev(nodes["Rmin"], torch.float64),
            dev(nodes["ptr"], torch.int64), dev(nodes["size"], torch.int64),
            dev(nodes["dim"].astype(np.uint8), torch.uint8), dev(bb_indices, torch.int64), int(depth.max()))


def _validate_params(n_buckets: int, cells_per_leaf: int) -> None:
    if n_buckets < 2:
        raise ValueError("n_buckets must be >= 2")
    if cells_per_leaf < 1:
        raise ValueError("cells_per_leaf must be >= 1")
    if n_buckets > MAX_N_BUCKETS:
        raise ValueError(f"n_buckets must be <= {MAX_N_BUCKETS} on the GPU builder")


class CellTree2dBase:
    """Common attributes and host views of CellTree2d / EdgeCellTree2d."""

    _tree: _GpuTree
    _elements_name = "faces"
    _host: dict

    # -- host views (upstream public attributes) --------------------------
    def _cached(self, name, fn):
        if name not in self._host:
            self._host[name] = fn()
        return self._host[name]

    @property
    def vertices(self) -> np.ndarray:
        return self._cached("vertices", lambda: self._tree.vertices.cpu().numpy())

    @property
    def nodes(self) -> np.ndarray:
        return self._cached("nodes", self._tree.host_nodes)

    @property
    def bb_indices(self) -> np.ndarray:
        return self._cached("bb_indices", lambda: self._tree.bb_indices.cpu().numpy())

    @property
    def bb_coords(self) -> np.ndarray:
        return self._cached("bb_coords", lambda: self._tree.bb_coords.cpu().numpy())

    @property
    def bb_distances(self) -> np.ndarray:
        return self._cached("bb_distances", lambda: self._tree.bb_distances.cpu().numpy())

    @property
    def bbox(self) -> np.ndarray:
        return self._tree.bbox

    @property
    def celltree_data(self) -> CellTreeData:
        return CellTreeData(
            getattr(self, self._elements_name), self.vertices, self.nodes, self.bb_indices, self.bb_coords,
            self.bbox, self.cells_per_leaf,
        )

    @property
    def node_bounds(self) -> np.ndarray:
        """Bounds (xmin, xmax, ymin, ymax) of every node (celltree_base.py:62-64)."""
        out, _ = self._tree.node_bounds(self._host.get("nodes"))
        return out.cpu().numpy()

    def validate_node_bounds(self) -> np.ndarray:
        """For every node whether its children (or leaf boxes) lie inside its
        bounds (celltree_base.py:66-80).  Uses the host ``nodes`` array when it
        has been accessed (and possibly edited), like upstream."""
        return self._tree.validate_node_bounds(self._host.get("nodes")).cpu().numpy().astype(bool)

    def to_dict_of_lists(self):
        """celltree_base.py:82-114"""
        child = self.nodes["child"]
        d = {}
        for parent_index, c in enumerate(child):
            d[parent_index] = [] if c == -1 else [int(c), int(c) + 1]
        return d

    # -- helpers -----------------------------------------------------------
    def _tolerance(self, tolerance: Optional[float]) -> float:
        if tolerance is None:
            return default_tolerance(self._tree.max_diagonal)
        return float(tolerance)
