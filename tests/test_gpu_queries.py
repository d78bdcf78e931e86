"""Multi-result queries, pair kernels, barycentric weights and node-bound
diagnostics on the GPU against the upstream fixtures and the oracle.
Indices must be identical (and in the same order); float outputs are computed
in the upstream evaluation order and must be identical too."""

import numpy as np
import pytest

from meshes import GOLDEN, meshes
from numba_celltree_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

G = np.load(GOLDEN / "golden_trees.npz")


def same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.dtype.kind == "f":
        assert np.array_equal(a, b, equal_nan=True)
    else:
        assert np.array_equal(a, b)


def teq(a, b):
    """Bitwise-equal device tensors, NaN equal to NaN."""
    import torch

    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    if a.is_floating_point():
        na, nb = torch.isnan(a), torch.isnan(b)
        return torch.equal(na, nb) and torch.equal(torch.where(na, 0.0, a), torch.where(nb, 0.0, b))
    return torch.equal(a, b)


def case(i):
    p = f"c{i}_"
    return {k[len(p):]: G[k] for k in G.files if k.startswith(p)}


@pytest.mark.parametrize("i", range(int(G["n_cases"])))
def test_queries_match_upstream_fixtures(i):
    from numba_celltree_gb300 import CellTree2d

    c = case(i)
    nb, cpl = (int(x) for x in c["params"])
    t = CellTree2d(c["vertices"], c["faces_in"], -1, nb, cpl)
    bi, bj = t.locate_boxes(c["boxes"])
    same(bi, c["box_i"])
    same(bj, c["box_j"])
    for got, key in zip(t.intersect_boxes(c["boxes"]), ("ibox_i", "ibox_j", "ibox_a")):
        same(got, c[key])
    for got, key in zip(t.intersect_edges(c["edges"]), ("edge_i", "edge_j", "edge_xy")):
        same(got, c[key])
    for got, key in zip(t.intersect_faces(c["qv"], c["qf"], -1), ("face_i", "face_j", "face_a")):
        same(got, c[key])
    qf = c["qf"].astype(np.int64).copy()
    for got, key in zip(t.locate_faces(c["qv"].copy(), qf), ("lface_i", "lface_j")):
        same(got, c[key])
    for prec in ("fp32", "fp64"):
        t.precision = prec
        for got, key in zip(t.compute_barycentric_weights(c["points"]), ("bary_i", "bary_w")):
            same(got, c[key])
    same(t.node_bounds, c["node_bounds"])
    same(t.validate_node_bounds(), c["node_valid"])


@pytest.mark.parametrize("i", range(int(G["n_edge_cases"])))
def test_edge_tree_matches_upstream_fixtures(i):
    from numba_celltree_gb300 import EdgeCellTree2d

    p = f"e{i}_"
    c = {k[len(p):]: G[k] for k in G.files if k.startswith(p)}
    nb, cpl = (int(x) for x in c["params"])
    t = EdgeCellTree2d(c["vertices"], c["edges"], nb, cpl)
    for f in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        same(t.nodes[f], c["node_" + f])
    same(t.bb_indices, c["bb_indices"])
    same(t.bb_coords, c["bb_coords"])
    same(t.locate_points(c["points"]), c["locate"])
    for got, key in zip(t.intersect_edges(c["segs"]), ("edge_i", "edge_j", "edge_xy")):
        same(got, c[key])


@pytest.mark.parametrize("name", ["tri150", "mixed60", "utm80", "rot_quads"])
def test_queries_match_oracle(oracle, name):
    from numba_celltree_gb300 import CellTree2d

    xy, f = meshes()[name]
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    lo, hi = xy.min(0), xy.max(0)
    span = float((hi - lo).max())
    boxes = syn.random_boxes(3000, lo, hi, 0.001 * span, 0.05 * span, seed=1)
    for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
        same(a, b)
    for a, b in zip(g.intersect_boxes(boxes), o.intersect_boxes(boxes)):
        same(a, b)
    segs = np.concatenate([syn.random_segments(400, lo, hi, seed=2), xy[f[:200, :2]], xy[f[:50, [1, 2]]]])
    for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
        same(a, b)
    # a second mesh for face queries (shifted, so faces straddle tree faces)
    qxy, qf = syn.triangle_mesh(25, seed=9, extent=tuple(hi - lo), offset=tuple(lo + 0.013 * span))
    for a, b in zip(g.intersect_faces(qxy, qf, -1), o.intersect_faces(qxy, qf, -1)):
        same(a, b)
    qf1 = qf.copy()
    qf2 = qf.copy()
    for a, b in zip(g.locate_faces(qxy, qf1), o.locate_faces(qxy, qf2)):
        same(a, b)
    same(qf1, qf2)
    pts = np.concatenate([syn.uniform_points(5000, lo, hi, seed=3, margin=0.02), xy[:300],
                          syn.near_edge_points(xy, f[:, :3], 500, dist=1e-9 * span, seed=4)])
    for a, b in zip(g.compute_barycentric_weights(pts), o.compute_barycentric_weights(pts)):
        same(a, b)
    same(g.node_bounds, o.node_bounds)
    same(g.validate_node_bounds(), o.validate_node_bounds())


def test_edge_tree_matches_oracle(oracle):
    from numba_celltree_gb300 import EdgeCellTree2d

    xy, f = syn.triangle_mesh(60, seed=12)
    e = np.unique(np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1), axis=0)
    for nb, cpl in [(4, 2), (2, 1), (7, 3)]:
        g = EdgeCellTree2d(xy, e, nb, cpl)
        o = oracle.OracleEdgeCellTree2d(xy, e, nb, cpl)
        for fld in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
            same(g.nodes[fld], o.nodes[fld])
        same(g.bb_indices, o.bb_indices)
        pts = np.concatenate([syn.uniform_points(4000, (0, 0), (1, 1), seed=5), xy,
                              0.5 * (xy[e[:, 0]] + xy[e[:, 1]]), 0.3 * xy[e[:, 0]] + 0.7 * xy[e[:, 1]]])
        same(g.locate_points(pts), o.locate_points(pts))
        same(g.locate_points(pts, 1e-3), o.locate_points(pts, 1e-3))
        segs = np.concatenate([syn.random_segments(300, (0, 0), (1, 1), seed=6), xy[e[:100]]])
        for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
            same(a, b)


def test_split_segment_traversal_matches_uncut(oracle):
    """Segment traversals cut into subtree work items (several item sizes,
    down to a few cells, i.e. cuts near the leaves) give the uncut
    traversal's candidates and results, and the oracle's: long and short
    segments, segments missing the mesh, points, NaN and inf endpoints,
    face trees (mode 1) and edge trees (mode 0)."""
    import torch

    from numba_celltree_gb300 import CellTree2d, EdgeCellTree2d

    xy, f = syn.mixed_mesh(70, 60, seed=31, extent=(70.0, 60.0))
    rng = np.random.default_rng(32)
    a0 = rng.uniform((0.0, 0.0), (70.0, 60.0), (600, 2))
    segs = np.concatenate([
        syn.random_segments(300, (-5.0, -5.0), (75.0, 65.0), seed=33),  # long, some leaving the mesh
        np.stack([a0, a0 + rng.uniform(-2, 2, (600, 2))], 1),  # short
        np.array([[[80.0, 80.0], [90.0, 95.0]], [[10.5, 10.5], [10.5, 10.5]], [[0.0, 30.0], [70.0, 30.0]],
                  [[np.nan, 1.0], [3.0, 4.0]], [[1.0, 1.0], [np.inf, 4.0]], [[35.0, -10.0], [35.0, 70.0]]]),
    ])
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    t = g._tree
    sd = torch.as_tensor(segs, device="cuda")
    base = t.locate_edges(sd, 1, {"threads": 128, "work_order": False, "split": 0})
    exp = o.intersect_edges(segs)
    for a, b in zip(base, exp):
        same(a.cpu().numpy(), b)
    # uncut, without the counting pass's scratch, and with a scratch of 2
    # candidates (most segments through the second traversal)
    for spec_max, spec_cap in ((0, 64), (1 << 22, 2)):
        t.SPEC_MAX_SEGMENTS, t.SEG_SPEC_CAP = spec_max, spec_cap
        got = t.locate_edges(sd, 1, {"threads": 64, "work_order": True, "split": 0})
        for a, b in zip(got, base):
            assert teq(a, b), (spec_max, spec_cap)
    del t.SPEC_MAX_SEGMENTS, t.SEG_SPEC_CAP
    counts0 = t.count_edge_candidates(sd, 1)
    for split in (2, 7, 64, 1024):
        cfg = {"threads": 128, "work_order": split == 7, "split": split}
        assert t.edge_cut(cfg) is not None
        got = t.locate_edges(sd, 1, cfg)
        for a, b in zip(got, base):
            assert teq(a, b), split
        _, ccnt, _, items = t.edge_candidate_ranges(sd, 1, None, t.edge_cut(cfg))
        assert items is not None and torch.equal(ccnt, counts0), split
    # work items beyond the device budget: coarser cuts, same results
    from numba_celltree_gb300 import celltree_base

    cfg = {"threads": 128, "work_order": False, "split": 2}
    n_items = t.edge_candidate_ranges(sd, 1, None, t.edge_cut(cfg))[3][2]
    try:
        t.ITEMS_CHECK_MIN = 0
        t.device_budget = lambda b: n_items // 5
        _, _, _, items = t.edge_candidate_ranges(sd, 1, None, t.edge_cut(cfg))
        assert 0 < items[2] <= n_items // 5
        got = t.locate_edges(sd, 1, cfg)
        for a, b in zip(got, base):
            assert teq(a, b)
    finally:
        del t.ITEMS_CHECK_MIN, t.device_budget
    assert t.ITEMS_CHECK_MIN == celltree_base._GpuTree.ITEMS_CHECK_MIN
    # edge tree (edge-edge mode)
    e = np.unique(np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]]]), axis=1), axis=0)
    e = e[(e >= 0).all(1)]
    ge = EdgeCellTree2d(xy, e)
    oe = oracle.OracleEdgeCellTree2d(xy, e)
    te = ge._tree
    base = te.locate_edges(sd, 0, {"threads": 128, "work_order": False, "split": 0})
    for split in (3, 50):
        got = te.locate_edges(sd, 0, {"threads": 64, "work_order": False, "split": split})
        for a, b in zip(got, base):
            assert teq(a, b), split
    for a, b in zip(ge.intersect_edges(segs), oe.intersect_edges(segs)):
        same(a, b)


def test_box_subtree_jobs_match_inline(oracle):
    """Subtrees wholly inside a query box written by one warp per subtree
    after the traversal (ct_write_boxes_ws), and small batches counted and
    written in one traversal with a per-box scratch (ct_count_boxes_spec /
    ct_write_boxes_spec, a scratch of 3 pairs forcing most boxes through the
    second traversal), give the pairs the box's own thread writes in line
    (ct_write_boxes) and the oracle's: big boxes over whole subtrees, small
    ones, boxes beyond the mesh, cells_per_leaf 1-3."""
    import ctypes

    import torch

    from numba_celltree_gb300 import CellTree2d, _device, _lib

    xy, f = syn.mixed_mesh(90, 70, seed=51, extent=(90.0, 70.0))
    boxes = np.concatenate([
        syn.random_boxes(2500, (-5.0, -5.0), (95.0, 75.0), 0.2, 60.0, seed=52, log_uniform=True),
        np.array([[-10.0, 100.0, -10.0, 80.0], [0.0, 90.0, 0.0, 70.0], [40.0, 40.5, 30.0, 30.5]]),
    ])
    bd = torch.as_tensor(boxes, device="cuda")
    for cpl, spec_max, spec_cap in ((1, 0, 64), (2, 0, 64), (3, 0, 64), (2, 1 << 16, 64), (1, 1 << 16, 3), (3, 1, 64)):
        g = CellTree2d(xy, f, -1, 4, cpl)
        t = g._tree
        t.BOX_JOBS_MIN_PAIRS = 0  # the queued path at any size
        t.SPEC_MAX_BOXES = spec_max  # 0: two traversals; else one, with SPEC_CAP pairs kept per box
        t.SPEC_CAP = spec_cap
        ii, jj = t.locate_boxes(bd, {"threads": 256, "work_order": cpl == 2, "job_cells": 8 * cpl})
        n = len(boxes)
        counts = t.count_boxes(bd)
        offsets, total = t.scan(counts)
        assert total == int(ii.shape[0]) and total > 100_000
        i2 = torch.empty_like(ii)
        j2 = torch.empty_like(jj)
        _lib.check(_lib.load().ct_write_boxes(ctypes.byref(t.desc), _device.ptr(bd), n, None, _device.ptr(offsets),
                                              _device.ptr(i2), _device.ptr(j2), _device.stream()), "inline")
        assert torch.equal(ii, i2) and torch.equal(jj, j2), (cpl, spec_max, spec_cap)
        o = oracle.OracleCellTree2d(xy, f, -1, 4, cpl)
        for a, b in zip((ii, jj), o.locate_boxes(boxes)):
            same(a.cpu().numpy(), b)
        for a, b in zip(g.intersect_boxes(boxes[:300]), o.intersect_boxes(boxes[:300])):
            same(a, b)


def test_box_queries_on_grid_lines(oracle):
    """Boxes whose sides lie exactly on cell edges of an unjittered grid (and
    one ulp either side), at a UTM-size offset too: the node-box pruning and
    the inside-subtree shortcut keep upstream's strict overlap test."""
    from numba_celltree_gb300 import CellTree2d

    rng = np.random.default_rng(61)
    for off in ((0.0, 0.0), (5.0e5, 4.2e6)):
        xy, f = syn.triangle_mesh(60, 50, seed=62, extent=(60.0, 50.0), offset=off, jitter=0.0)
        g = CellTree2d(xy, f, -1)
        o = oracle.OracleCellTree2d(xy, f, -1)
        x0 = off[0] + rng.integers(-2, 60, 3000).astype(np.float64)
        y0 = off[1] + rng.integers(-2, 50, 3000).astype(np.float64)
        w = rng.integers(0, 30, 3000).astype(np.float64)
        h = rng.integers(0, 30, 3000).astype(np.float64)
        boxes = np.stack([x0, x0 + w, y0, y0 + h], 1)
        nud = boxes.copy()
        nud[0::2, 0] = np.nextafter(nud[0::2, 0], -np.inf)
        nud[1::2, 1] = np.nextafter(nud[1::2, 1], np.inf)
        nud[0::3, 2] = np.nextafter(nud[0::3, 2], np.inf)
        nud[1::3, 3] = np.nextafter(nud[1::3, 3], -np.inf)
        boxes = np.concatenate([boxes, nud])
        for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
            same(a, b)
        for a, b in zip(g.intersect_boxes(boxes[:1500]), o.intersect_boxes(boxes[:1500])):
            same(a, b)


def _grazing_segments(xy, f, n, seed):
    """Segments that run along cell edges, through vertices, one ulp off
    edges and vertices, axis-aligned on grid lines and nearly parallel to
    edges: where a filter that is not certified would drop a result."""
    rng = np.random.default_rng(seed)
    fi = rng.integers(0, len(f), n)
    v0, v1 = xy[f[fi, 0]], xy[f[fi, 1]]
    span = float((xy.max(0) - xy.min(0)).max())
    d = v1 - v0
    far = xy[f[rng.integers(0, len(f), n), 2]]
    out = [
        np.stack([v0, v1], 1),  # exactly an edge
        np.stack([v0 - 3.0 * d, v1 + 5.0 * d], 1),  # an edge's line, extended over neighbours
        np.stack([np.nextafter(v0, v0 + 1.0), np.nextafter(v1, v1 - 1.0)], 1),  # one ulp off
        np.stack([v0 + np.array([0.0, 1e-12]) * span, v1 + np.array([0.0, -1e-12]) * span], 1),
        np.stack([v0, far], 1),  # vertex to vertex across cells
        np.stack([v0, v0 + (far - v0) * (1.0 + 2.0 ** -40)], 1),  # just past a vertex
        np.stack([v0 - d * 1e6, v0 + np.array([d[:, 1], -d[:, 0]]).T * 1e-9 + d * 1e6], 1),  # nearly parallel
    ]
    ys = xy[rng.integers(0, len(xy), n // 4), 1]
    lo, hi = xy.min(0), xy.max(0)
    out.append(np.stack([np.stack([np.full_like(ys, lo[0] - 1.0), ys], 1),
                         np.stack([np.full_like(ys, hi[0] + 1.0), ys], 1)], 1))  # horizontal on grid lines
    xs = xy[rng.integers(0, len(xy), n // 4), 0]
    out.append(np.stack([np.stack([xs, np.full_like(xs, hi[1] + 1.0)], 1),
                         np.stack([xs, np.full_like(xs, lo[1] - 1.0)], 1)], 1))  # vertical, downwards
    return np.concatenate(out)


@pytest.mark.parametrize("name", ["grid_tri", "utm_tri", "mixed"])
def test_line_filter_keeps_results(oracle, name):
    """The traversal's line filter (nodes and cells whose box the segment's
    line surely misses are skipped) prunes candidates but never a result:
    results with and without it are identical, and equal to the oracle's, on
    segments along and one ulp off cell edges, through vertices, on grid
    lines (an unjittered grid), with UTM-size offsets; edge trees too."""
    import torch

    from numba_celltree_gb300 import CellTree2d, EdgeCellTree2d

    if name == "grid_tri":
        xy, f = syn.triangle_mesh(40, 30, seed=41, extent=(40.0, 30.0), jitter=0.0)
    elif name == "utm_tri":
        xy, f = syn.triangle_mesh(50, 40, seed=42, extent=(50.0, 40.0), offset=(5.0e5, 4.2e6))
    else:
        xy, f = syn.mixed_mesh(50, 40, seed=43, extent=(50.0, 40.0))
    lo, hi = xy.min(0), xy.max(0)
    segs = np.concatenate([_grazing_segments(xy, f, 300, 44),
                           syn.random_segments(200, lo - 1.0, hi + 1.0, seed=45)])
    sd = torch.as_tensor(segs, device="cuda")
    g = CellTree2d(xy, f, -1)
    t = g._tree
    cfg = {"threads": 128, "work_order": False, "split": 0}
    on = t.locate_edges(sd, 1, cfg)
    cnt_on = int(t.count_edge_candidates(sd, 1).sum())
    assert t.desc.bb_leaf32
    keep, t.desc.bb_leaf32 = t.desc.bb_leaf32, None
    try:
        off = t.locate_edges(sd, 1, cfg)
        cnt_off = int(t.count_edge_candidates(sd, 1).sum())
    finally:
        t.desc.bb_leaf32 = keep
    assert cnt_on < cnt_off
    for a, b in zip(on, off):
        assert teq(a, b)
    split = t.locate_edges(sd, 1, {"threads": 64, "work_order": True, "split": 16})
    for a, b in zip(split, on):
        assert teq(a, b)
    exp = oracle.OracleCellTree2d(xy, f, -1).intersect_edges(segs)
    for a, b in zip(on, exp):
        same(a.cpu().numpy(), b)
    # edge tree over the mesh's edges (edge-edge mode, lines_intersect)
    e = np.unique(np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]]]), axis=1), axis=0)
    e = e[(e >= 0).all(1)]
    if name == "utm_tri":
        # the padded box of an axis-aligned edge at this offset has its
        # centroid past the last bucket: upstream's build fails on it (its
        # partition runs out of buckets), and so do the oracle and this build
        from numba_celltree_gb300._lib import CellTreeError

        with pytest.raises(CellTreeError, match="outside every bucket"):
            EdgeCellTree2d(xy, e)
        with pytest.raises(RuntimeError, match="outside every bucket"):
            oracle.OracleEdgeCellTree2d(xy, e)
        return
    ge = EdgeCellTree2d(xy, e)
    te = ge._tree
    on = te.locate_edges(sd, 0, cfg)
    keep, te.desc.bb_leaf32 = te.desc.bb_leaf32, None
    try:
        off = te.locate_edges(sd, 0, cfg)
    finally:
        te.desc.bb_leaf32 = keep
    assert keep
    for a, b in zip(on, off):
        assert teq(a, b)
    for a, b in zip(ge.intersect_edges(segs), oracle.OracleEdgeCellTree2d(xy, e).intersect_edges(segs)):
        same(a, b)


@pytest.mark.parametrize("name", ["grid_tri", "utm_tri", "mixed"])
def test_float32_certificates_are_sound(name):
    """The segment test's float32 certificates against upstream's float64
    Cohen-Sutherland verdict on every (segment, cell) pair the unfiltered
    traversal produces: the interval verdict is undecided or equal, and the
    line filter claims a miss only where the float64 clip rejects.  Random
    and grazing segments (along and one ulp off edges, through vertices, on
    grid lines), UTM-size offsets."""
    import ctypes

    import torch

    from numba_celltree_gb300 import CellTree2d, _device, _lib

    if name == "grid_tri":
        xy, f = syn.triangle_mesh(60, 50, seed=81, extent=(60.0, 50.0), jitter=0.0)
    elif name == "utm_tri":
        xy, f = syn.triangle_mesh(60, 50, seed=82, extent=(60.0, 50.0), offset=(5.0e5, 4.2e6))
    else:
        xy, f = syn.mixed_mesh(60, 50, seed=83, extent=(60.0, 50.0))
    lo, hi = xy.min(0), xy.max(0)
    rng = np.random.default_rng(84)
    a0 = rng.uniform(lo, hi, (20_000, 2))
    segs = np.concatenate([_grazing_segments(xy, f, 2000, 85), syn.random_segments(2000, lo - 1.0, hi + 1.0, seed=86),
                           np.stack([a0, a0 + rng.uniform(-3, 3, (20_000, 2))], 1)])
    sd = torch.as_tensor(segs, device="cuda")
    t = CellTree2d(xy, f, -1)._tree
    t.ensure_box_index()
    lib = _lib.load()
    P, st = _device.ptr, _device.stream()
    keep, t.desc.bb_leaf32 = t.desc.bb_leaf32, None  # candidates of the unfiltered traversal
    try:
        n = len(segs)
        cnt = torch.empty(n, dtype=torch.int64, device="cuda")
        _lib.check(lib.ct_count_edge_candidates(ctypes.byref(t.desc), 1, P(sd), n, None, P(cnt), st), "count")
        off, nc = t.scan(cnt)
        cseg = torch.empty(nc, dtype=torch.int32, device="cuda")
        cpos = torch.empty(nc, dtype=torch.int32, device="cuda")
        _lib.check(lib.ct_write_edge_candidates(ctypes.byref(t.desc), 1, P(sd), n, None, P(off), P(cseg), P(cpos),
                                                st), "write")
    finally:
        t.desc.bb_leaf32 = keep
    assert nc > 500_000
    out = torch.empty((nc, 3), dtype=torch.int8, device="cuda")
    _lib.check(lib.ct_cs_certificates(ctypes.byref(t.desc), P(sd), P(cseg), P(cpos), nc, P(out), st), "cert")
    o = out.cpu().numpy().astype(np.int64)
    f64, f32, miss = o[:, 0], o[:, 1], o[:, 2]
    assert (f64 >= 0).all()
    decided = f32 >= 0
    assert (f32[decided] == f64[decided]).all(), np.nonzero(decided & (f32 != f64))[0][:10]
    assert decided.mean() > 0.8, decided.mean()  # the float32 verdict settles most pairs (grazing ones aside)
    assert (f64[miss == 1] == 0).all()
    assert miss.sum() > 0 and (f64 == 1).sum() > 0


def test_long_segments_sorted(oracle):
    """Segments crossing thousands of cells: the per-segment sort runs in
    global memory (more than 1024 results per segment)."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(300, seed=13)
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    segs = np.array([[[0.0, 0.0], [1.0, 1.0]], [[0.0, 1.0], [1.0, 0.0]], [[0.0, 0.5], [1.0, 0.5]],
                     [[0.5, 0.0], [0.5, 1.0]], [[0.7, 0.7], [0.7, 0.7]]])
    got = g.intersect_edges(segs)
    exp = o.intersect_edges(segs)
    assert np.bincount(got[0]).max() > 1024
    for a, b in zip(got, exp):
        same(a, b)


def test_known_answers():
    """test_celltree.py:333-420, 528-618, 631-639 through the GPU classes."""
    from numba_celltree_gb300 import CellTree2d

    nodes = np.array([[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [2.0, 2.0], [4.0, 0.0], [4.0, 2.0], [6.0, 0.0],
                      [6.0, 2.0], [0.0, 4.0], [2.0, 4.0], [4.0, 4.0], [6.0, 4.0]])
    faces = np.array([[0, 8, 9, 5, 2], [9, 11, 7, 5, -1], [4, 7, 6, -1, -1]], dtype=np.intc)
    t = CellTree2d(nodes, faces, -1, n_buckets=2, cells_per_leaf=1)
    boxes = np.array([[1.0, 2.0, 1.0, 2.0], [4.0, 5.0, 0.0, 1.0], [4.0, 5.0, 2.0, 3.0], [-1.0, 0.0, 0.0, 4.0],
                      [6.0, 8.0, 0.0, 4.0], [0.0, 6.0, -1.0, 0.0], [0.0, 6.0, 4.0, 5.0]])
    i, j = t.locate_boxes(boxes)
    assert np.array_equal(i, [0, 1, 2]) and np.array_equal(j, [0, 2, 1])
    i, j, _ = t.intersect_boxes(boxes)
    assert np.array_equal(i, [0, 1, 2]) and np.array_equal(j, [0, 2, 1])
    edges = np.array([[[1.0, 1.0], [2.0, 2.0]], [[4.0, 3.0], [5.0, 4.0]], [[5.0, 0.0], [6.0, 1.0]],
                      [[-2.0, -1.0], [0.0, 1.0]], [[-2.0, -1.0], [-2.0, -1.0]]])
    i, j, xy = t.intersect_edges(edges)
    assert np.array_equal(i, [0, 1, 2]) and np.array_equal(j, [0, 1, 2]) and np.allclose(xy, edges[:3])
    i, j, xy = t.intersect_edges(edges[:, ::-1])
    assert np.array_equal(i, [0, 1, 2]) and np.allclose(xy, edges[:3, ::-1])
    nodes2 = np.array([[0.0, 0.0], [2.0, 0.0], [1.0, 2.0], [3.0, 2.0]])
    t = CellTree2d(nodes2, np.array([[0, 1, 2], [1, 3, 2]]), -1)
    idx, w = t.compute_barycentric_weights(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 1.0]]))
    assert np.array_equal(idx, [0, 0, 1])
    assert np.allclose(w, [[1.0, 0.0, 0.0], [0.25, 0.25, 0.5], [0.5, 0.25, 0.25]])
    q = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0], [4.0, 0.0], [4.0, 4.0]])
    t = CellTree2d(q, np.array([[0, 1, 2, 3], [1, 4, 5, 2]]), -1)
    idx, w = t.compute_barycentric_weights(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 1.0]]))
    assert np.array_equal(idx, [0, 0, 0])
    assert np.allclose(w, [[1, 0, 0, 0], [0.25, 0.25, 0.25, 0.25], [0, 0.5, 0.5, 0]])
    d = np.load(GOLDEN / "reference_data.npz")
    t = CellTree2d(d["voronoi_xy"], d["voronoi"], -1)
    nbnd = t.node_bounds
    xmin, xmax, ymin, ymax = t.bbox
    assert nbnd.shape == (len(t.nodes), 4)
    assert (nbnd[:, 0] >= xmin).all() and (nbnd[:, 1] <= xmax).all()
    assert (nbnd[:, 2] >= ymin).all() and (nbnd[:, 3] <= ymax).all()
    assert t.validate_node_bounds().all()
    t.nodes[71]["Lmax"] = -0.02319655  # upstream issue #2 (test_celltree.py:613-618)
    assert not t.validate_node_bounds()[73]
    t = CellTree2d(d["xy"], d["triangles"], -1, n_buckets=4)
    dl = t.to_dict_of_lists()
    assert list(dl.keys()) == list(range(len(t.nodes)))
    assert max(len(v) for v in dl.values()) == 2
    centroids = d["xy"][d["triangles"]].mean(axis=1)
    assert np.array_equal(t.locate_points(centroids), np.arange(len(centroids)))


def test_edge_tree_known_answers():
    """test_edgecelltree.py:12-92 through the GPU class."""
    from numba_celltree_gb300 import EdgeCellTree2d

    v = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [2.0, 1.0]])
    e = np.array([[0, 1], [1, 2], [2, 3]], dtype=np.int32)
    t = EdgeCellTree2d(v, e)
    assert t.vertices.shape == (4, 2) and t.edges.shape == (3, 2) and t.nodes.shape == (3,)
    assert t.n_buckets == 4 and t.cells_per_leaf == 2
    assert np.array_equal(t.bb_indices, [0, 1, 2])
    assert np.allclose(t.bb_coords, [[0, 1, 0, 0], [1, 2, 0, 0], [2, 2, 0, 1]], atol=1e-9)
    assert np.allclose(t.bbox, [0.0, 2.0, 0.0, 1.0], atol=1e-9)
    assert np.array_equal(t.locate_points(np.array([[0.5, 0.0], [1.5, 0.0], [2.0, 0.5]])), [0, 1, 2])
    assert np.array_equal(t.locate_points(np.array([[0.5, 0.5], [1.5, 0.5], [2.0, 0.5]])), [-1, -1, 2])
    vv = np.array([[171805.657000002, 563516.366], [171889.594000001, 563437.333000001]])
    t2 = EdgeCellTree2d(vv, np.array([[0, 1]]))
    p = np.array([[171882.49385095935, 563444.0183244612]])
    assert np.array_equal(t2.locate_points(p, tolerance=1e-8), [0])
    assert np.array_equal(t2.locate_points(p, tolerance=1e-9), [0])
    segs = np.array([[[1.0, -1.0], [1.0, 1.0]], [[3.0, 1.0], [-1.0, -1.0]], [[0.0, -1.0], [0.0, 1.0]],
                     [[-2.0, -1.0], [-3.0, -1.0]]])
    i, j, xy = t.intersect_edges(segs)
    assert np.array_equal(i, [0, 1, 1]) and np.array_equal(j, [0, 2, 1])
    assert np.allclose(xy, [[1.0, 0.0], [2.0, 0.5], [1.0, 0.0]], atol=1e-9)


def test_errors_and_casting():
    """test_celltree.py:95-164: casting, shape and bound errors."""
    from numba_celltree_gb300 import CellTree2d

    nodes2 = [[0.0, 0.0], [2.0, 0.0], [1.0, 2.0], [3.0, 2.0]]
    faces2 = [[0, 1, 2], [1, 3, 2]]
    CellTree2d(nodes2, faces2, -1)
    CellTree2d(np.array(nodes2, dtype=np.float32), np.array(faces2, dtype=np.int32), -1)
    t = CellTree2d(np.array(nodes2), np.array([[0, 1, 2, -999], [1, 3, 2, -999]]), -999)
    assert t.faces[0, -1] == -1 and t.faces[1, -1] == -1
    with pytest.raises(ValueError):
        CellTree2d([(1, 2, 3), (3, 4, 5), (4, 5, 6)], faces2, -1)
    with pytest.raises(ValueError):
        CellTree2d(nodes2, [0, 1, 2, 1, 3, 2], -1)
    with pytest.raises(ValueError):
        CellTree2d(np.array(nodes2), np.array(faces2), -1, cells_per_leaf=-1)
    with pytest.raises(ValueError):
        CellTree2d(np.array(nodes2), np.array(faces2), -1, n_buckets=0)
    with pytest.raises(ValueError):
        CellTree2d(np.array(nodes2), np.array([[0, 1, 7], [1, 3, 2]]), -1)  # index out of range
    t = CellTree2d(nodes2, faces2, -1)
    with pytest.raises(ValueError):
        t.locate_points([(1, 2, 3), (3, 4, 5), (4, 5, 6)])
    with pytest.raises(ValueError):
        t.intersect_faces([(1, 2, 3), (3, 4, 5), (4, 5, 6)], faces2, -1)
    with pytest.raises(ValueError):
        t.locate_boxes(np.array([0.0, 1.0, 2.0, 3.0]))
    with pytest.raises(ValueError):
        t.intersect_boxes(np.array([0.0, 1.0, 2.0, 3.0]))
    with pytest.raises(ValueError):
        t.intersect_edges(np.array([[0.0, 1.0], [2.0, 3.0]]))


@pytest.mark.gpu
def test_work_ordered_boxes_and_segments_match_oracle(oracle):
    """Batches large enough to run in work order (heavy-tailed box sizes and
    segment lengths): same pairs, same order as the oracle."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.mixed_mesh(60, 50, seed=8, extent=(60.0, 50.0))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    boxes = syn.random_boxes(20000, (0.0, 0.0), (60.0, 50.0), 0.01, 20.0, seed=2, log_uniform=True)
    for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
        assert np.array_equal(a, b)
    for a, b in zip(g.intersect_boxes(boxes[:6000]), o.intersect_boxes(boxes[:6000])):
        assert np.array_equal(a, b)
    rng = np.random.default_rng(4)
    a0 = rng.uniform(0, 60, (9000, 2))
    ang = rng.uniform(0, 2 * np.pi, 9000)
    ln = np.exp(rng.uniform(np.log(0.01), np.log(40.0), 9000))
    segs = np.stack([a0, a0 + np.stack([ln * np.cos(ang), ln * np.sin(ang)], 1)], 1)
    for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.gpu
def test_output_budgeted_chunks_reassemble_the_full_results(monkeypatch):
    """Multi-result queries in ranges of queries whose results stay within a
    budget (iter_locate_boxes / iter_intersect_boxes / iter_intersect_edges,
    and the automatic ranges of numpy batches that exceed the device memory):
    the concatenated ranges equal the one-pass results, in order."""
    import torch

    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.mixed_mesh(60, 50, seed=8, extent=(60.0, 50.0))
    g = CellTree2d(xy, f, -1)
    boxes = syn.random_boxes(3000, (0.0, 0.0), (60.0, 50.0), 0.01, 20.0, seed=2, log_uniform=True)
    segs = syn.random_segments(700, (0.0, 0.0), (60.0, 50.0), seed=3)  # long segments
    bd, sd = torch.as_tensor(boxes, device="cuda"), torch.as_tensor(segs, device="cuda")
    full = [tuple(x.cpu().numpy() for x in g.locate_boxes(bd)), tuple(x.cpu().numpy() for x in g.intersect_boxes(bd)),
            tuple(x.cpu().numpy() for x in g.intersect_edges(sd))]
    assert len(full[2][0]) > 20000
    for budget in (1, 997, 50_000):
        parts = [list(g.iter_locate_boxes(boxes, budget)), list(g.iter_intersect_boxes(boxes, budget)),
                 list(g.iter_intersect_edges(segs, budget))]
        if budget == 1:
            assert len(parts[0]) == len(boxes) and len(parts[2]) == len(segs)
        for p, ref in zip(parts, full):
            for k in range(len(ref)):
                got = np.concatenate([c[k] for c in p])
                assert np.array_equal(got, ref[k], equal_nan=True)
    # numpy batches beyond the device budget take the ranges automatically
    from numba_celltree_gb300 import celltree_base

    monkeypatch.setattr(celltree_base._GpuTree, "device_budget", lambda self, b: 4096)
    for got, ref in zip((g.locate_boxes(boxes), g.intersect_boxes(boxes), g.intersect_edges(segs)), full):
        for a, b in zip(got, ref):
            assert np.array_equal(a, b, equal_nan=True)
    # empty batches
    for got in (g.locate_boxes(boxes[:0]), g.intersect_edges(segs[:0])):
        assert all(len(x) == 0 for x in got)


def test_segment_sort_sizes_and_ties():
    """sort_intersections_by_edge (geometry_utils.py:564-574) on segments of
    every size class of the sort -- one result, warp sorts of up to 32, 64
    and 128, the block sort in shared and in global memory -- with equal
    distances (stable: candidate order kept) and NaN points (last)."""
    import ctypes

    import torch

    from numba_celltree_gb300 import _device, _lib

    rng = np.random.default_rng(91)
    sizes = [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 500, 1023, 1024, 1025, 3000, 0, 7]
    n = len(sizes)
    segs = rng.uniform(-10, 10, (n, 2, 2))
    counts = np.array(sizes, dtype=np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    total = int(counts.sum())
    ii = np.repeat(np.arange(n), counts).astype(np.int64)
    xy = rng.uniform(-10, 10, (total, 2, 2))
    # ties: repeat some points within segments; NaNs
    rep = rng.choice(total, total // 5, replace=False)
    xy[rep] = xy[np.maximum(rep - 1, 0)]
    xy[rng.choice(total, total // 50, replace=False)] = np.nan
    jj = rng.integers(0, 1 << 40, total).astype(np.int64)
    dev = "cuda"
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    s_d, o_d, c_d, ii_d, jj_d, xy_d = T(segs), T(offsets), T(counts), T(ii), T(jj), T(xy)
    jj2 = torch.empty_like(jj_d)
    xy2 = torch.empty_like(xy_d)
    lib = _lib.load()
    wsz = int(lib.ct_sort_workspace_size(total))
    ws = torch.empty(wsz, dtype=torch.uint8, device=dev)
    P = _device.ptr
    _lib.check(lib.ct_sort_intersections(P(s_d), n, P(o_d), P(c_d), P(ii_d), P(jj_d), P(xy_d), total, P(jj2), P(xy2),
                                         P(ws), wsz, _device.stream()), "sort")
    # expected: per segment, stable order by t = (c - a) . (b - a), NaN last
    a = segs[ii, 0]
    b = segs[ii, 1]
    t = (xy[:, 0, 0] - a[:, 0]) * (b[:, 0] - a[:, 0]) + (xy[:, 0, 1] - a[:, 1]) * (b[:, 1] - a[:, 1])
    tk = np.where(np.isnan(t), np.inf, t)
    nan_last = np.isnan(t).astype(np.int64)
    order = np.lexsort((np.arange(total), tk, nan_last, ii))
    same(jj2.cpu().numpy(), jj[order])
    same(xy2.cpu().numpy(), xy[order])
