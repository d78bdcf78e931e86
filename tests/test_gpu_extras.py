"""Tree serialisation, the two exported helpers as batched kernels, and the
regridding step (CSR weights from intersection pairs, area-weighted mean)."""

import numpy as np
import pytest

from numba_celltree_gb300 import synthetic as syn


@pytest.mark.gpu
def test_save_load_roundtrip(tmp_path, oracle):
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.mixed_mesh(30, 25, seed=3, extent=(30.0, 25.0))
    g = CellTree2d(xy, f, -1, n_buckets=6, cells_per_leaf=3)
    path = tmp_path / "tree.npz"
    g.save(path)
    h = CellTree2d.load(path)
    assert h.nodes.tobytes() == g.nodes.tobytes()
    assert np.array_equal(h.bb_indices, g.bb_indices)
    assert np.array_equal(h.faces, g.faces)
    assert (h.n_buckets, h.cells_per_leaf) == (6, 3)
    pts = np.concatenate([syn.uniform_points(20000, xy.min(0) - 0.2, xy.max(0) + 0.2, seed=1),
                          syn.near_edge_points(xy, f, 3000, dist=0.0, seed=2)])
    ref = oracle.OracleCellTree2d(xy, f, -1, n_buckets=6, cells_per_leaf=3).locate_points(pts)
    assert np.array_equal(h.locate_points(pts), ref)
    # from the upstream CellTreeData layout (here: the oracle's)
    o = oracle.OracleCellTree2d(xy, f, -1)
    k = CellTree2d.from_celltree_data(o.celltree_data)
    assert k.nodes.tobytes() == o.nodes.tobytes()
    assert np.array_equal(k.locate_points(pts), o.locate_points(pts))


@pytest.mark.gpu
def test_load_rejects_corrupt_nodes(tmp_path):
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(10, seed=1)
    g = CellTree2d(xy, f, -1)
    nodes = g.nodes.copy()
    nodes["child"][0] = 0  # a node that is its own child
    with pytest.raises(ValueError):
        CellTree2d._from_arrays(g.vertices, g.faces, nodes, g.bb_indices, 4, 2)
    bad = g.bb_indices.copy()
    bad[0] = bad[1]
    with pytest.raises(ValueError):
        CellTree2d._from_arrays(g.vertices, g.faces, g.nodes, bad, 4, 2)


@pytest.mark.gpu
def test_liang_barsky_batch_matches_oracle(oracle):
    from numba_celltree_gb300 import algorithms

    rng = np.random.default_rng(0)
    n = 20000
    a = rng.uniform(-2, 3, (n, 2))
    b = rng.uniform(-2, 3, (n, 2))
    b[::50] = a[::50]                      # zero-length
    b[1::50, 0] = a[1::50, 0]              # vertical
    b[2::50, 1] = a[2::50, 1]              # horizontal
    lo = rng.uniform(-1, 1, (n, 2))
    boxes = np.stack([lo[:, 0], lo[:, 0] + rng.uniform(0, 2, n), lo[:, 1], lo[:, 1] + rng.uniform(0, 2, n)], 1)
    ok, c, d = algorithms.liang_barsky_line_box_clip_batch(a, b, boxes)
    for i in range(0, n, 97):
        r = oracle.liang_barsky_line_box_clip(a[i], b[i], boxes[i])
        assert bool(ok[i]) == r[0]
        np.testing.assert_array_equal(c[i], np.array(r[1]))
        np.testing.assert_array_equal(d[i], np.array(r[2]))
    one = algorithms.liang_barsky_line_box_clip((0.0, 0.5), (2.0, 0.5), (0.5, 1.5, 0.0, 1.0))
    assert one[0] and one[1] == (0.5, 0.5) and one[2] == (1.5, 0.5)


@pytest.mark.gpu
def test_points_in_triangles_matches_oracle(oracle):
    from numba_celltree_gb300 import algorithms

    xy, f = syn.triangle_mesh(30, seed=4)
    rng = np.random.default_rng(1)
    n = 30000
    fi = rng.integers(0, len(f), n)
    tri = xy[f[fi]]
    w = rng.dirichlet([1, 1, 1], n) * 1.2 - 0.1   # some outside
    pts = np.einsum("nk,nkd->nd", w, tri)
    pts[::7] = xy[f[fi[::7], 0]]                   # on vertices
    got = algorithms.points_in_triangles(pts, fi, f, xy, 1e-12)
    ref = oracle.points_in_triangles(pts, fi, f, xy, 1e-12)
    assert np.array_equal(got, ref)
    with pytest.raises(IndexError):
        algorithms.points_in_triangles(pts[:3], np.array([0, len(f), 1]), f, xy, 1e-12)


@pytest.mark.gpu
def test_regrid_weighted_mean_matches_dense():
    """The example's dense weight matrix and area-weighted mean, sparse on
    the GPU (examples/spatial_indexing_2d_grids.py:245-313)."""
    from numba_celltree_gb300 import CellTree2d
    from numba_celltree_gb300.regrid import WeightMatrix

    xy, f = syn.triangle_mesh(12, seed=5, extent=(10.0, 10.0))
    tree = CellTree2d(xy, f, -1)
    dx, dy = 1.0, -1.0
    y, x = np.meshgrid(np.arange(10.0, 0.0 + dy, dy), np.arange(0.0, 10.0 + dx, dx), indexing="ij")
    ny, nx = y.shape[0] - 1, x.shape[1] - 1
    coords = np.column_stack([a.ravel() for a in [x[:-1, :-1], x[1:, 1:], y[1:, 1:], y[:-1, :-1]]])
    ri, ci, area = tree.intersect_boxes(coords)
    dense = np.zeros((ny * nx, len(f)))
    dense[ri, ci] = area
    cx, cy = xy[f].mean(axis=1).T
    z = np.sin(0.6 * cx + 2) + np.sin(0.2 * cy)
    wsum = dense @ np.ones(len(f))
    ref = np.full(ny * nx, np.nan)
    ok = wsum > 0
    ref[ok] = (dense @ z)[ok] / wsum[ok]
    W = WeightMatrix.from_intersections(ri, ci, area, ny * nx, len(f))
    got = W.mean(z)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, equal_nan=True)
    np.testing.assert_allclose(W.weight_sum.cpu().numpy(), wsum, rtol=1e-12)
    assert (W.to_scipy().toarray() == dense).all()
    # face-to-face: the query-major pairs of intersect_faces
    qxy, qf = syn.quad_mesh(7, seed=6, extent=(10.0, 10.0), rotate_deg=5.0)
    i, j, a = tree.intersect_faces(qxy, qf, -1)
    W2 = WeightMatrix.from_intersections(i, j, a, len(qf), len(f))
    d2 = np.zeros((len(qf), len(f)))
    d2[i, j] = a
    s2 = d2.sum(1)
    r2 = np.full(len(qf), np.nan)
    r2[s2 > 0] = (d2 @ z)[s2 > 0] / s2[s2 > 0]
    np.testing.assert_allclose(W2.mean(z), r2, rtol=1e-12, equal_nan=True)
    with pytest.raises(ValueError):
        WeightMatrix.from_intersections(i[::-1], j, a, len(qf), len(f))


@pytest.mark.gpu
def test_shared_reduction_calls_from_two_threads():
    """ct_validate_elements (like ct_bbox_summary, ct_vertex_extent and
    ct_pack_tree) uses a small reduction array inside the library: two host
    threads calling it at once on their own streams, one with an index out of
    range and one with valid faces, must each get their own verdict."""
    import ctypes
    import threading

    import torch

    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    xy, f = syn.triangle_mesh(300, seed=7)  # 180,000 faces
    good = torch.as_tensor(f, device="cuda")
    bad = good.clone()
    bad[-1, 2] = xy.shape[0]  # one index past the vertex array
    results = {"good": [], "bad": []}

    def worker(name, faces):
        torch.cuda.set_device(0)
        s = torch.cuda.Stream()
        flag = ctypes.c_int32(-1)
        for _ in range(40):
            assert lib.ct_validate_elements(faces.data_ptr(), faces.shape[0], 3, 3, xy.shape[0],
                                            ctypes.byref(flag), s.cuda_stream) == 0
            results[name].append(flag.value)

    th = [threading.Thread(target=worker, args=(k, t)) for k, t in (("good", good), ("bad", bad))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert results["good"] == [0] * 40
    assert results["bad"] == [1] * 40


def _degenerate_polygons(rng, n, K, grid):
    """n polygons of up to K vertices on a coarse grid (so vertices fall
    exactly on other polygons' edge lines), with repeated consecutive
    vertices, collinear runs and non-convex shapes; -1 padded."""
    out = np.full((n, K), -1, dtype=np.int64)
    for i in range(n):
        m = int(rng.integers(3, K + 1))
        idx = rng.integers(0, grid * grid, size=m)
        if rng.random() < 0.3:  # a repeated consecutive vertex
            k = int(rng.integers(1, m))
            idx[k] = idx[k - 1]
        out[i, :m] = idx
    return out


@pytest.mark.gpu
def test_pair_areas_on_degenerate_polygons_match_oracle(oracle):
    """ct_area_of_intersection / ct_box_area_of_intersection (the converged
    Sutherland-Hodgman clip) against the oracle's sequential clip, bit for
    bit, on polygons built to hit the clip's edge cases: vertices on clip
    lines, zero-length edges, collinear and parallel edges, non-convex
    subjects, clippers of either orientation, empty overlaps."""
    import ctypes

    import torch

    from numba_celltree_gb300 import _device, _lib

    lib = _lib.load()
    O = oracle
    rng = np.random.default_rng(81)
    for grid, scale, K in ((5, 1.0, 4), (7, 1.0 / 3.0, 6), (4, 1e3, 5), (9, 0.1, 8)):
        g = np.arange(grid, dtype=np.float64) * scale
        xy = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2) + 0.25 * scale
        fa = _degenerate_polygons(rng, 400, K, grid)
        fb = _degenerate_polygons(rng, 400, K, grid)
        ia = rng.integers(0, 400, 20000).astype(np.int64)
        ib = rng.integers(0, 400, 20000).astype(np.int64)
        exp = np.empty(len(ia))
        O.lib().cto_area_of_intersection(xy.ctypes.data, xy.ctypes.data, fa.ctypes.data, K, fb.ctypes.data, K,
                                         ia.ctypes.data, ib.ctypes.data, len(ia), exp.ctypes.data)
        d = {k: torch.as_tensor(v, device="cuda") for k, v in
             dict(xy=xy, fa=fa, fb=fb, ia=ia, ib=ib).items()}
        got = torch.empty(len(ia), dtype=torch.float64, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        P = _device.ptr
        assert lib.ct_area_of_intersection(P(d["xy"]), P(d["fa"]), K, P(d["xy"]), P(d["fb"]), K, P(d["ia"]),
                                           P(d["ib"]), len(ia), P(got), P(err), _device.stream()) == 0
        assert np.array_equal(got.cpu().numpy(), exp, equal_nan=True), grid
        # polygons_intersect (the float32-filtered separating-axis test):
        # grid polygons touch exactly along edges and at vertices
        exp_sat = np.empty(len(ia), dtype=np.uint8)
        O.lib().cto_polygons_intersect(xy.ctypes.data, xy.ctypes.data, fa.ctypes.data, K, fb.ctypes.data, K,
                                       ia.ctypes.data, ib.ctypes.data, len(ia), exp_sat.ctypes.data)
        sat = torch.empty(len(ia), dtype=torch.uint8, device="cuda")
        assert lib.ct_polygons_intersect(P(d["xy"]), P(d["fa"]), K, P(d["xy"]), P(d["fb"]), K, P(d["ia"]),
                                         P(d["ib"]), len(ia), P(sat), _device.stream()) == 0
        assert np.array_equal(sat.cpu().numpy(), exp_sat), grid
        # boxes as subjects
        lo = rng.integers(0, grid, size=(3000, 2)) * scale + 0.25 * scale
        hi = lo + rng.integers(0, 3, size=(3000, 2)) * scale
        boxes = np.stack([lo[:, 0], hi[:, 0], lo[:, 1], hi[:, 1]], 1)
        ibx = rng.integers(0, 3000, 20000).astype(np.int64)
        exp = np.empty(len(ibx))
        O.lib().cto_box_area_of_intersection(boxes.ctypes.data, xy.ctypes.data, fb.ctypes.data, K, ibx.ctypes.data,
                                             ib.ctypes.data, len(ibx), exp.ctypes.data)
        bd, ibd = torch.as_tensor(boxes, device="cuda"), torch.as_tensor(ibx, device="cuda")
        assert lib.ct_box_area_of_intersection(P(bd), P(d["xy"]), P(d["fb"]), K, P(ibd), P(d["ib"]), len(ibx),
                                               P(got), P(err), _device.stream()) == 0
        assert np.array_equal(got.cpu().numpy(), exp, equal_nan=True), grid
        assert int(err.item()) == 0
    del ctypes


@pytest.mark.gpu
def test_edge_tree_save_load_roundtrip(tmp_path, oracle):
    """EdgeCellTree2d.save / load / from_celltree_data: same nodes, same
    answers, no rebuild."""
    from numba_celltree_gb300 import EdgeCellTree2d

    rng = np.random.default_rng(31)
    xy = rng.uniform(0.0, 50.0, (400, 2))
    edges = rng.integers(0, 400, (900, 2))
    edges = edges[edges[:, 0] != edges[:, 1]]
    g = EdgeCellTree2d(xy, edges, n_buckets=5, cells_per_leaf=3)
    path = tmp_path / "edges.npz"
    g.save(path)
    h = EdgeCellTree2d.load(path)
    assert h.nodes.tobytes() == g.nodes.tobytes()
    assert np.array_equal(h.bb_indices, g.bb_indices)
    assert (h.n_buckets, h.cells_per_leaf) == (5, 3)
    pts = np.concatenate([rng.uniform(0.0, 50.0, (5000, 2)), xy[edges[:300, 0]]])
    segs = np.stack([rng.uniform(0.0, 50.0, (500, 2)), rng.uniform(0.0, 50.0, (500, 2))], 1)
    assert np.array_equal(h.locate_points(pts), g.locate_points(pts))
    for a, b in zip(h.intersect_edges(segs), g.intersect_edges(segs)):
        assert np.array_equal(a, b, equal_nan=True)
    o = oracle.OracleEdgeCellTree2d(xy, edges)
    k = EdgeCellTree2d.from_celltree_data(o.celltree_data)
    assert k.nodes.tobytes() == o.nodes.tobytes()
    assert np.array_equal(k.locate_points(pts), o.locate_points(pts))
    with pytest.raises(ValueError):
        from numba_celltree_gb300 import CellTree2d

        CellTree2d.load(path)  # not a face tree
