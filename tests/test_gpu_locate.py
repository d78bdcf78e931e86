"""locate_points on the GPU (float32 and float64 forms) against the oracle
and the upstream fixtures: identical cell indices."""

import numpy as np
import pytest

from meshes import GOLDEN, meshes
from numba_celltree_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _points(xy, f, n, seed):
    lo, hi = xy.min(0), xy.max(0)
    span = float((hi - lo).max())
    pts = [
        syn.uniform_points(n, lo, hi, seed=seed, margin=0.05),
        xy[np.random.default_rng(seed).integers(0, len(xy), n // 10)],
        syn.near_edge_points(xy, f[:, :3], n // 4, dist=1e-9 * span, seed=seed + 1),
        syn.near_edge_points(xy, f[:, :3], n // 4, dist=1e-6 * span, seed=seed + 2),
        syn.near_edge_points(xy, f[:, :3], n // 8, dist=0.0, seed=seed + 3),
    ]
    return np.concatenate(pts)


@pytest.mark.parametrize("name", list(meshes().keys()))
@pytest.mark.parametrize("precision", ["fp32", "fp32-inline", "fp64"])
def test_locate_matches_oracle(oracle, name, precision):
    from numba_celltree_gb300 import CellTree2d

    xy, f = meshes()[name]
    g = CellTree2d(xy, f, -1)
    g.precision = precision
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = _points(xy, f, 20000, seed=hash(name) % 1000)
    assert np.array_equal(g.locate_points(pts), o.locate_points(pts))
    span = float((xy.max(0) - xy.min(0)).max())
    for tol in (1e-9 * span, 1e-4 * span, 0.0):
        assert np.array_equal(g.locate_points(pts, tol), o.locate_points(pts, tol))


def test_locate_matches_upstream_fixtures():
    from numba_celltree_gb300 import CellTree2d

    G = np.load(GOLDEN / "golden_trees.npz")
    for i in range(int(G["n_cases"])):
        p = f"c{i}_"
        nb, cpl = (int(x) for x in G[p + "params"])
        g = CellTree2d(G[p + "vertices"], G[p + "faces_in"], -1, nb, cpl)
        span = float((G[p + "vertices"].max(0) - G[p + "vertices"].min(0)).max())
        for prec in ("fp32", "fp32-inline", "fp64"):
            g.precision = prec
            assert np.array_equal(g.locate_points(G[p + "points"]), G[p + "locate"]), (i, prec)
            assert np.array_equal(g.locate_points(G[p + "points"], 1e-3 * span), G[p + "locate_tol"]), (i, prec)


def test_locate_utm_precision_stress(oracle):
    """UTM-like offsets (5e5, 4.2e6), 1 m cells, points within 1e-9 m of edges."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(300, seed=21, extent=(300.0, 300.0), offset=(5.0e5, 4.2e6))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    rng = np.random.default_rng(5)
    pts = np.concatenate([
        syn.uniform_points(200000, xy.min(0), xy.max(0), seed=3),
        syn.near_edge_points(xy, f, 50000, dist=1e-9, seed=4),
        syn.near_edge_points(xy, f, 20000, dist=0.0, seed=6),
        xy[rng.integers(0, len(xy), 5000)],
    ])
    ref = o.locate_points(pts)
    for prec in ("fp32", "fp32-inline", "fp64"):
        g.precision = prec
        assert np.array_equal(g.locate_points(pts), ref)
    for bits in (0, 8, 16, 24):
        import torch
        p_d = torch.as_tensor(pts, device="cuda")
        o_d = torch.empty(len(pts), dtype=torch.int64, device="cuda")
        g._tree.locate(p_d, o_d, g.default_tolerance(), "fp32", sort_bits=bits)
        assert np.array_equal(o_d.cpu().numpy(), ref), bits


def test_locate_device_tensors(oracle):
    import torch
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(50, seed=2)
    g = CellTree2d(torch.as_tensor(xy, device="cuda"), torch.as_tensor(f, device="cuda"), -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = syn.uniform_points(5000, (0, 0), (1, 1), seed=1, margin=0.1)
    out = g.locate_points(torch.as_tensor(pts, device="cuda"))
    assert out.is_cuda and out.dtype == torch.int64
    assert np.array_equal(out.cpu().numpy(), o.locate_points(pts))


def test_locate_known_answers():
    """test_celltree.py:167-330 through the GPU classes."""
    from numba_celltree_gb300 import CellTree2d

    nodes2 = np.array([[0.0, 0.0], [2.0, 0.0], [1.0, 2.0], [3.0, 2.0]])
    faces2 = np.array([[0, 1, 2], [1, 3, 2]], dtype=np.intc)
    t = CellTree2d(nodes2, faces2, -1)
    for prec in ("fp32", "fp32-inline", "fp64"):
        t.precision = prec
        assert np.array_equal(t.locate_points(np.array([[1.0, 1.0], [2.0, 1.0], [-1.0, 1.0]])), [0, 1, -1])
        pts = np.array([[-0.09, 0.0], [2.0, 1.0], [-1.0, 1.0]])
        assert np.array_equal(t.locate_points(pts, tolerance=1e-9), [-1, 1, -1])
        assert np.array_equal(t.locate_points(pts, tolerance=1e-1), [0, 1, -1])
    nodes = np.array([[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [2.0, 2.0], [4.0, 0.0], [4.0, 2.0], [6.0, 0.0],
                      [6.0, 2.0], [0.0, 4.0], [2.0, 4.0], [4.0, 4.0], [6.0, 4.0]])
    faces = np.array([[0, 8, 9, 5, 2], [9, 11, 7, 5, -1], [4, 7, 6, -1, -1]], dtype=np.intc)
    t = CellTree2d(nodes, faces, -1, n_buckets=2, cells_per_leaf=1)
    pts = np.array([[-9e-9, 0.0], [2.0, -9e-9], [-9e-9, 1.0], [1.0, -9e-9], [-1.1e-8, 1.0], [1.0, -1.1e-8],
                    [-1.1e-8, 0.0], [2.0, -1.5e-8]])
    for prec in ("fp32", "fp32-inline", "fp64"):
        t.precision = prec
        assert np.array_equal(t.locate_points(np.array([[1.0, 1.0], [5.0, 0.5], [5.0, 3.0], [-1.0, 1.0]])),
                              [0, 2, 1, -1])
        assert np.array_equal(t.locate_points(pts), [-1] * 8)
        assert np.array_equal(t.locate_points(pts, tolerance=1e-8), [0, 0, 0, 0, -1, -1, -1, -1])


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [1000, 4096, 1 << 25])
@pytest.mark.parametrize("pinned", [False, True])
def test_locate_host_pipeline(oracle, monkeypatch, chunk, pinned):
    """Host batches stream through the chunked upload / query / download
    pipeline: ragged last chunk, pageable and pinned inputs, empty input."""
    import torch
    from numba_celltree_gb300 import CellTree2d, _pipeline
    from numba_celltree_gb300 import synthetic as syn

    monkeypatch.setattr(_pipeline, "CHUNK_POINTS", chunk)
    xy, f = syn.triangle_mesh(40, seed=8, extent=(40.0, 40.0), offset=(1.0e3, -2.0e3))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = np.concatenate([
        syn.uniform_points(9000, xy.min(0) - 1.0, xy.max(0) + 1.0, seed=2),
        syn.near_edge_points(xy, f, 1500, dist=0.0, seed=3),
    ])
    if pinned:
        buf = torch.empty(pts.shape, dtype=torch.float64, pin_memory=True)
        buf.numpy()[:] = pts
        pts = buf.numpy()
    ref = o.locate_points(pts)
    got = g.locate_points(pts)
    assert isinstance(got, np.ndarray) and got.dtype == np.int64
    assert np.array_equal(got, ref)
    assert g.locate_points(pts[:0]).shape == (0,)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["writeable", "read_only", "offset_8"])
def test_locate_host_pipeline_registers_pageable_input(oracle, monkeypatch, layout):
    """Pageable host arrays page-locked in place chunk by chunk (every chunk
    on its own pages), read-only arrays, and arrays whose rows cannot start
    on a page boundary (staging copy instead): same results as the oracle;
    the pages are released after each call (a second call registers them
    again)."""
    from numba_celltree_gb300 import CellTree2d, _pipeline
    from numba_celltree_gb300 import synthetic as syn

    monkeypatch.setattr(_pipeline, "CHUNK_POINTS", 5000)
    monkeypatch.setattr(_pipeline, "REGISTER_MIN_BYTES", 0)
    xy, f = syn.triangle_mesh(60, seed=18, extent=(60.0, 60.0), offset=(3.0e5, 6.0e6))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = syn.uniform_points(70_001, xy.min(0) - 1.0, xy.max(0) + 1.0, seed=19)
    if layout == "offset_8":
        raw = np.empty(2 * len(pts) + 1, dtype=np.float64)
        view = raw[1:].reshape(-1, 2) if raw.ctypes.data % 16 == 0 else raw[:-1].reshape(-1, 2)
        view[:] = pts
        assert view.ctypes.data % 16 == 8
        pts = view
    elif layout == "read_only":
        pts = pts.copy()
        pts.setflags(write=False)
    ref = o.locate_points(np.ascontiguousarray(pts))
    for _ in range(2):
        assert np.array_equal(g.locate_points(pts), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("cells_bpsm", [4, 6, 8])
def test_candidate_list_launch_variants(oracle, cells_bpsm):
    """Every launch shape of the candidate-list stage (4, 6 or 8 blocks per
    SM) gives the oracle's indices, on sorted batches with and without the
    bucketed result scatter."""
    import torch
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(150, 100, seed=24, extent=(150.0, 100.0), offset=(4.0e5, 3.0e6))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    t = g._tree
    tol = g.default_tolerance()
    for n in (300_001, (1 << 23) + 77):
        pts = syn.uniform_points(n, xy.min(0) - 0.5, xy.max(0) + 0.5, seed=25)
        pts[::50] = syn.near_edge_points(xy, f, len(pts[::50]), dist=1e-9, seed=26)
        p_d = torch.as_tensor(pts, device="cuda")
        out = torch.empty(n, dtype=torch.int64, device="cuda")
        t.locate(p_d, out, tol, "fp32", config={"sort_bits": 16, "cells_bpsm": cells_bpsm, "fast_bpsm": 16})
        got = out.cpu().numpy()
        sample = np.random.default_rng(27).integers(0, n, 100_000)
        assert np.array_equal(got[sample], o.locate_points(pts[sample]))
        g.precision = "fp64"
        assert np.array_equal(got, g.locate_points(p_d).cpu().numpy())
        g.precision = "fp32"


@pytest.mark.gpu
@pytest.mark.parametrize("density", [0.05, 16.0])
def test_candidate_lists_at_grid_densities(oracle, density):
    """Candidate lists on a coarse grid (many cells per grid cell) and a fine
    one (most cells overlap more grid cells than the counting pass records
    per cell, so the filling pass repeats their geometry): the batched float32
    form gives the oracle's indices, near edges included."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(80, 60, seed=21, extent=(80.0, 60.0), offset=(1.0e5, 2.0e5))
    g = CellTree2d(xy, f, -1)
    g._tree.rebuild_index(density)
    assert g._tree.cand_idx is not None
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = np.concatenate([syn.uniform_points(200_000, xy.min(0) - 0.5, xy.max(0) + 0.5, seed=22),
                          syn.near_edge_points(xy, f, 20_000, dist=1e-9, seed=23)])
    g.precision = "fp32"
    assert np.array_equal(g.locate_points(pts), o.locate_points(pts))
    assert np.array_equal(g.locate_points(pts, 1e-4), o.locate_points(pts, 1e-4))


@pytest.mark.gpu
def test_locate_start_grid_edges(oracle):
    """Queries on the lines of the start-node grid, on the bbox boundary and
    just outside it, and on vertices: same result as the oracle in every
    form; the grid is populated (most cells skip at least the root)."""
    import torch
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(120, 60, seed=17, extent=(120.0, 60.0), offset=(7.5e5, 5.1e6))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    t = g._tree
    gnx, gny = int(t.desc.grid_nx), int(t.desc.grid_ny)
    # about one grid cell per mesh cell (14,400 triangles), nearly square
    assert 13_000 < gnx * gny < 16_000 and abs(gnx - 2 * gny) <= 2
    starts = t.grid_start.cpu().numpy()
    assert (starts > 0).mean() > 0.5
    xmin, xmax, ymin, ymax = [float(v) for v in g.bbox]
    gx = np.linspace(xmin, xmax, gnx + 1)
    gy = np.linspace(ymin, ymax, gny + 1)
    rng = np.random.default_rng(9)
    line_pts = np.concatenate([
        np.stack([rng.choice(gx, 4000), rng.uniform(ymin, ymax, 4000)], 1),
        np.stack([rng.uniform(xmin, xmax, 4000), rng.choice(gy, 4000)], 1),
    ])
    eps = np.array([0.0, 1e-12, -1e-12, 1e-7, -1e-7])
    border = np.concatenate([
        np.stack([xmin + rng.choice(eps, 2000), rng.uniform(ymin, ymax, 2000)], 1),
        np.stack([xmax + rng.choice(eps, 2000), rng.uniform(ymin, ymax, 2000)], 1),
        np.stack([rng.uniform(xmin, xmax, 2000), ymin + rng.choice(eps, 2000)], 1),
        np.stack([rng.uniform(xmin, xmax, 2000), ymax + rng.choice(eps, 2000)], 1),
        np.array([[xmin, ymin], [xmax, ymax], [xmin, ymax], [xmax, ymin]]),
    ])
    pts = np.concatenate([line_pts, border, xy[rng.integers(0, len(xy), 3000)],
                          syn.near_edge_points(xy, f, 4000, dist=0.0, seed=12)])
    ref = o.locate_points(pts)
    for prec in ("fp32", "fp32-inline", "fp64"):
        g.precision = prec
        assert np.array_equal(g.locate_points(pts), ref), prec
    p_d = torch.as_tensor(pts, device="cuda")
    o_d = torch.empty(len(pts), dtype=torch.int64, device="cuda")
    for bits in (0, 8, 16, 24):
        t.locate(p_d, o_d, g.default_tolerance(), "fp32", sort_bits=bits)
        assert np.array_equal(o_d.cpu().numpy(), ref), bits


@pytest.mark.gpu
def test_locate_without_start_grid(oracle):
    """grid_nx = grid_ny = 0 (the state for a degenerate bbox): every query
    starts at the root, same results."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.quad_mesh(50, 30, seed=4)
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = np.concatenate([syn.uniform_points(20000, xy.min(0) - 0.5, xy.max(0) + 0.5, seed=1),
                          syn.near_edge_points(xy, f, 3000, dist=0.0, seed=2)])
    ref = o.locate_points(pts)
    g._tree.desc.grid_nx = 0
    g._tree.desc.grid_ny = 0
    for prec in ("fp32", "fp64"):
        g.precision = prec
        assert np.array_equal(g.locate_points(pts), ref), prec


@pytest.mark.gpu
def test_build_rejects_zero_height_mesh(oracle):
    """Cells on one line: the reference's bucket test cannot place the
    centroids, the oracle raises, and so does the GPU build."""
    from numba_celltree_gb300 import CellTree2d
    from numba_celltree_gb300._lib import CellTreeError

    x = np.arange(20, dtype=np.float64)
    xy = np.stack([x, np.zeros_like(x)], 1)
    f = np.stack([np.arange(18), np.arange(1, 19), np.arange(2, 20)], 1).astype(np.int64)
    with pytest.raises(Exception):
        oracle.OracleCellTree2d(xy, f, -1)
    with pytest.raises(CellTreeError):
        CellTree2d(xy, f, -1)


@pytest.mark.gpu
def test_locate_record_capacity_overflow(oracle):
    """Every query on an edge or vertex: far more uncertain queries than
    candidate records (n/8 + 4096), so most take the float64 overflow pass."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(80, seed=31, extent=(80.0, 80.0), offset=(3.0e5, 6.0e6))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    rng = np.random.default_rng(3)
    pts = np.concatenate([syn.near_edge_points(xy, f, 60000, dist=0.0, seed=5),
                          xy[rng.integers(0, len(xy), 20000)]])
    ref = o.locate_points(pts)
    g.precision = "fp32"
    assert np.array_equal(g.locate_points(pts), ref)


@pytest.mark.gpu
def test_locate_candidate_lists_and_overlaps(oracle):
    """Candidate lists: populated for face trees; overlapping cells (every
    point inside two cells) go through the traversal and keep the
    reference's first hit; a tolerance above the lists' cover uses the
    traversal for every query."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.quad_mesh(40, 30, seed=6, extent=(40.0, 30.0), offset=(2.0e5, 3.0e6))
    g = CellTree2d(xy, f, -1)
    d = g._tree.desc
    assert d.cand_tol > 0 and d.cand_n >= len(f)
    o = oracle.OracleCellTree2d(xy, f, -1)
    pts = np.concatenate([syn.uniform_points(30000, xy.min(0) - 0.3, xy.max(0) + 0.3, seed=8),
                          syn.near_edge_points(xy, f, 5000, dist=1e-9, seed=9)])
    ref = o.locate_points(pts)
    assert np.array_equal(g.locate_points(pts), ref)
    for tol in (d.cand_tol * 0.5, d.cand_tol * 4.0, 1e-3):
        assert np.array_equal(g.locate_points(pts, tol), o.locate_points(pts, tol)), tol
    # two copies of the mesh, the second shifted by half a cell
    xy2 = np.concatenate([xy, xy + [0.5, 0.5]])
    f2 = np.concatenate([f, f + len(xy)])
    g2 = CellTree2d(xy2, f2, -1)
    o2 = oracle.OracleCellTree2d(xy2, f2, -1)
    assert np.array_equal(g2.locate_points(pts), o2.locate_points(pts))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [65537, 70001, 100002, 1_000_003, 3_061_726])
def test_locate_sorted_batch_sizes_not_multiple_of_4(oracle, n):
    """Sorted batches (>= 2^16 queries) of every residue mod 4, including many
    queries per cell: the radix sort's per-block histograms must match its
    scatter exactly."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(41, 20, seed=3, extent=(41.0, 20.0), offset=(-4765.3, 1431.0))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    lo, hi = xy.min(0), xy.max(0)
    pts = syn.uniform_points(n, lo - 0.5 * (hi - lo), hi + 0.5 * (hi - lo), seed=n)
    assert np.array_equal(g.locate_points(pts), o.locate_points(pts))


def _awkward_cells(kind, seed=21):
    """A jittered mesh plus awkward cells on top of it: collinear cells,
    repeated vertices, slivers 1e-7 m thin, cells much larger and much
    smaller than a grid cell, and (quads) non-convex darts."""
    rng = np.random.default_rng(seed)
    off = np.array([3.1e5, 5.2e6])
    if kind == "tri":
        xy, f = syn.triangle_mesh(60, 40, seed=11, extent=(60.0, 40.0), offset=tuple(off))
    else:
        xy, f = syn.quad_mesh(60, 40, seed=11, extent=(60.0, 40.0), offset=tuple(off))
    K = f.shape[1]
    verts, faces = [xy], [f]
    base = len(xy)

    def add(polys):
        nonlocal base
        polys = np.asarray(polys, dtype=np.float64)  # (m, k, 2)
        m, k = polys.shape[:2]
        idx = base + np.arange(m * k).reshape(m, k)
        row = np.full((m, K), -1, dtype=np.int64)
        row[:, :k] = idx
        verts.append(polys.reshape(-1, 2))
        faces.append(row)
        base += m * k

    def pts(m, lo=(0.0, 0.0), hi=(60.0, 40.0)):
        return off + rng.uniform(lo, hi, (m, 2))

    p, d = pts(150), rng.normal(0.0, 1.0, (150, 2))
    add(np.stack([p, p + d, p + 2.0 * d], 1))                  # collinear
    a, b = pts(150), pts(150, (-1.0, -1.0), (1.0, 1.0)) - off
    add(np.stack([a, a, a + b], 1))                           # repeated vertex
    n_ = np.stack([-b[:, 1], b[:, 0]], 1) / np.linalg.norm(b, axis=1)[:, None]
    add(np.stack([a, a + b, a + 0.5 * b + 1e-7 * n_], 1))     # sliver
    c = pts(12, (10.0, 10.0), (50.0, 30.0))
    add(np.stack([c, c + [25.0, 3.0], c + [-4.0, 18.0]], 1))  # large, over many grid cells
    c = pts(150)
    add(np.stack([c, c + [1e-3, 0.0], c + [0.0, 1e-3]], 1))   # tiny
    if kind == "quad":
        c = pts(150)
        add(np.stack([c, c + [2.0, 0.0], c + [0.4, 0.4], c + [0.0, 2.0]], 1))  # non-convex darts
        c = pts(100)
        add(np.stack([c, c + [1.0, 0.2], c + [1.0, 0.2], c + [0.3, 1.1]], 1))  # repeated vertex
    return np.concatenate(verts), np.concatenate(faces)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tri", "quad"])
def test_locate_clipped_lists_awkward_cells(oracle, kind):
    """Candidate entries clipped to their grid cell: degenerate, thin, large,
    tiny and non-convex cells over a regular mesh, queries on edges (at 0 and
    1e-12 m), vertices and grid lines -- the batched float32 form gives the
    oracle's indices."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = _awkward_cells(kind)
    g = CellTree2d(xy, f, -1)
    d = g._tree.desc
    assert d.cand_tol > 0 and int(d.grid_nx) > 0
    o = oracle.OracleCellTree2d(xy, f, -1)
    xmin, xmax, ymin, ymax = [float(v) for v in g.bbox]
    rng = np.random.default_rng(3)
    gx = xmin + (xmax - xmin) * np.arange(int(d.grid_nx) + 1) / int(d.grid_nx)
    gy = ymin + (ymax - ymin) * np.arange(int(d.grid_ny) + 1) / int(d.grid_ny)
    tri_rows = np.where((f[:, :3] >= 0).all(1))[0]
    fe = f[tri_rows][:, :3]
    pts = np.concatenate([
        syn.uniform_points(120_000, (xmin - 1.0, ymin - 1.0), (xmax + 1.0, ymax + 1.0), seed=4),
        syn.near_edge_points(xy, fe, 20_000, dist=0.0, seed=5),
        syn.near_edge_points(xy, fe, 20_000, dist=1e-12, seed=6),
        xy[rng.integers(0, len(xy), 5000)],
        np.stack([rng.choice(gx, 5000), rng.uniform(ymin, ymax, 5000)], 1),
        np.stack([rng.uniform(xmin, xmax, 5000), rng.choice(gy, 5000)], 1),
    ])
    assert np.array_equal(g.locate_points(pts), o.locate_points(pts))
