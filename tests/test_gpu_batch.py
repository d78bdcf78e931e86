"""Batched build and locate of many meshes (CellTreeBatch): every mesh's tree
and every query result equal those of the mesh built and queried alone (and
the oracle's); the batched locate replays from a CUDA graph."""

import numpy as np
import pytest

from numba_celltree_gb300 import synthetic as syn


def _meshes():
    out = []
    rng = np.random.default_rng(0)
    sizes = [(1, 1), (5, 4), (8, 8), (30, 20), (70, 50), (150, 110), (3, 2), (200, 120)]
    for k, (nx, ny) in enumerate(sizes):
        off = (rng.uniform(-1e3, 1e3), rng.uniform(-1e3, 1e3))
        if k % 3 == 0:
            xy, f = syn.triangle_mesh(nx, ny, seed=k, extent=(float(nx), float(ny)), offset=off)
        elif k % 3 == 1:
            xy, f = syn.quad_mesh(nx, ny, seed=k, extent=(float(nx), float(ny)), offset=off)
        else:
            xy, f = syn.mixed_mesh(nx, ny, seed=k, extent=(float(nx), float(ny)))
            xy = xy + np.array(off)
        out.append((xy, f))
    return out


def _points(meshes, seed=1):
    pts = []
    for k, (xy, f) in enumerate(meshes):
        lo, hi = xy.min(0), xy.max(0)
        m = 500 + 300 * k
        pts.append(np.concatenate([
            syn.uniform_points(m, lo - 0.5, hi + 0.5, seed=seed + k),
            syn.near_edge_points(xy, f, m // 5, dist=0.0, seed=seed + 100 + k),
            xy[np.random.default_rng(k).integers(0, len(xy), 20)],
        ]))
    return pts


@pytest.mark.gpu
def test_forest_build_matches_single_builds(oracle):
    from numba_celltree_gb300 import CellTree2d, CellTreeBatch

    meshes = _meshes()
    batch = CellTreeBatch(meshes, -1)
    assert len(batch) == len(meshes)
    for k, (xy, f) in enumerate(meshes):
        alone = CellTree2d(xy, f, -1)
        t = batch[k]
        assert np.array_equal(t.bb_indices, alone.bb_indices), k
        assert t.nodes.tobytes() == alone.nodes.tobytes(), k
        assert np.array_equal(t.faces, alone.faces), k
        if k in (0, 3, 5):
            o = oracle.OracleCellTree2d(xy, f, -1)
            assert np.array_equal(t.bb_indices, o.bb_indices)
            assert t.nodes.tobytes() == o.nodes.tobytes()


@pytest.mark.gpu
def test_forest_locate_matches_single_locate(oracle):
    from numba_celltree_gb300 import CellTreeBatch

    meshes = _meshes()
    batch = CellTreeBatch(meshes, -1)
    pts = _points(meshes)
    got = batch.locate_points(pts)
    for k, (xy, f) in enumerate(meshes):
        ref = oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k])
        assert np.array_equal(got[k], ref), k
        assert np.array_equal(batch[k].locate_points(pts[k]), ref), k
    # one tolerance for all meshes, above the candidate lists' cover
    got = batch.locate_points(pts, tolerance=1e-3)
    for k, (xy, f) in enumerate(meshes):
        ref = oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k], 1e-3)
        assert np.array_equal(got[k], ref), k


@pytest.mark.gpu
def test_forest_locate_cuda_graph():
    import torch
    from numba_celltree_gb300 import CellTreeBatch

    meshes = _meshes()
    batch = CellTreeBatch(meshes, -1)
    pts = _points(meshes, seed=7)
    counts = [len(p) for p in pts]
    plan = batch.plan_locate(counts)
    pts_d = torch.as_tensor(np.concatenate(pts), device="cuda")
    out = torch.empty(plan.n_points, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.launch(pts_d, out)  # warm-up outside capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.launch(pts_d, out)
    for seed in (11, 12):
        new = _points(meshes, seed=seed)
        new = [p[:c] if len(p) >= c else np.resize(p, (c, 2)) for p, c in zip(new, counts)]
        pts_d.copy_(torch.as_tensor(np.concatenate(new)))
        out.fill_(-7)
        g.replay()
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        for k in range(len(meshes)):
            a, b = int(plan.offsets[k]), int(plan.offsets[k + 1])
            assert np.array_equal(res[a:b], batch[k].locate_points(new[k])), (seed, k)


@pytest.mark.gpu
def test_forest_locate_odd_total(oracle):
    """Batched locate with a sorted total that is not a multiple of 4 and
    meshes with many queries per cell."""
    from numba_celltree_gb300 import CellTreeBatch

    meshes = [syn.triangle_mesh(41, 20, seed=3, extent=(41.0, 20.0), offset=(-4765.3, 1431.0)),
              syn.quad_mesh(7, 5, seed=4, extent=(7.0, 5.0), offset=(30.0, -40.0)),
              syn.triangle_mesh(90, 60, seed=5, extent=(90.0, 60.0))]
    counts = [70001, 3, 100002]
    pts = []
    for (xy, f), m in zip(meshes, counts):
        lo, hi = xy.min(0), xy.max(0)
        pts.append(syn.uniform_points(m, lo - 0.5 * (hi - lo), hi + 0.5 * (hi - lo), seed=m))
    batch = CellTreeBatch(meshes, -1)
    got = batch.locate_points(pts)
    for k, (xy, f) in enumerate(meshes):
        assert np.array_equal(got[k], oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k])), k


@pytest.mark.gpu
def test_result_scatter_above_threshold(oracle):
    """More than 2^23 queries on one tree take the sorted-result path with the
    bucketed scatter (single tree and batch): identical to the float64 form
    on every point and to the oracle on a sample; the batch's large mesh
    gives the same indices as the mesh queried alone."""
    import torch
    from numba_celltree_gb300 import CellTree2d, CellTreeBatch

    n = (1 << 23) + 12345
    xy, f = syn.triangle_mesh(300, 200, seed=3, extent=(300.0, 200.0), offset=(2.5e5, 6.1e6))
    lo, hi = xy.min(0), xy.max(0)
    pts = np.concatenate([syn.uniform_points(n - 40000, lo - 1.0, hi + 1.0, seed=5),
                          syn.near_edge_points(xy, f, 40000, dist=0.0, seed=6)])
    p_d = torch.as_tensor(pts, device="cuda")
    g = CellTree2d(xy, f, -1)
    r32 = g.locate_points(p_d)
    g.precision = "fp64"
    r64 = g.locate_points(p_d)
    assert torch.equal(r32, r64)
    g.precision = "fp32"
    # numpy input: the host pipeline (one chunk above the threshold)
    assert np.array_equal(g.locate_points(pts), r32.cpu().numpy())
    o = oracle.OracleCellTree2d(xy, f, -1)
    sample = np.random.default_rng(7).integers(0, n, 200_000)
    assert np.array_equal(r32.cpu().numpy()[sample], o.locate_points(pts[sample]))
    # batch: the large mesh plus two small ones
    small = _meshes()[:2]
    meshes = [(xy, f)] + small
    qs = [pts] + _points(small)
    batch = CellTreeBatch(meshes)
    res = batch.locate_points(qs)
    assert np.array_equal(res[0], r32.cpu().numpy())
    for k in (1, 2):
        alone = CellTree2d(*meshes[k], -1)
        assert np.array_equal(res[k], alone.locate_points(qs[k]))
