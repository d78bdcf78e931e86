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
@pytest.mark.parametrize("device_levels", [True, False])
def test_forest_build_matches_single_builds(oracle, device_levels):
    from numba_celltree_gb300 import CellTree2d, CellTreeBatch

    meshes = _meshes()
    batch = CellTreeBatch(meshes, -1, device_levels=device_levels)
    assert (batch.forest is not None) == device_levels
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


@pytest.mark.gpu
def test_device_driven_forest_build_replays_from_a_graph():
    """ct_build_forest_async (every level on the device, no host
    synchronisation) captured once in a CUDA graph and replayed on moved
    coordinates of meshes of the same sizes: each replay's trees equal the
    meshes built alone."""
    import torch

    from numba_celltree_gb300 import CellTree2d, _device, _lib
    from numba_celltree_gb300.batch import ForestBuild

    def boxes(meshes):
        lib = _lib.load()
        parts = []
        for xy, f in meshes:
            v = torch.as_tensor(xy, device="cuda")
            fd = torch.as_tensor(f, device="cuda").clone()
            bb = torch.empty((len(f), 4), dtype=torch.float64, device="cuda")
            assert lib.ct_counter_clockwise(v.data_ptr(), fd.data_ptr(), len(f), f.shape[1], _device.stream()) == 0
            assert lib.ct_face_bboxes(v.data_ptr(), fd.data_ptr(), len(f), f.shape[1], bb.data_ptr(),
                                      _device.stream()) == 0
            parts.append(bb)
        return torch.cat(parts)

    meshes = _meshes()
    fb = ForestBuild([len(f) for _, f in meshes], torch.device("cuda", 0))
    bb = boxes(meshes)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fb.launch(bb)  # warm-up outside the capture (function attributes, module load)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fb.launch(bb)
    for seed in (11, 12):
        moved = []
        for k, (xy, f) in enumerate(meshes):
            rng = np.random.default_rng(seed * 100 + k)
            moved.append((xy + rng.uniform(-0.05, 0.05, xy.shape), f))
        bb.copy_(boxes(moved))
        g.replay()
        node_off, depth = fb.result()
        for k, (xy, f) in enumerate(moved):
            alone = CellTree2d(xy, f, -1)
            a, b = int(node_off[k]), int(node_off[k + 1])
            assert b - a == len(alone.nodes), (seed, k)
            assert np.array_equal(fb.child[a:b].cpu().numpy(), alone.nodes["child"]), (seed, k)
            assert np.array_equal(fb.Lmax[a:b].cpu().numpy(), alone.nodes["Lmax"]), (seed, k)
            assert np.array_equal(fb.Rmin[a:b].cpu().numpy(), alone.nodes["Rmin"]), (seed, k)
            assert np.array_equal(fb.ptr[a:b].cpu().numpy(), alone.nodes["ptr"]), (seed, k)
            e0, e1 = int(fb.tree_off[k]), int(fb.tree_off[k + 1])
            assert np.array_equal(fb.bb_indices[e0:e1].cpu().numpy(), alone.bb_indices), (seed, k)
            assert depth[k] == alone._tree.max_depth


def test_k_runs_group_consecutive_meshes_of_one_width():
    from numba_celltree_gb300.batch import k_runs

    Ks = [3, 3, 4, 6, 6, 6, 3]
    sizes = np.array([5, 2, 7, 1, 1, 3, 4])
    tree_off = np.concatenate([[0], np.cumsum(sizes)])
    face_off = np.concatenate([[0], np.cumsum(sizes * np.array(Ks))])
    runs = k_runs(Ks, tree_off, face_off)
    assert runs == [(0, 7, 3, 0), (7, 7, 4, 21), (14, 5, 6, 49), (19, 4, 3, 79)]
    assert k_runs([], [0], [0]) == []


@pytest.mark.gpu
def test_forest_pipeline_build_and_locate_replay_from_one_graph(oracle):
    """ForestPipeline: face boxes, tree build, device-side index and batched
    locate of triangle, quad and mixed meshes in one CUDA graph, replayed on
    moved vertices and new points: every mesh's results equal the mesh built
    and queried alone (and the oracle's on the first geometry)."""
    from numba_celltree_gb300 import CellTree2d
    from numba_celltree_gb300.batch import ForestPipeline

    meshes = _meshes()
    pts = _points(meshes)
    counts = [len(p) for p in pts]
    pipe = ForestPipeline(meshes, counts)
    res = pipe.run(np.concatenate([xy for xy, _ in meshes]), np.concatenate(pts)).cpu().numpy()
    assert 0 < pipe.candidate_entries() <= pipe.cand_capacity  # the locate used candidate lists
    for k, (xy, f) in enumerate(meshes):
        a, b = int(pipe.offsets[k]), int(pipe.offsets[k + 1])
        ref = oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k])
        assert np.array_equal(res[a:b], ref), k
    pipe.capture()
    for seed in (11, 12):
        moved = []
        for k, (xy, f) in enumerate(meshes):
            rng = np.random.default_rng(seed * 100 + k)
            moved.append((xy + rng.uniform(-0.05, 0.05, xy.shape), f))
        new = _points(moved, seed=seed)
        new = [p[:c] if len(p) >= c else np.resize(p, (c, 2)) for p, c in zip(new, counts)]
        res = pipe.run(np.concatenate([xy for xy, _ in moved]), np.concatenate(new)).cpu().numpy()
        for k, (xy, f) in enumerate(moved):
            a, b = int(pipe.offsets[k]), int(pipe.offsets[k + 1])
            assert np.array_equal(res[a:b], CellTree2d(xy, f, -1).locate_points(new[k])), (seed, k)


@pytest.mark.gpu
def test_forest_pipeline_without_room_for_candidate_lists(oracle):
    """A candidate-list capacity below the build's entries: the build runs
    the locate without lists, with the same results."""
    from numba_celltree_gb300.batch import ForestPipeline

    meshes = _meshes()[:6]
    pts = _points(meshes, seed=5)
    pipe = ForestPipeline(meshes, [len(p) for p in pts], candidate_entries_per_cell=0.01)
    res = pipe.run(None, np.concatenate(pts)).cpu().numpy()
    assert pipe.candidate_entries() > pipe.cand_capacity
    for k, (xy, f) in enumerate(meshes):
        a, b = int(pipe.offsets[k]), int(pipe.offsets[k + 1])
        assert np.array_equal(res[a:b], oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k])), k


@pytest.mark.gpu
def test_forest_pipeline_given_tolerance_and_empty_mesh_points(oracle):
    """One tolerance for every mesh, and meshes without points."""
    from numba_celltree_gb300.batch import ForestPipeline

    meshes = _meshes()[:5]
    pts = _points(meshes, seed=3)
    pts[1] = pts[1][:0]
    pts[3] = pts[3][:0]
    pipe = ForestPipeline(meshes, [len(p) for p in pts], tolerance=1e-3)
    res = pipe.run(None, np.concatenate(pts)).cpu().numpy()
    for k, (xy, f) in enumerate(meshes):
        a, b = int(pipe.offsets[k]), int(pipe.offsets[k + 1])
        assert np.array_equal(res[a:b], oracle.OracleCellTree2d(xy, f, -1).locate_points(pts[k], 1e-3)), k


@pytest.mark.gpu
def test_batches_of_one_mesh(oracle):
    """A batch holding a single mesh (host-driven and device-driven forest
    builds, the pipeline) equals the mesh built and queried alone: the forest
    layout keeps a per-element tree index even for one tree."""
    import torch

    from numba_celltree_gb300 import CellTree2d, CellTreeBatch
    from numba_celltree_gb300.batch import ForestBuild, ForestPipeline

    xy, f = syn.triangle_mesh(120, 90, seed=21, extent=(120.0, 90.0))
    alone = CellTree2d(xy, f, -1)
    for device_levels in (False, True):
        batch = CellTreeBatch([(xy, f)], -1, device_levels=device_levels)
        assert batch[0].nodes.tobytes() == alone.nodes.tobytes(), device_levels
        assert np.array_equal(batch[0].bb_indices, alone.bb_indices), device_levels
    fb = ForestBuild([len(f)], torch.device("cuda", 0))
    fb.launch(alone._tree.bb_coords)
    node_off, depth = fb.result()
    nn = int(node_off[1])
    assert nn == len(alone.nodes) and depth[0] == alone._tree.max_depth
    assert np.array_equal(fb.child[:nn].cpu().numpy(), alone.nodes["child"])
    assert np.array_equal(fb.bb_indices.cpu().numpy(), alone.bb_indices)
    pts = syn.uniform_points(20_000, xy.min(0), xy.max(0), seed=22, margin=0.02)
    pipe = ForestPipeline([(xy, f)], [len(pts)])
    res = pipe.run(xy, pts).cpu().numpy()
    assert np.array_equal(res, oracle.OracleCellTree2d(xy, f, -1).locate_points(pts))


@pytest.mark.gpu
def test_batch_of_small_meshes_only():
    """Every mesh at most one subtree (128 cells): the level loops have no
    work and the warp subtrees build every tree; both forest builds equal
    the meshes built alone."""
    from numba_celltree_gb300 import CellTree2d, CellTreeBatch

    meshes = [syn.triangle_mesh(nx, ny, seed=30 + nx, extent=(float(nx), float(ny)))
              for nx, ny in [(1, 1), (2, 3), (8, 8), (5, 6), (7, 9)]]
    assert max(len(f) for _, f in meshes) <= 128
    for device_levels in (False, True):
        batch = CellTreeBatch(meshes, -1, device_levels=device_levels)
        for k, (xy, f) in enumerate(meshes):
            alone = CellTree2d(xy, f, -1)
            assert batch[k].nodes.tobytes() == alone.nodes.tobytes(), (device_levels, k)
            assert np.array_equal(batch[k].bb_indices, alone.bb_indices), (device_levels, k)
