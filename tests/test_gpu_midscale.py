"""Parity at mid scale: sizes between the small fixture meshes and the
16M-cell benchmark mesh, each still checked in seconds.

* a 1,002,528-cell triangle mesh: ``nodes`` / ``bb_indices`` of the GPU build
  and 2M located points (1 % within 1e-9 of an edge or vertex) equal the
  oracle's, in every point-location form;
* the conservative-regridding shape at a tenth of its size (100k jittered
  triangles queried against 50k quads rotated 7 degrees, offset 0.37 cell)
  plus boxes and segments on a mixed polygon mesh: every query equals the
  oracle's (indices in the same order, float outputs bit for bit);
* the adjoint of the area of intersection on that mesh pair: central finite
  differences (h = 1e-6) at 1,000 sampled pairs, and the barycentric-weight
  adjoint at 1,000 sampled points.
"""

import numpy as np
import pytest

from numba_celltree_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.array_equal(a, b, equal_nan=(a.dtype.kind == "f"))


def test_million_cell_build_and_locate_match_oracle(oracle):
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(708, seed=61, extent=(708.0, 708.0), offset=(3.1e5, 5.7e6))
    assert len(f) == 1_002_528
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    for fld in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        same(g.nodes[fld], o.nodes[fld])
    same(g.bb_indices, o.bb_indices)
    pts = syn.uniform_points(2_000_000, xy.min(0), xy.max(0), seed=62, margin=0.01)
    pts[::100] = syn.near_edge_points(xy, f, len(pts[::100]), dist=1e-9, seed=63)
    expected = o.locate_points(pts)
    for prec in ("fp32", "fp32-inline", "fp64"):
        g.precision = prec
        same(g.locate_points(pts), expected)


@pytest.fixture(scope="module")
def regrid_pair():
    """Tree: 50k quads rotated 7 degrees, offset 0.37 cell; query: 100k jittered
    triangles on the same [0, 31.6] x [0, 15.8] extent."""
    from numba_celltree_gb300 import CellTree2d
    from oracle import oracle as O

    O.build()
    txy, tf = syn.quad_mesh(316, 158, seed=64, extent=(31.6, 15.8), offset=(0.037, 0.037), rotate_deg=7.0)
    qxy, qf = syn.triangle_mesh(316, 158, seed=65, extent=(31.6, 15.8))
    return txy, tf, qxy, qf, CellTree2d(txy, tf, -1), O.OracleCellTree2d(txy, tf, -1)


def test_regrid_shape_every_query_matches_oracle(regrid_pair):
    txy, tf, qxy, qf, g, o = regrid_pair
    for a, b in zip(g.intersect_faces(qxy, qf, -1), o.intersect_faces(qxy, qf, -1)):
        same(a, b)
    q1, q2 = qf.copy(), qf.copy()
    for a, b in zip(g.locate_faces(qxy, q1), o.locate_faces(qxy, q2)):
        same(a, b)
    same(q1, q2)
    pts = syn.uniform_points(1_000_000, txy.min(0), txy.max(0), seed=66)
    pts[::100] = syn.near_edge_points(txy, tf, len(pts[::100]), dist=1e-12, seed=67)
    for a, b in zip(g.compute_barycentric_weights(pts), o.compute_barycentric_weights(pts)):
        same(a, b)
    boxes = syn.random_boxes(50_000, txy.min(0), txy.max(0), 0.01, 5.0, seed=68, log_uniform=True)
    for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
        same(a, b)
    for a, b in zip(g.intersect_boxes(boxes[:20_000]), o.intersect_boxes(boxes[:20_000])):
        same(a, b)
    rng = np.random.default_rng(69)
    a0 = rng.uniform(txy.min(0), txy.max(0), (100_000, 2))
    ang = rng.uniform(0.0, 2 * np.pi, 100_000)
    ln = rng.uniform(0.0, 2.0, 100_000)
    segs = np.stack([a0, a0 + np.stack([ln * np.cos(ang), ln * np.sin(ang)], 1)], 1)
    for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
        same(a, b)


def test_mixed_mesh_boxes_and_segments_match_oracle(oracle):
    """Mixed polygons (K = 6) at a tenth of the 4M-cell shape's cell count:
    boxes with log-uniform sides, segments with uniform endpoints."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.mixed_mesh(632, 632, seed=70, extent=(316.0, 316.0))
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    for fld in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        same(g.nodes[fld], o.nodes[fld])
    same(g.bb_indices, o.bb_indices)
    boxes = syn.random_boxes(20_000, (0.0, 0.0), (316.0, 316.0), 0.03, 16.0, seed=71, log_uniform=True)
    for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
        same(a, b)
    for a, b in zip(g.intersect_boxes(boxes), o.intersect_boxes(boxes)):
        same(a, b)
    segs = syn.random_segments(2_000, (0.0, 0.0), (316.0, 316.0), seed=72)
    for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
        same(a, b)


def _fd_check(fwd, base, grad, samples, h=1e-6, rtol=1e-6):
    """Central differences of sum(g * fwd(vertices)) at the sampled (vertex,
    coordinate) slots against the analytic gradient.  Rows of fwd whose
    inputs a perturbation does not touch are bit-identical on both sides, so
    only the affected terms enter the difference.  A sample whose derivative
    is not smooth at the scale of h (the perturbation moves a vertex across
    another mesh's edge line) shows up as disagreement between h and h / 2;
    at most 1 % of the samples may be set aside that way."""
    import torch

    bad, kinks = [], 0
    for k, c in samples:
        fd = []
        for hh in (h, 0.5 * h):
            vp, vm = base.clone(), base.clone()
            vp[k, c] += hh
            vm[k, c] -= hh
            fd.append(float((fwd(vp) - fwd(vm)).sum()) / (2 * hh))
        an = float(grad[k, c])
        scale = max(1.0, abs(an))
        if abs(fd[0] - fd[1]) > 1e-4 * scale:
            kinks += 1
            continue
        if abs(fd[0] - an) > rtol * scale:
            bad.append((k, c, fd[0], an))
    assert not bad, bad[:5]
    assert kinks <= len(samples) // 100, kinks
    del torch


def test_clip_area_adjoint_fd_on_1000_pairs(regrid_pair):
    import torch

    from numba_celltree_gb300 import autodiff

    txy, tf, qxy, qf, g, _ = regrid_pair
    ClipArea = autodiff._functions()[0]
    v = torch.tensor(qxy, device="cuda")
    tv = g._tree.vertices.clone()
    v_d, f_d = g._faces_on_device(v, qf)
    ii, jj = g._locate_faces_dev(v_d, f_d)
    err = g._tree.error_word
    te = g._tree.elements
    n = int(ii.shape[0])
    assert n > 300_000
    gw = torch.tensor(np.random.default_rng(73).normal(size=n), device="cuda")
    vg, tvg = v.clone().requires_grad_(True), tv.clone().requires_grad_(True)
    gv, gtv = torch.autograd.grad((ClipArea.apply(vg, tvg, f_d, te, ii, jj, err) * gw).sum(), [vg, tvg])
    rng = np.random.default_rng(74)
    pairs = rng.choice(n, size=1000, replace=False)
    qfh, tfh = f_d.cpu().numpy(), te.cpu().numpy()
    iih, jjh = ii.cpu().numpy(), jj.cpu().numpy()
    qs, ts = [], []
    for t in pairs:
        # one vertex of the pair (query triangle or tree quad) and one coordinate
        if rng.random() < 0.5:
            qs.append((int(qfh[iih[t], rng.integers(0, 3)]), int(rng.integers(0, 2))))
        else:
            ts.append((int(tfh[jjh[t], rng.integers(0, 4)]), int(rng.integers(0, 2))))
    _fd_check(lambda vq: ClipArea.apply(vq, tv, f_d, te, ii, jj, err) * gw, v, gv, qs)
    _fd_check(lambda vt: ClipArea.apply(v, vt, f_d, te, ii, jj, err) * gw, tv, gtv, ts)


def test_barycentric_adjoint_fd_on_1000_points(regrid_pair):
    import torch

    from numba_celltree_gb300 import autodiff

    txy, tf, _, _, g, _ = regrid_pair
    Bary = autodiff._functions()[1]
    pts = syn.uniform_points(200_000, txy.min(0) + 0.5, txy.max(0) - 0.5, seed=75)
    p = torch.tensor(pts, device="cuda")
    idx, _ = g.compute_barycentric_weights(p)
    tol = g.default_tolerance()
    tv = g._tree.vertices.clone()
    G = torch.tensor(np.random.default_rng(76).normal(size=(len(pts), 4)), device="cuda")
    pg, tvg = p.clone().requires_grad_(True), tv.clone().requires_grad_(True)
    gp, gtv = torch.autograd.grad((Bary.apply(pg, tvg, g._tree, idx, tol) * G).sum(), [pg, tvg])
    rng = np.random.default_rng(77)
    ih = idx.cpu().numpy()
    found = np.nonzero(ih >= 0)[0]
    tfh = g._tree.elements.cpu().numpy()
    sel = rng.choice(found, size=1000, replace=False)
    ps = [(int(r), int(rng.integers(0, 2))) for r in sel[:500]]
    vs = [(int(tfh[ih[r], rng.integers(0, 4)]), int(rng.integers(0, 2))) for r in sel[500:]]
    _fd_check(lambda pp: Bary.apply(pp, tv, g._tree, idx, tol) * G, p, gp, ps, rtol=1e-5)
    _fd_check(lambda vv: Bary.apply(p, vv, g._tree, idx, tol) * G, tv, gtv, vs, rtol=1e-5)
