"""Adjoints of the area of intersection and of the barycentric weights.

Two independent references pin the reverse-mode kernels:
* a float64 restatement in torch (the upstream Sutherland-Hodgman clip with
  its fan area, the triangle and Wachspress weights, the on-edge branch)
  differentiated by torch.autograd;
* central finite differences, h = 1e-6, of the GPU forward itself.
"""

import numpy as np
import pytest

from numba_celltree_gb300 import synthetic as syn

torch = pytest.importorskip("torch")


# ---- torch restatement (float64, autograd) ---------------------------------
def _cross(u, v):
    return u[0] * v[1] - u[1] * v[0]


def _sh_area(subj, clip):
    """polygon_polygon_clip_area (sutherland_hodgman.py:83-148) + polygon_area."""
    output = list(subj)
    r = clip[-1]
    for s in clip:
        U = s - r
        if U[0].item() == 0 and U[1].item() == 0:
            continue
        N = torch.stack([-U[1], U[0]])
        subject, output = output, []
        a = subject[-1]
        a_in = (U[0] * (a[1] - r[1]) > U[1] * (a[0] - r[0])).item()
        for b in subject:
            V = b - a
            if V[0].item() == 0 and V[1].item() == 0:
                continue
            b_in = (U[0] * (b[1] - r[1]) > U[1] * (b[0] - r[0])).item()

            def isect():
                W = r - a
                nw, nv = (N * W).sum(), (N * V).sum()
                if nv.item() != 0:
                    return a + (nw / nv) * V
                return None

            if b_in:
                if not a_in:
                    p = isect()
                    if p is not None:
                        output.append(p)
                output.append(b)
            elif a_in:
                p = isect()
                if p is not None:
                    output.append(p)
                else:
                    b_in = True
                    output.append(b)
            a, a_in = b, b_in
        if len(output) < 3:
            return subj[0][0] * 0.0
        r = s
    p0 = output[0]
    U = output[1] - p0
    area = subj[0][0] * 0.0
    for c in output[2:]:
        V = p0 - c
        area = area + torch.abs(_cross(U, V))
        U = V
    return 0.5 * area


def _tri_weights(a, b, c, p):
    ab, ac, ap = b - a, c - a, p - a
    Aa, Ac, A = torch.abs(_cross(ab, ap)), torch.abs(_cross(ac, ap)), torch.abs(_cross(ab, ac))
    inv = 1.0 / A
    w, v = inv * Aa, inv * Ac
    return torch.stack([1.0 - v - w, v, w])


def _wachspress(poly, p, K, tol):
    n = len(poly)
    zero = p[0] * 0.0

    def edge_case(a, U, i, j):
        V = p - a
        w = torch.sqrt((V * V).sum()) / torch.sqrt((U * U).sum())
        out = [zero] * K
        out[i] = 1.0 - w
        out[j] = w
        return torch.stack(out)

    a, b = poly[-1], poly[0]
    U, V = b - a, p - a
    Ai = torch.abs(_cross(U, V))
    if (Ai * Ai).item() < (tol * (U * U).sum() * tol).item():
        return edge_case(a, U, n - 1, 0)
    ws = []
    for i in range(n):
        c = poly[(i + 1) % n]
        W = c - a
        Ci = torch.abs(_cross(U, W))
        U, V = c - b, p - b
        Aj = torch.abs(_cross(U, V))
        if (Aj * Aj).item() < (tol * (U * U).sum() * tol).item():
            return edge_case(b, U, i, (i + 1) % n)
        ws.append(2 * Ci / (Ai * Aj))
        a, b, Ai = b, c, Aj
    S = sum(ws)
    return torch.stack([w / S for w in ws] + [zero] * (K - n))


# ---- fixtures ---------------------------------------------------------------
def _meshes():
    # query: jittered triangles; tree: quads rotated 7 degrees, offset 0.37 cell
    qxy, qf = syn.triangle_mesh(12, 10, seed=41, extent=(12.0, 10.0), offset=(100.0, 200.0))
    txy, tf = syn.quad_mesh(9, 8, seed=42, extent=(11.0, 9.0), offset=(100.37, 200.37), rotate_deg=7.0)
    return qxy, qf, txy, tf


@pytest.mark.gpu
def test_clip_area_grad_matches_torch_autograd():
    from numba_celltree_gb300 import CellTree2d, autodiff

    qxy, qf, txy, tf = _meshes()
    tree = CellTree2d(txy, tf, -1)
    v = torch.tensor(qxy, device="cuda", requires_grad=True)
    tv = tree._tree.vertices.clone().requires_grad_(True)
    i, j, area = autodiff.intersect_faces(tree, v, qf, -1, tree_vertices=tv)
    # same pairs and areas as the plain method
    i0, j0, a0 = tree.intersect_faces(qxy, qf, -1)
    assert np.array_equal(i.cpu().numpy(), i0) and np.array_equal(j.cpu().numpy(), j0)
    assert np.array_equal(area.detach().cpu().numpy(), a0)
    g = torch.tensor(np.random.default_rng(1).normal(size=len(i0)), device="cuda")
    gv, gtv = torch.autograd.grad((area * g).sum(), [v, tv])
    # torch restatement on the host (same oriented faces as the tree / query)
    qfaces = tree._faces_on_device(torch.as_tensor(qxy), qf)[1]
    tree._locate_faces_dev(torch.as_tensor(qxy, device="cuda"), qfaces)  # orient query faces as upstream
    qfaces = qfaces.cpu().numpy()
    tfaces = tree._tree.elements.cpu().numpy()
    hv = torch.tensor(qxy, dtype=torch.float64, requires_grad=True)
    htv = torch.tensor(tree._tree.vertices.cpu().numpy(), dtype=torch.float64, requires_grad=True)
    gh = g.cpu()
    total = 0.0
    sel = np.random.default_rng(2).choice(len(i0), size=min(60, len(i0)), replace=False)
    mask = torch.zeros(len(i0), dtype=torch.float64)
    mask[sel] = 1.0
    for t in sel:
        fa = [k for k in qfaces[i0[t]] if k >= 0]
        fb = [k for k in tfaces[j0[t]] if k >= 0]
        a_ref = _sh_area([hv[k] for k in fa], [htv[k] for k in fb])
        assert abs(a_ref.item() - a0[t]) <= 1e-12 * max(1.0, abs(a0[t]))
        total = total + gh[t] * a_ref
    rv, rtv = torch.autograd.grad(total, [hv, htv])
    # kernel gradients restricted to the sampled pairs
    v2 = torch.tensor(qxy, device="cuda", requires_grad=True)
    tv2 = tree._tree.vertices.clone().requires_grad_(True)
    _, _, area2 = autodiff.intersect_faces(tree, v2, qf, -1, tree_vertices=tv2)
    kv, ktv = torch.autograd.grad((area2 * g * mask.cuda()).sum(), [v2, tv2])
    np.testing.assert_allclose(kv.cpu().numpy(), rv.numpy(), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(ktv.cpu().numpy(), rtv.numpy(), rtol=1e-9, atol=1e-12)
    assert torch.isfinite(gv).all() and torch.isfinite(gtv).all()


@pytest.mark.gpu
def test_clip_area_grad_finite_differences():
    from numba_celltree_gb300 import CellTree2d, autodiff

    qxy, qf, txy, tf = _meshes()
    tree = CellTree2d(txy, tf, -1)
    ClipArea = autodiff._functions()[0]
    v = torch.tensor(qxy, device="cuda")
    tv = tree._tree.vertices.clone()
    v_d, f_d = tree._faces_on_device(v, qf)
    ii, jj = tree._locate_faces_dev(v_d, f_d)
    err = tree._tree.error_word
    g = torch.tensor(np.random.default_rng(3).normal(size=len(ii)), device="cuda")

    def L(vq, vt):
        return float((ClipArea.apply(vq, vt, f_d, tree._tree.elements, ii, jj, err) * g).sum())

    vg = v.clone().requires_grad_(True)
    tvg = tv.clone().requires_grad_(True)
    gv, gtv = torch.autograd.grad((ClipArea.apply(vg, tvg, f_d, tree._tree.elements, ii, jj, err) * g).sum(),
                                  [vg, tvg])
    h = 1e-6
    rng = np.random.default_rng(4)
    for which, base, grad in (("query", v, gv), ("tree", tv, gtv)):
        for k in rng.choice(base.shape[0], size=12, replace=False):
            for c in (0, 1):
                vp, vm = base.clone(), base.clone()
                vp[k, c] += h
                vm[k, c] -= h
                if which == "query":
                    fd = (L(vp, tv) - L(vm, tv)) / (2 * h)
                else:
                    fd = (L(v, vp) - L(v, vm)) / (2 * h)
                an = float(grad[k, c])
                assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (which, k, c, fd, an)


def _bary_case(kind):
    if kind == "tri":
        xy, f = syn.triangle_mesh(10, 8, seed=51, extent=(10.0, 8.0), offset=(3.0e3, -7.0e2))
    else:
        xy, f = syn.mixed_mesh(10, 8, seed=52, extent=(10.0, 8.0))
    return xy, f


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tri", "poly"])
def test_barycentric_grad_matches_torch_autograd(kind):
    from numba_celltree_gb300 import CellTree2d, autodiff

    xy, f = _bary_case(kind)
    tree = CellTree2d(xy, f, -1)
    lo, hi = xy.min(0), xy.max(0)
    pts = np.concatenate([syn.uniform_points(300, lo, hi, seed=5), syn.near_edge_points(xy, f, 40, dist=0.0, seed=6)])
    # |p - a| is not differentiable at a vertex (torch: NaN, kernel: 0); keep
    # on-edge points, drop those that coincide with a vertex
    dmin = np.min(np.abs(pts[:, None, :] - xy[None, :, :]).sum(-1), axis=1)
    pts = pts[dmin > 1e-9]
    p = torch.tensor(pts, device="cuda", requires_grad=True)
    tv = tree._tree.vertices.clone().requires_grad_(True)
    idx, w = autodiff.compute_barycentric_weights(tree, p, tree_vertices=tv)
    i0, w0 = tree.compute_barycentric_weights(pts)
    assert np.array_equal(idx.cpu().numpy(), i0)
    assert np.array_equal(w.detach().cpu().numpy(), w0)
    G = torch.tensor(np.random.default_rng(7).normal(size=w0.shape), device="cuda")
    gp, gtv = torch.autograd.grad((w * G).sum(), [p, tv])
    assert torch.isfinite(gp).all() and torch.isfinite(gtv).all()
    # torch restatement
    faces = tree._tree.elements.cpu().numpy()
    K = faces.shape[1]
    tol = tree.default_tolerance()
    hp = torch.tensor(pts, dtype=torch.float64, requires_grad=True)
    htv = torch.tensor(tree._tree.vertices.cpu().numpy(), dtype=torch.float64, requires_grad=True)
    Gh = G.cpu()
    total = 0.0
    for r in range(len(pts)):
        if i0[r] < 0:
            continue
        face = faces[i0[r]]
        if K <= 3:
            wr = _tri_weights(htv[face[0]], htv[face[1]], htv[face[2]], hp[r])
        else:
            wr = _wachspress([htv[k] for k in face if k >= 0], hp[r], K, tol)
        np.testing.assert_allclose(wr.detach().numpy(), w0[r], rtol=0, atol=1e-13)
        total = total + (wr * Gh[r]).sum()
    rp, rtv = torch.autograd.grad(total, [hp, htv])
    np.testing.assert_allclose(gp.cpu().numpy(), rp.numpy(), rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(gtv.cpu().numpy(), rtv.numpy(), rtol=1e-9, atol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tri", "poly"])
def test_barycentric_grad_finite_differences(kind):
    from numba_celltree_gb300 import CellTree2d, autodiff

    xy, f = _bary_case(kind)
    tree = CellTree2d(xy, f, -1)
    Bary = autodiff._functions()[1]
    lo, hi = xy.min(0), xy.max(0)
    pts = syn.uniform_points(200, lo + 0.05, hi - 0.05, seed=8)
    p = torch.tensor(pts, device="cuda")
    idx, _ = tree.compute_barycentric_weights(p)
    tol = tree.default_tolerance()
    tv = tree._tree.vertices.clone()
    G = torch.tensor(np.random.default_rng(9).normal(size=(len(pts), max(3, tree._tree.K))), device="cuda")

    def L(pp, vv):
        return float((Bary.apply(pp, vv, tree._tree, idx, tol) * G).sum())

    pg, tvg = p.clone().requires_grad_(True), tv.clone().requires_grad_(True)
    gp, gtv = torch.autograd.grad((Bary.apply(pg, tvg, tree._tree, idx, tol) * G).sum(), [pg, tvg])
    h = 1e-6
    rng = np.random.default_rng(10)
    used = np.unique(tree._tree.elements.cpu().numpy()[idx.cpu().numpy()[idx.cpu().numpy() >= 0]])
    used = used[used >= 0]
    for k in rng.choice(used, size=10, replace=False):
        for c in (0, 1):
            vp, vm = tv.clone(), tv.clone()
            vp[k, c] += h
            vm[k, c] -= h
            fd = (L(p, vp) - L(p, vm)) / (2 * h)
            an = float(gtv[k, c])
            assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (k, c, fd, an)
    for k in rng.choice(len(pts), size=10, replace=False):
        for c in (0, 1):
            pp_, pm_ = p.clone(), p.clone()
            pp_[k, c] += h
            pm_[k, c] -= h
            fd = (L(pp_, tv) - L(pm_, tv)) / (2 * h)
            an = float(gp[k, c])
            assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (k, c, fd, an)
