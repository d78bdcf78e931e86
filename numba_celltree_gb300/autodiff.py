"""Differentiable forms of two tree queries (no upstream counterpart).

The intersection indices (which faces meet which tree faces, which face holds
a point) are piecewise constant, so they are computed once and held fixed;
the float64 values on top of them -- the area of intersection
(``CellTree2d.intersect_faces``, celltree.py:228-269) and the barycentric
weights (``CellTree2d.compute_barycentric_weights``, celltree.py:306-351) --
are ``torch.autograd.Function`` s whose forward passes are the upstream
computations (bit-identical to the non-differentiable methods) and whose
backward passes are the reverse-mode kernels of ``csrc/ct_adjoint.cu``.

Gradients flow to float64 CUDA tensors that hold the vertex coordinates:
the query mesh's ``vertices`` and ``tree_vertices``, a tensor equal to the
tree's own vertex array (``CellTree2d.vertices``) that stands in for it.
"""

from __future__ import annotations

import ctypes
from typing import Optional

from . import _device, _lib
from .cast import cast_faces, cast_vertices


def _torch():
    return _device.torch()


def _check_vertices(v, n_vertices: int, name: str):
    torch = _torch()
    if not (isinstance(v, torch.Tensor) and v.is_cuda and v.dtype == torch.float64):
        raise ValueError(f"{name} must be a float64 CUDA tensor")
    if v.ndim != 2 or v.shape[1] != 2 or v.shape[0] != n_vertices:
        raise ValueError(f"{name} must have shape ({n_vertices}, 2)")
    return v


def _make_functions():
    torch = _torch()

    class ClipArea(torch.autograd.Function):
        """area[t] = polygon_polygon_clip_area(face_a[ia[t]], face_b[ib[t]])."""

        @staticmethod
        def forward(ctx, va, vb, fa, fb, ia, ib, err):
            n = int(ia.shape[0])
            area = torch.empty((n,), dtype=torch.float64, device=va.device)
            va_c, vb_c = va.detach().contiguous(), vb.detach().contiguous()
            _lib.check(
                _lib.load().ct_area_of_intersection(
                    _device.ptr(va_c), _device.ptr(fa), int(fa.shape[1]), _device.ptr(vb_c), _device.ptr(fb),
                    int(fb.shape[1]), _device.ptr(ia), _device.ptr(ib), n, _device.ptr(area), _device.ptr(err),
                    _device.stream(),
                ),
                "area_of_intersection",
            )
            ctx.save_for_backward(va_c, vb_c, fa, fb, ia, ib)
            ctx.err = err  # the tree's error word: reset and written in place, not saved
            return area

        @staticmethod
        def backward(ctx, g):
            va, vb, fa, fb, ia, ib = ctx.saved_tensors
            err = ctx.err
            err.zero_()
            gva = torch.zeros_like(va)
            gvb = torch.zeros_like(vb)
            g = g.detach().to(torch.float64).contiguous()
            _lib.check(
                _lib.load().ct_area_of_intersection_grad(
                    _device.ptr(va), _device.ptr(fa), int(fa.shape[1]), _device.ptr(vb), _device.ptr(fb),
                    int(fb.shape[1]), _device.ptr(ia), _device.ptr(ib), int(ia.shape[0]), _device.ptr(g),
                    _device.ptr(gva), _device.ptr(gvb), _device.ptr(err), _device.stream(),
                ),
                "area_of_intersection_grad",
            )
            if int(err.item()):
                raise _lib.CellTreeError("area_of_intersection_grad: clip polygon scratch overflow")
            return (gva if ctx.needs_input_grad[0] else None, gvb if ctx.needs_input_grad[1] else None,
                    None, None, None, None, None)

    class BarycentricWeights(torch.autograd.Function):
        """weights[i] of point i in tree face face_index[i] (zero row for -1)."""

        @staticmethod
        def forward(ctx, points, tree_vertices, tree, face_index, tol):
            n = int(points.shape[0])
            K = tree.K
            KW = K if K > 3 else 3
            pts = points.detach().contiguous()
            tv = tree_vertices.detach().contiguous()
            w = torch.empty((n, KW), dtype=torch.float64, device=points.device)
            desc = _lib.CtTree.from_buffer_copy(tree.desc)
            desc.vertices = _device.ptr(tv)
            _lib.check(
                _lib.load().ct_barycentric_weights(
                    ctypes.byref(desc), _device.ptr(pts), _device.ptr(face_index), n, float(tol), _device.ptr(w),
                    _device.stream(),
                ),
                "barycentric",
            )
            ctx.save_for_backward(pts, tv, face_index)
            ctx.tree = tree
            ctx.tol = float(tol)
            return w

        @staticmethod
        def backward(ctx, g):
            pts, tv, face_index = ctx.saved_tensors
            tree = ctx.tree
            K = tree.K
            KW = K if K > 3 else 3
            gv = torch.zeros_like(tv)
            gp = torch.empty_like(pts)
            g = g.detach().to(torch.float64).contiguous()
            _lib.check(
                _lib.load().ct_barycentric_weights_grad(
                    _device.ptr(pts), _device.ptr(face_index), int(pts.shape[0]), _device.ptr(tv),
                    _device.ptr(tree.elements), K, KW, ctx.tol, _device.ptr(g), _device.ptr(gv), _device.ptr(gp),
                    _device.stream(),
                ),
                "barycentric_weights_grad",
            )
            return (gp if ctx.needs_input_grad[0] else None, gv if ctx.needs_input_grad[1] else None,
                    None, None, None)

    return ClipArea, BarycentricWeights


_FUNCS = None


def _functions():
    global _FUNCS
    if _FUNCS is None:
        _FUNCS = _make_functions()
    return _FUNCS


def intersect_faces(tree, vertices, faces, fill_value: int = -1, tree_vertices=None):
    """Differentiable ``CellTree2d.intersect_faces``.

    ``vertices`` (float64 CUDA tensor, may require grad) and ``faces`` of the
    query mesh; ``tree_vertices`` defaults to the tree's own vertex tensor.
    Returns ``(face_indices, tree_face_indices, area)`` as CUDA tensors, the
    same pairs and areas as the method; ``area`` carries gradients to
    ``vertices`` and ``tree_vertices`` (indices held fixed).
    """
    torch = _torch()
    ClipArea, _ = _functions()
    t = tree._tree
    tv = t.vertices if tree_vertices is None else _check_vertices(tree_vertices, int(t.vertices.shape[0]),
                                                                      "tree_vertices")
    if not (isinstance(vertices, torch.Tensor) and vertices.is_cuda):
        vertices = torch.as_tensor(cast_vertices(vertices), device=t.device)
    v = _check_vertices(vertices, int(vertices.shape[0]), "vertices")
    f = cast_faces(faces.detach().cpu().numpy() if isinstance(faces, torch.Tensor) else faces, fill_value)
    v_d, f_d = tree._faces_on_device(v.detach(), f)
    if f_d.shape[0] == 0:
        e = torch.empty((0,), dtype=torch.int64, device=t.device)
        return e, e, torch.empty((0,), dtype=torch.float64, device=t.device)
    i, j = tree._locate_faces_dev(v_d, f_d)  # orients f_d counter-clockwise in place, as upstream
    t.reset_error()
    area = ClipArea.apply(v, tv, f_d, t.elements, i, j, t.error_word)
    t.raise_on_device_error()
    keep = area.detach() > 0
    return i[keep], j[keep], area[keep]


def compute_barycentric_weights(tree, points, tolerance: Optional[float] = None, tree_vertices=None):
    """Differentiable ``CellTree2d.compute_barycentric_weights``.

    Returns ``(face_indices, weights)`` as CUDA tensors; ``weights`` carries
    gradients to ``points`` and ``tree_vertices`` (the face indices held
    fixed).
    """
    torch = _torch()
    _, BarycentricWeights = _functions()
    t = tree._tree
    tol = tree._tolerance(tolerance)
    tv = t.vertices if tree_vertices is None else _check_vertices(tree_vertices, int(t.vertices.shape[0]),
                                                                      "tree_vertices")
    if not (isinstance(points, torch.Tensor) and points.is_cuda):
        points = torch.as_tensor(cast_vertices(points), device=t.device)
    p = _check_vertices(points, int(points.shape[0]), "points")
    idx = torch.empty((int(p.shape[0]),), dtype=torch.int64, device=t.device)
    t.reset_error()
    tree.launch_locate(p.detach().contiguous(), idx, tol, tree.precision)
    t.raise_on_device_error()
    w = BarycentricWeights.apply(p, tv, t, idx, tol)
    return idx, w
