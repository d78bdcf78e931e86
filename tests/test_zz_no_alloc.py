"""The allocation-free build entry point (ct_build_tree_noalloc).

Callers that cannot allocate device memory -- code running inside a runtime
that owns all device memory, or a plugin that may not call cudaMalloc -- build
trees through ct_build_tree_noalloc, whose scratch is a fixed device array in
the library.  This test calls it through the C ABI, twice in a row, and checks
that its nodes and bb_indices equal those of the allocating entry point
(ct_build_tree + ct_build_emit, used by CellTree2d).  Tree construction is
integer and index work, so the comparison is exact.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("child", "Lmax", "Rmin", "ptr", "size", "dim")


def _noalloc_build(xy, faces, n_buckets, cells_per_leaf):
    import torch

    from numba_celltree_gb300 import _device, _lib

    lib = _lib.load()
    st = _device.stream()
    v = torch.as_tensor(np.ascontiguousarray(xy, dtype=np.float64), device="cuda")
    f = torch.as_tensor(np.ascontiguousarray(faces, dtype=np.int64), device="cuda")
    n, K = int(f.shape[0]), int(f.shape[1])
    _lib.check(lib.ct_counter_clockwise(v.data_ptr(), f.data_ptr(), n, K, st))
    bb = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    _lib.check(lib.ct_face_bboxes(v.data_ptr(), f.data_ptr(), n, K, bb.data_ptr(), st))
    cap = int(lib.ct_pessimistic_n_nodes(n))
    child = torch.empty(cap, dtype=torch.int64, device="cuda")
    Lmax = torch.empty(cap, dtype=torch.float64, device="cuda")
    Rmin = torch.empty(cap, dtype=torch.float64, device="cuda")
    ptr = torch.empty(cap, dtype=torch.int64, device="cuda")
    size = torch.empty(cap, dtype=torch.int64, device="cuda")
    dim = torch.empty(cap, dtype=torch.uint8, device="cuda")
    bbi = torch.empty(n, dtype=torch.int64, device="cuda")
    n_nodes = ctypes.c_int64(0)
    depth = ctypes.c_int32(0)
    _lib.check(
        lib.ct_build_tree_noalloc(
            bb.data_ptr(), n, n_buckets, cells_per_leaf, child.data_ptr(), Lmax.data_ptr(), Rmin.data_ptr(),
            ptr.data_ptr(), size.data_ptr(), dim.data_ptr(), cap, bbi.data_ptr(), ctypes.byref(n_nodes),
            ctypes.byref(depth), st,
        ),
        "ct_build_tree_noalloc",
    )
    m = n_nodes.value
    out = {k: t[:m].cpu().numpy() for k, t in zip(FIELDS, (child, Lmax, Rmin, ptr, size, dim))}
    return out, bbi.cpu().numpy()


def _check_against_allocating(xy, faces, n_buckets, cells_per_leaf):
    from numba_celltree_gb300 import CellTree2d

    ref = CellTree2d(xy, faces, -1, n_buckets, cells_per_leaf)
    nodes, bbi = _noalloc_build(xy, faces, n_buckets, cells_per_leaf)
    for k in FIELDS:
        got = nodes[k].astype(bool) if k == "dim" else nodes[k]
        assert np.array_equal(got, ref.nodes[k]), k
    assert np.array_equal(bbi, ref.bb_indices)


def test_noalloc_build_matches_allocating_build_twice():
    from numba_celltree_gb300 import synthetic as syn

    # two calls in a row: a larger mesh first, then a smaller one, so stale
    # scratch contents of the first call would show up in the second
    xy1, f1 = syn.triangle_mesh(80, seed=31)  # 12,800 cells
    xy2, f2 = syn.mixed_mesh(30, seed=32)
    _check_against_allocating(xy1, f1, 4, 2)
    _check_against_allocating(xy2, f2, 3, 1)


def test_noalloc_build_rejects_oversize():
    import torch

    from numba_celltree_gb300 import _device, _lib

    lib = _lib.load()
    n = 16385
    bb = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
    z = torch.zeros(4, dtype=torch.int64, device="cuda")
    status = lib.ct_build_tree_noalloc(
        bb.data_ptr(), n, 4, 2, z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(),
        4, z.data_ptr(), None, None, _device.stream(),
    )
    assert status == _lib.CT_ERR_ARG
    assert b"16384" in lib.ct_last_error_message()
