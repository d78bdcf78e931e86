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


def test_noalloc_build_at_the_size_limit():
    """16,384 cells with n_buckets = 32 and cells_per_leaf = 1: the largest
    scratch the entry point accepts, where a wrong scratch layout would show."""
    from numba_celltree_gb300 import synthetic as syn

    xy, f = syn.triangle_mesh(128, 64, seed=33, extent=(2.0, 1.0))
    assert f.shape[0] == 16384
    _check_against_allocating(xy, f, 32, 1)
    _check_against_allocating(xy, f, 2, 1)


def _raw_build(lib, bb_ptr, n, n_buckets, cells_per_leaf, noalloc, st):
    """One build through the C ABI (noalloc or ct_build_tree + ct_build_emit)
    on device boxes bb_ptr; returns (status, n_nodes, node fields, bb_indices)."""
    import torch

    cap = int(lib.ct_pessimistic_n_nodes(n))
    arrs = [torch.full((cap,), -7, dtype=dt, device="cuda")
            for dt in (torch.int64, torch.float64, torch.float64, torch.int64, torch.int64, torch.uint8)]
    bbi = torch.full((max(n, 1),), -7, dtype=torch.int64, device="cuda")
    n_nodes, depth = ctypes.c_int64(-1), ctypes.c_int32(-1)
    ptrs = [a.data_ptr() for a in arrs]
    if noalloc:
        status = lib.ct_build_tree_noalloc(bb_ptr, n, n_buckets, cells_per_leaf, *ptrs, cap, bbi.data_ptr(),
                                           ctypes.byref(n_nodes), ctypes.byref(depth), st)
    else:
        wsz = int(lib.ct_build_workspace_size(n, n_buckets, 1))
        ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device="cuda")
        status = lib.ct_build_tree(bb_ptr, n, n_buckets, cells_per_leaf, 1, ws.data_ptr(), wsz,
                                   ctypes.byref(n_nodes), ctypes.byref(depth), st)
        if status == 0:
            status = lib.ct_build_emit(ws.data_ptr(), n, n_buckets, 1, *ptrs, bbi.data_ptr(), st)
    m = max(n_nodes.value, 0)
    return status, n_nodes.value, [a[:m].cpu().numpy() for a in arrs], bbi[:n].cpu().numpy()


def test_noalloc_build_of_zero_cells():
    """n = 0: a single empty root node, as from the allocating entry points."""
    import torch

    from numba_celltree_gb300 import _device, _lib

    lib = _lib.load()
    st = _device.stream()
    bb = torch.zeros((1, 4), dtype=torch.float64, device="cuda")
    s0, n0, f0, _ = _raw_build(lib, bb.data_ptr(), 0, 4, 2, True, st)
    s1, n1, f1, _ = _raw_build(lib, bb.data_ptr(), 0, 4, 2, False, st)
    assert s0 == 0 and s1 == 0
    assert n0 == n1 == 1
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)


_RESET_SCRIPT = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from numba_celltree_gb300 import _lib, synthetic as syn

lib = _lib.load()
rt = ctypes.CDLL("libcudart.so.13")
P = ctypes.c_void_p

def dalloc(nbytes):
    p = P()
    assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 8))) == 0
    return p.value

def h2d(arr):
    arr = np.ascontiguousarray(arr)
    p = dalloc(arr.nbytes)
    assert rt.cudaMemcpy(P(p), P(arr.ctypes.data), ctypes.c_size_t(arr.nbytes), 1) == 0
    return p

def d2h(p, n, dt):
    out = np.empty(n, dtype=dt)
    assert rt.cudaMemcpy(P(out.ctypes.data), P(p), ctypes.c_size_t(out.nbytes), 2) == 0
    return out

xy, f = syn.mixed_mesh(40, seed=34)
n, K = f.shape

def build(noalloc):
    v, fa = h2d(xy), h2d(f)
    assert lib.ct_counter_clockwise(v, fa, n, K, None) == 0
    bb = dalloc(n * 32)
    assert lib.ct_face_bboxes(v, fa, n, K, bb, None) == 0
    cap = int(lib.ct_pessimistic_n_nodes(n))
    out = [dalloc(cap * 8) for _ in range(5)] + [dalloc(cap)]
    bbi = dalloc(n * 8)
    nn, md = ctypes.c_int64(0), ctypes.c_int32(0)
    if noalloc:
        s = lib.ct_build_tree_noalloc(bb, n, 4, 2, *out, cap, bbi, ctypes.byref(nn), ctypes.byref(md), None)
        assert s == 0, lib.ct_last_error_message()
    else:
        wsz = int(lib.ct_build_workspace_size(n, 4, 1))
        ws = dalloc(wsz)
        assert lib.ct_build_tree(bb, n, 4, 2, 1, ws, wsz, ctypes.byref(nn), ctypes.byref(md), None) == 0
        assert lib.ct_build_emit(ws, n, 4, 1, *out, bbi, None) == 0
    m = nn.value
    dts = (np.int64, np.float64, np.float64, np.int64, np.int64, np.uint8)
    return [d2h(p, m, dt) for p, dt in zip(out, dts)] + [d2h(bbi, n, np.int64)]

for round_ in range(2):
    a, b = build(True), build(False)
    assert all(np.array_equal(x, y) for x, y in zip(a, b)), round_
    # end this process's context: the next call must look the array up again
    assert rt.cudaDeviceReset() == 0
print("reset ok")
"""


def test_noalloc_build_after_context_reset():
    """The cached device address of the static scratch belongs to a context:
    after cudaDeviceReset (in a child process, so no other test's state is
    touched) the entry point must look it up again and still build the same
    tree as the allocating entry points."""
    import os
    import pathlib
    import subprocess
    import sys

    root = str(pathlib.Path(__file__).resolve().parents[1])
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, root], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reset ok" in r.stdout


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
