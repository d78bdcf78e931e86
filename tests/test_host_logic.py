"""Host-side logic that needs no GPU: the chunk schedule of the host-batch
pipeline."""

from numba_celltree_gb300._pipeline import chunk_bounds, page_cuts


def test_chunk_bounds_cover_in_order_and_ramp():
    for chunk in (1000, 4096, 1 << 25):
        for n in (0, 1, 7, 999, 1000, 1001, 4_194_304, 10_000_000, 268_435_456, 100_000_001):
            b = chunk_bounds(n, chunk)
            if n == 0:
                assert b == []
                continue
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(len(b) - 1))
            sizes = [e - s for s, e in b]
            assert all(0 < k <= chunk for k in sizes)
    sizes = [e - s for s, e in chunk_bounds(268_435_456, 1 << 25)]
    assert sizes[0] == 1 << 22 and sizes[-1] <= 1 << 22 and max(sizes) == 1 << 25


def test_page_cuts_give_every_chunk_its_own_pages():
    page = 65536
    for addr in (0x7F0000000000, 0x7F0000000010, 0x7F000000FFF0, 0x7F0000001230):
        for n, chunk in ((268_435_456, 1 << 25), (10_000, 1000), (5_000_000, 1 << 22), (4096, 1000)):
            b = page_cuts(addr, 16, chunk_bounds(n, chunk), page)
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] and b[i][0] < b[i][1] for i in range(len(b) - 1))
            for s, _ in b[1:]:
                assert (addr + 16 * s) % page == 0
            # page ranges of consecutive chunks do not overlap
            for (s0, e0), (s1, e1) in zip(b[:-1], b[1:]):
                last_page0 = (addr + 16 * e0 - 1) // page
                first_page1 = (addr + 16 * s1) // page
                assert last_page0 < first_page1
    assert page_cuts(0x7F0000000008, 16, chunk_bounds(10_000, 1000), page) is None
    assert page_cuts(0x7F0000000000, 16, [], page) == []


def test_grid_shape_is_near_square_and_bounded():
    """ct_grid_shape (host code of the C-ABI library, no GPU needed): about
    cells_per_element grid cells per mesh cell, nearly square grid cells,
    at least 16 per axis, at most 2^26 in all; degenerate extents fall back
    to a square grid; bad densities are rejected."""
    import ctypes

    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    gx, gy = ctypes.c_int32(0), ctypes.c_int32(0)

    def shape(n, w, h, d=1.0):
        assert lib.ct_grid_shape(n, w, h, d, ctypes.byref(gx), ctypes.byref(gy)) == 0
        return gx.value, gy.value

    x, y = shape(16_000_000, 4000.0, 2000.0)
    assert (x, y) == (5657, 2828)
    x, y = shape(16_000_000, 4000.0, 2000.0, 4.0)
    assert abs(x * y - 64_000_000) < 64_000_000 * 0.001 and abs(x - 2 * y) <= 2
    for n, w, h in [(1, 1.0, 1.0), (100, 10.0, 1.0), (10**6, 1.0, 1000.0), (10**9, 3.0, 1.0)]:
        x, y = shape(n, w, h)
        assert x >= 16 and y >= 16 and x * y <= 1 << 26
        if 16 < x and 16 < y and x * y < 1 << 26:
            # nearly square cells: the grid's aspect follows the bbox's
            assert abs((w / x) / (h / y) - 1.0) < 0.05
    assert shape(10**9, 1.0, 1.0)[0] * shape(10**9, 1.0, 1.0)[1] <= 1 << 26
    assert shape(1000, 0.0, 0.0) == shape(1000, 1.0, 1.0)
    assert lib.ct_grid_shape(10, 1.0, 1.0, 0.0, ctypes.byref(gx), ctypes.byref(gy)) != 0
    assert lib.ct_grid_shape(10, 1.0, 1.0, float("nan"), ctypes.byref(gx), ctypes.byref(gy)) != 0


def test_ctypes_mirrors_match_the_library_structs():
    """The Python mirrors of ct_tree and ct_forest_plan have the C layouts'
    sizes (and the library rejects unknown structure ids)."""
    import ctypes

    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    assert lib.ct_abi_sizeof(0) == ctypes.sizeof(_lib.CtTree)
    assert lib.ct_abi_sizeof(1) == ctypes.sizeof(_lib.CtForestPlan)
    assert lib.ct_abi_sizeof(2) == ctypes.sizeof(_lib.CtForestIndex)
    assert lib.ct_abi_sizeof(7) == 0


def test_noalloc_scratch_holds_the_largest_accepted_build():
    """ct_build_tree_noalloc accepts up to 16,384 cells with any n_buckets in
    [2, 32] on an 8 MiB static scratch: the allocating builder's workspace for
    the largest such case (n_buckets = 32, capacity factor 1) must fit."""
    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    for nb in (2, 4, 8, 16, 32):
        need = lib.ct_build_workspace_size(16384, nb, 1)
        assert 0 < need <= 8 << 20, (nb, need)


def test_library_exports_every_declared_entry_point():
    """Every function include/celltree_gb300.h declares is exported by the
    built library, and the ctypes binding declares no name the header lacks."""
    import pathlib
    import re

    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    hdr = (pathlib.Path(__file__).resolve().parents[1] / "include" / "celltree_gb300.h").read_text()
    names = set(re.findall(r"^\s*(?:const\s+)?(?:int|size_t|int64_t|char)\s*\*?\s*(ct_\w+)\s*\(", hdr, re.M))
    assert len(names) > 50
    missing = sorted(n for n in names if not hasattr(lib, n))
    assert not missing, missing
    assert set(_lib.SIGNATURES) <= names, sorted(set(_lib.SIGNATURES) - names)


def test_new_entry_points_reject_bad_arguments_before_any_launch():
    """The box and segment entry points validate their arguments on the host
    and fail with CT_ERR_ARG / CT_ERR_WORKSPACE before touching the device
    (runs without a GPU): bad modes, cut depths and scratch caps, too-small
    workspaces, trees without nodes."""
    import ctypes

    from numba_celltree_gb300 import _lib

    lib = _lib.load()
    empty = _lib.CtTree()
    t = _lib.CtTree()
    t.n_nodes, t.max_depth, t.n_max_vert, t.n_elements = 1, 0, 3, 1
    T, E = ctypes.byref(t), ctypes.byref(empty)
    dummy = 64  # never dereferenced: every call below fails its checks first
    ARG, WS = _lib.CT_ERR_ARG, _lib.CT_ERR_WORKSPACE
    assert lib.ct_count_edge_items(E, 1, dummy, 5, None, 4, dummy, None) == ARG  # no nodes
    assert lib.ct_count_edge_items(T, 2, dummy, 5, None, 4, dummy, None) == ARG  # mode
    assert lib.ct_count_edge_items(T, 0, dummy, 5, None, 4, dummy, None) == ARG  # edge mode on a face tree
    assert lib.ct_count_edge_items(T, 1, dummy, 5, None, 65, dummy, None) == ARG  # cut depth
    assert lib.ct_count_edge_items(T, 1, dummy, 5, None, -1, dummy, None) == ARG
    assert lib.ct_write_edge_items(T, 1, dummy, 5, None, 99, dummy, dummy, dummy, None) == ARG
    assert lib.ct_count_item_candidates(T, 3, dummy, dummy, dummy, 5, dummy, None) == ARG
    assert lib.ct_segment_candidate_ranges(dummy, dummy, -1, dummy, dummy, 0, dummy, dummy, None) == ARG
    assert lib.ct_count_edge_candidates_spec(T, 1, dummy, 5, None, dummy, dummy, 0, None) == ARG  # cap
    assert lib.ct_count_edge_candidates_spec(T, 1, dummy, 5, None, dummy, dummy, 4097, None) == ARG
    assert lib.ct_count_edge_candidates_spec(T, 1, dummy, 5, None, dummy, None, 64, None) == ARG  # no scratch
    assert lib.ct_write_edge_candidates_spec(T, 1, dummy, 5, None, dummy, dummy, dummy, 0, dummy, dummy,
                                             None) == ARG
    assert lib.ct_count_boxes_spec(T, dummy, 5, None, dummy, dummy, 0, None) == ARG
    assert lib.ct_count_boxes_spec(E, dummy, 5, None, dummy, dummy, 16, None) == ARG
    wsz = int(lib.ct_write_boxes_workspace_size(1000, 8))
    assert wsz >= 256 + (1000 // 8 + 1) * 32
    assert int(lib.ct_write_boxes_workspace_size(1000, 0)) == wsz  # 0 means the default, 8 cells
    assert int(lib.ct_write_boxes_workspace_size(1000, 1)) == int(lib.ct_write_boxes_workspace_size(1000, 2))
    assert lib.ct_write_boxes_ws(T, dummy, 5, None, dummy, 1000, 8, dummy, dummy, dummy, wsz - 1, None) == WS
    assert lib.ct_write_boxes_ws(T, dummy, 5, None, dummy, -1, 8, dummy, dummy, dummy, wsz, None) == ARG
    assert lib.ct_write_boxes_spec(T, dummy, 5, None, dummy, dummy, dummy, 16, 1000, 8, dummy, dummy, dummy,
                                   wsz - 1, None) == WS
    swz = int(lib.ct_sort_workspace_size(1000))
    assert swz >= 1000 * 32 + (1000 // 129 + 2) * 4
    assert lib.ct_sort_intersections(dummy, 5, dummy, dummy, dummy, dummy, dummy, 1000, dummy, dummy, dummy,
                                     swz - 1, None) == WS
    assert lib.ct_cs_certificates(E, dummy, dummy, dummy, 5, dummy, None) == ARG


def test_segment_split_rule():
    """edge_cut: segment traversals are cut into work items about `split`
    cells large below SPLIT_MAX_SEGMENTS segments (by default), never for
    trees of at most `split` cells or too deep for the stacked traversal."""
    from types import SimpleNamespace

    import numpy as np

    from numba_celltree_gb300.celltree_base import _GpuTree

    G = _GpuTree
    t = SimpleNamespace(n=5_000_000, max_depth=24, BATCHED_MAX_STACK=G.BATCHED_MAX_STACK,
                        SPLIT_CELLS=G.SPLIT_CELLS, SPLIT_MAX_SEGMENTS=G.SPLIT_MAX_SEGMENTS)
    cut = G.edge_cut(t, {}, 200)
    assert cut == int(np.ceil(np.log2(5_000_000 / G.SPLIT_CELLS)))  # 13: about 1024 cells per item
    assert G.edge_cut(t, {}, G.SPLIT_MAX_SEGMENTS) is None  # large batches run uncut
    assert G.edge_cut(t, {"split": 0}, 200) is None
    assert G.edge_cut(t, {"split": 256}, 10**7) == int(np.ceil(np.log2(5_000_000 / 256)))
    t.max_depth = 20
    assert G.edge_cut(t, {"split": 2}, 200) == 20  # at most the tree depth (log2(2.5e6) > 21)
    t.max_depth = 24
    t.n = 900
    assert G.edge_cut(t, {}, 200) is None  # a tree of at most `split` cells
    t.n, t.max_depth = 5_000_000, G.BATCHED_MAX_STACK - 1
    assert G.edge_cut(t, {}, 200) is None  # too deep for the stacked traversal
