"""GPU tree construction against the oracle and the upstream fixtures:
faces (after the counter-clockwise fix), bb_coords, nodes and bb_indices must
be bit-identical."""

import numpy as np
import pytest

from meshes import GOLDEN, meshes
from numba_celltree_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

FIELDS = ("child", "Lmax", "Rmin", "ptr", "size", "dim")
PARAMS = [(4, 2), (2, 1), (3, 3), (8, 2), (4, 1), (5, 4), (32, 2), (16, 8)]


def _same_tree(g, o):
    assert np.array_equal(g.faces if hasattr(o, "faces") else g.bb_indices, o.faces if hasattr(o, "faces") else o.bb_indices)
    assert np.array_equal(g.bb_coords, o.bb_coords)
    assert np.array_equal(g.bbox, o.bbox)
    gn, on = g.nodes, o.nodes
    assert len(gn) == len(on), (len(gn), len(on))
    for f in FIELDS:
        a, b = gn[f], on[f]
        bad = np.nonzero(a != b)[0] if f != "Lmax" and f != "Rmin" else np.nonzero(a.view(np.int64) != b.view(np.int64))[0]
        assert len(bad) == 0, (f, bad[:10], a[bad[:5]], b[bad[:5]])
    assert np.array_equal(g.bb_indices, o.bb_indices)


@pytest.mark.parametrize("name", list(meshes().keys()))
@pytest.mark.parametrize("nb,cpl", PARAMS)
def test_build_matches_oracle(oracle, name, nb, cpl):
    from numba_celltree_gb300 import CellTree2d

    xy, f = meshes()[name]
    g = CellTree2d(xy, f, -1, nb, cpl)
    o = oracle.OracleCellTree2d(xy, f, -1, nb, cpl)
    _same_tree(g, o)


def test_build_matches_upstream_fixtures():
    from numba_celltree_gb300 import CellTree2d

    G = np.load(GOLDEN / "golden_trees.npz")
    for i in range(int(G["n_cases"])):
        p = f"c{i}_"
        nb, cpl = (int(x) for x in G[p + "params"])
        g = CellTree2d(G[p + "vertices"], G[p + "faces_in"], -1, nb, cpl)
        assert np.array_equal(g.faces, G[p + "faces"])
        for fld in FIELDS:
            assert np.array_equal(g.nodes[fld], G[p + "node_" + fld]), (i, fld)
        assert np.array_equal(g.bb_indices, G[p + "bb_indices"])
        assert np.array_equal(g.bb_coords, G[p + "bb_coords"])


@pytest.mark.parametrize("n", [1, 2, 3, 5, 127, 128, 129, 300, 2049])
@pytest.mark.parametrize("cpl", [1, 2])
def test_build_small_and_boundary_sizes(oracle, n, cpl):
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(64, seed=n)
    rng = np.random.default_rng(n)
    f = f[rng.permutation(len(f))[:n]]
    g = CellTree2d(xy, f, -1, 4, cpl)
    o = oracle.OracleCellTree2d(xy, f, -1, 4, cpl)
    _same_tree(g, o)


def test_build_degenerate_duplicates(oracle):
    """Identical cells force the all-in-one-bucket path (dimension flip, then leaf)."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(30, seed=11)
    f = np.concatenate([f, np.repeat(f[:3], 400, axis=0), f[100:140]])
    for nb, cpl in [(4, 2), (2, 1), (3, 5)]:
        g = CellTree2d(xy, f, -1, nb, cpl)
        o = oracle.OracleCellTree2d(xy, f, -1, nb, cpl)
        _same_tree(g, o)


def test_build_columns_flip_dimension_in_large_nodes(oracle):
    """Columns and rows of cells one cell wide: every centroid of a large
    node shares one bucket along the node's dimension, so the multi-CTA
    levels flip it and split along the other (the second statistics pass)."""
    from numba_celltree_gb300 import CellTree2d

    for nx, ny in ((1, 3000), (3000, 1), (2, 1500)):
        xy, f = syn.quad_mesh(nx, ny, seed=15, extent=(float(nx), float(ny)), jitter=0.0)
        for nb, cpl in ((4, 2), (3, 1)):
            g = CellTree2d(xy, f, -1, nb, cpl)
            o = oracle.OracleCellTree2d(xy, f, -1, nb, cpl)
            _same_tree(g, o)


def test_build_signed_zero_bounds(oracle):
    """Boxes whose extremes are -0.0 and +0.0: first occurrence decides the sign."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(40, seed=12, extent=(2.0, 2.0), offset=(-1.0, -1.0))
    xy = xy.copy()
    xy[np.isclose(xy[:, 0], 0.0, atol=1e-3), 0] = 0.0
    neg = np.nonzero(xy[:, 0] == 0.0)[0][::2]
    xy[neg, 0] = -0.0
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    _same_tree(g, o)


def test_build_large_levels(oracle):
    """Enough cells for several multi-CTA levels (tiles) before the warp subtrees."""
    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(400, seed=13)
    g = CellTree2d(xy, f, -1)
    o = oracle.OracleCellTree2d(xy, f, -1)
    _same_tree(g, o)
    xy, f = syn.mixed_mesh(250, seed=14)
    g = CellTree2d(xy, f, -1, 6, 3)
    o = oracle.OracleCellTree2d(xy, f, -1, 6, 3)
    _same_tree(g, o)


@pytest.mark.gpu
@pytest.mark.parametrize("nb, cpl", [(4, 2), (3, 1), (8, 4)])
def test_build_regular_grids_tied_split_costs(oracle, nb, cpl):
    """Unjittered grids: many nodes whose split_plane costs tie exactly (the
    float32 cost screening must leave those to the float64 comparison and
    its first-minimum rule), at integer and at large offset coordinates."""
    from numba_celltree_gb300 import CellTree2d

    for nx, ny, extent, offset in [(32, 16, (64.0, 32.0), (0.0, 0.0)), (150, 150, (300.0, 300.0), (5.0e5, 4.2e6))]:
        xy, f = syn.triangle_mesh(nx, ny, seed=1, extent=extent, offset=offset, jitter=0.0)
        g = CellTree2d(xy, f, -1, nb, cpl)
        o = oracle.OracleCellTree2d(xy, f, -1, nb, cpl)
        _same_tree(g, o)
        xy, f = syn.quad_mesh(nx, ny, seed=1, extent=extent, offset=offset, jitter=0.0)
        g = CellTree2d(xy, f, -1, nb, cpl)
        o = oracle.OracleCellTree2d(xy, f, -1, nb, cpl)
        _same_tree(g, o)
