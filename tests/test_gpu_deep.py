"""Trees deeper than the traversal stacks (upstream's stacks grow without
limit, utils.py:88-97).  A degenerate mesh of geometrically nested
triangles, built with n_buckets = 2 and cells_per_leaf = 1, peels one cell
per tree level: depth ~ n.  Point location (stack of 510 levels) and the box
and segment traversals (126 levels) then walk the tree through its parent
links, in the same order; every result must equal the oracle's."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def nested_triangles(n):
    """Triangle k spans (0.2 s, s), (s, 0.2 s), (s, s) with s = 2^-k: its
    centroid (0.73 s) lies in the upper half of every node range it is the
    largest cell of, the next cell's (0.37 s) in the lower half."""
    s = 2.0 ** -np.arange(n, dtype=np.float64)
    xy = np.stack([np.stack([0.2 * s, s], 1), np.stack([s, 0.2 * s], 1), np.stack([s, s], 1)], 1).reshape(-1, 2)
    faces = np.arange(3 * n, dtype=np.int64).reshape(n, 3)
    return xy, faces


@pytest.mark.parametrize("n", [200, 600])
def test_deep_tree_queries_match_oracle(oracle, n):
    from numba_celltree_gb300 import CellTree2d

    xy, f = nested_triangles(n)
    g = CellTree2d(xy, f, -1, n_buckets=2, cells_per_leaf=1)
    o = oracle.OracleCellTree2d(xy, f, -1, 2, 1)
    assert g._tree.max_depth > (510 if n == 600 else 126)
    for fld in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        assert np.array_equal(g.nodes[fld], o.nodes[fld]), fld
    assert np.array_equal(g.bb_indices, o.bb_indices)
    rng = np.random.default_rng(7)
    k = np.arange(n)
    s = 2.0 ** -k
    pts = np.concatenate([
        rng.uniform(0.0, 1.0, (5000, 2)),
        np.stack([0.8 * s, 0.8 * s], 1),       # inside cell k
        np.stack([0.6 * s, 0.6 * s], 1),       # on the hypotenuse-ish side of cell k
        np.stack([s, 0.5 * s], 1),             # on an edge of cell k
    ])
    expected = o.locate_points(pts)
    for prec in ("fp32", "fp32-inline", "fp64"):
        g.precision = prec
        assert np.array_equal(g.locate_points(pts), expected), prec
    boxes = np.concatenate([
        np.stack([0.5 * s, 1.5 * s, 0.5 * s, 1.5 * s], 1),
        np.concatenate([np.sort(rng.uniform(0, 1, (300, 2)), 1), np.sort(rng.uniform(0, 1, (300, 2)), 1)], 1),
    ])
    for a, b in zip(g.locate_boxes(boxes), o.locate_boxes(boxes)):
        assert np.array_equal(a, b)
    for a, b in zip(g.intersect_boxes(boxes), o.intersect_boxes(boxes)):
        assert np.array_equal(a, b)
    segs = np.concatenate([
        np.stack([np.stack([0.9 * s, 0.3 * s], 1), np.stack([0.3 * s, 0.9 * s], 1)], 1),
        rng.uniform(0, 1, (300, 2, 2)),
    ])
    for a, b in zip(g.intersect_edges(segs), o.intersect_edges(segs)):
        assert np.array_equal(a, b, equal_nan=True)
