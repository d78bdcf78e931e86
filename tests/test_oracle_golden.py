"""The oracle (C restatement) against fixtures produced by the upstream
package itself (tests/golden/make_golden.py): bit-exact trees and queries."""

import numpy as np
import pytest

from meshes import GOLDEN

G = np.load(GOLDEN / "golden_trees.npz")
N_CASES = int(G["n_cases"])
N_EDGE = int(G["n_edge_cases"])


def case(i):
    p = f"c{i}_"
    return {k[len(p):]: G[k] for k in G.files if k.startswith(p)}


def ecase(i):
    p = f"e{i}_"
    return {k[len(p):]: G[k] for k in G.files if k.startswith(p)}


def assert_same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape
    if a.dtype.kind == "f":
        assert np.array_equal(a, b, equal_nan=True)
    else:
        assert np.array_equal(a, b)


@pytest.mark.parametrize("i", range(N_CASES))
def test_oracle_tree_and_queries(oracle, i):
    c = case(i)
    nb, cpl = (int(x) for x in c["params"])
    t = oracle.OracleCellTree2d(c["vertices"], c["faces_in"], -1, nb, cpl)
    assert_same(t.faces, c["faces"])
    for f in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        assert_same(t.nodes[f], c["node_" + f])
    assert_same(t.bb_indices, c["bb_indices"])
    assert_same(t.bb_coords, c["bb_coords"])
    assert_same(t.bbox, c["bbox"])
    assert_same(t.locate_points(c["points"]), c["locate"])
    span = float((c["vertices"].max(0) - c["vertices"].min(0)).max())
    assert_same(t.locate_points(c["points"], 1e-3 * span), c["locate_tol"])
    i_, j_ = t.locate_boxes(c["boxes"])
    assert_same(i_, c["box_i"])
    assert_same(j_, c["box_j"])
    for got, key in zip(t.intersect_boxes(c["boxes"]), ("ibox_i", "ibox_j", "ibox_a")):
        assert_same(got, c[key])
    for got, key in zip(t.intersect_edges(c["edges"]), ("edge_i", "edge_j", "edge_xy")):
        assert_same(got, c[key])
    for got, key in zip(t.intersect_faces(c["qv"], c["qf"], -1), ("face_i", "face_j", "face_a")):
        assert_same(got, c[key])
    qf = c["qf"].astype(np.int64).copy()
    for got, key in zip(t.locate_faces(c["qv"].copy(), qf), ("lface_i", "lface_j")):
        assert_same(got, c[key])
    for got, key in zip(t.compute_barycentric_weights(c["points"]), ("bary_i", "bary_w")):
        assert_same(got, c[key])
    assert_same(t.node_bounds, c["node_bounds"])
    assert_same(t.validate_node_bounds(), c["node_valid"])


@pytest.mark.parametrize("i", range(N_EDGE))
def test_oracle_edge_tree(oracle, i):
    c = ecase(i)
    nb, cpl = (int(x) for x in c["params"])
    t = oracle.OracleEdgeCellTree2d(c["vertices"], c["edges"], nb, cpl)
    for f in ("child", "Lmax", "Rmin", "ptr", "size", "dim"):
        assert_same(t.nodes[f], c["node_" + f])
    assert_same(t.bb_indices, c["bb_indices"])
    assert_same(t.bb_coords, c["bb_coords"])
    assert_same(t.locate_points(c["points"]), c["locate"])
    for got, key in zip(t.intersect_edges(c["segs"]), ("edge_i", "edge_j", "edge_xy")):
        assert_same(got, c[key])
