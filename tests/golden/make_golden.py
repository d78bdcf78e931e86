"""Generate the golden fixtures from the upstream numba_celltree package.

Runs the upstream package in its own pure-Python mode (NUMBA_DISABLE_JIT=1,
the mode its CI uses for coverage) with the small numba stand-in in
``_numba_stub/``, on seeded inputs, and stores inputs and outputs as npz:

* ``reference_data.npz``: the mesh files of the upstream test-suite
  (tests/data/xy.txt, triangles.txt, voronoi_xy.txt, voronoi.txt).
* ``golden_trees.npz``: per case the tree (NodeDType fields, bb_indices,
  bb_coords, ccw faces) and the results of every query.

Usage (needs the upstream sources; not needed to run the tests):

    python tests/golden/make_golden.py /path/to/numba_celltree
"""

from __future__ import annotations

import os
import pathlib
import sys

HERE = pathlib.Path(__file__).resolve().parent
os.environ["NUMBA_DISABLE_JIT"] = "1"
sys.dont_write_bytecode = True


def main(upstream: str) -> None:
    sys.path.insert(0, str(HERE / "_numba_stub"))
    sys.path.insert(0, upstream)
    sys.path.insert(0, str(HERE.parents[1]))
    import numpy as np
    from numba_celltree import CellTree2d, EdgeCellTree2d

    from numba_celltree_gb300 import synthetic as syn

    data = pathlib.Path(upstream) / "tests" / "data"
    ref = {
        "xy": np.loadtxt(data / "xy.txt", dtype=float),
        "triangles": np.loadtxt(data / "triangles.txt", dtype=np.int64),
        "voronoi_xy": np.loadtxt(data / "voronoi_xy.txt", dtype=float),
        "voronoi": np.loadtxt(data / "voronoi.txt", dtype=np.int64),
    }
    np.savez_compressed(HERE / "reference_data.npz", **ref)

    meshes = {
        "triplot": (ref["xy"], ref["triangles"]),
        "voronoi": (ref["voronoi_xy"], ref["voronoi"]),
        "tri20": syn.triangle_mesh(20, seed=0),
        "quad15": syn.quad_mesh(15, seed=1),
        "mixed20": syn.mixed_mesh(20, seed=2),
        "utm12": syn.triangle_mesh(12, seed=3, extent=(12.0, 12.0), offset=(5.0e5, 4.2e6)),
    }
    params = {
        "triplot": [(4, 2), (2, 1), (3, 3)],
        "voronoi": [(4, 2), (2, 1)],
        "tri20": [(4, 2), (4, 1), (8, 3)],
        "quad15": [(4, 2), (5, 1)],
        "mixed20": [(4, 2), (2, 2)],
        "utm12": [(4, 2)],
    }
    out = {}
    rng = np.random.default_rng(2024)
    ci = 0
    for name, (xy, faces) in meshes.items():
        lo, hi = xy.min(0), xy.max(0)
        span = hi - lo
        pts = np.concatenate(
            [
                rng.uniform(lo - 0.05 * span, hi + 0.05 * span, size=(400, 2)),
                xy[rng.integers(0, len(xy), 40)],
                syn.near_edge_points(xy, faces[:, :3], 60, dist=1e-9 * float(span.max()), seed=ci),
            ]
        )
        c = rng.uniform(lo, hi, size=(60, 2))
        s = rng.uniform(0.01, 0.25, size=(60, 2)) * span
        boxes = np.stack([c[:, 0], c[:, 0] + s[:, 0], c[:, 1], c[:, 1] + s[:, 1]], axis=1)
        edges = np.concatenate([rng.uniform(lo, hi, size=(40, 2, 2)), xy[faces[:10, :2]]])
        qv = rng.uniform(lo, hi, size=(24, 2))
        qf = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8], [9, 10, 11], [12, 13, 14], [15, 16, 17], [2, 5, 20]])
        for nb, cpl in params[name]:
            t = CellTree2d(xy, faces, -1, nb, cpl)
            p = f"c{ci}_"
            out[p + "name"] = np.array(name)
            out[p + "params"] = np.array([nb, cpl])
            out[p + "vertices"] = xy
            out[p + "faces_in"] = faces
            out[p + "faces"] = t.faces
            for f in t.nodes.dtype.names:
                out[p + "node_" + f] = t.nodes[f]
            out[p + "bb_indices"] = t.bb_indices
            out[p + "bb_coords"] = t.bb_coords
            out[p + "bbox"] = t.bbox
            out[p + "points"] = pts
            out[p + "locate"] = t.locate_points(pts)
            out[p + "locate_tol"] = t.locate_points(pts, 1e-3 * float(span.max()))
            out[p + "boxes"] = boxes
            i, j = t.locate_boxes(boxes)
            out[p + "box_i"], out[p + "box_j"] = i, j
            i, j, a = t.intersect_boxes(boxes)
            out[p + "ibox_i"], out[p + "ibox_j"], out[p + "ibox_a"] = i, j, a
            out[p + "edges"] = edges
            i, j, x = t.intersect_edges(edges)
            out[p + "edge_i"], out[p + "edge_j"], out[p + "edge_xy"] = i, j, x
            out[p + "qv"] = qv
            out[p + "qf"] = qf
            i, j, a = t.intersect_faces(qv, qf, -1)
            out[p + "face_i"], out[p + "face_j"], out[p + "face_a"] = i, j, a
            qf2 = qf.astype(np.int64).copy()
            i, j = t.locate_faces(qv.copy(), qf2)
            out[p + "lface_i"], out[p + "lface_j"] = i, j
            idx, w = t.compute_barycentric_weights(pts)
            out[p + "bary_i"], out[p + "bary_w"] = idx, w
            out[p + "node_bounds"] = t.node_bounds
            out[p + "node_valid"] = t.validate_node_bounds()
            ci += 1
    # edge trees
    ev = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [2.0, 1.0]])
    ee = np.array([[0, 1], [1, 2], [2, 3]])
    xy, f = syn.triangle_mesh(10, seed=9)
    e2 = np.unique(np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1), axis=0)
    ecases = [("edges3", ev, ee, 4, 2), ("grid_edges", xy, e2, 4, 2), ("grid_edges1", xy, e2, 2, 1)]
    for k, (name, v, e, nb, cpl) in enumerate(ecases):
        t = EdgeCellTree2d(v, e, nb, cpl)
        p = f"e{k}_"
        out[p + "name"] = np.array(name)
        out[p + "params"] = np.array([nb, cpl])
        out[p + "vertices"] = v
        out[p + "edges"] = e
        for fld in t.nodes.dtype.names:
            out[p + "node_" + fld] = t.nodes[fld]
        out[p + "bb_indices"] = t.bb_indices
        out[p + "bb_coords"] = t.bb_coords
        pts = np.concatenate([rng.uniform(-0.1, 1.1, size=(200, 2)) * (v.max(0) - v.min(0)) + v.min(0), v,
                              0.5 * (v[e[:, 0]] + v[e[:, 1]])])
        out[p + "points"] = pts
        out[p + "locate"] = t.locate_points(pts)
        segs = np.concatenate([rng.uniform(v.min(0), v.max(0), size=(40, 2, 2)), v[e[:6]]])
        out[p + "segs"] = segs
        i, j, x = t.intersect_edges(segs)
        out[p + "edge_i"], out[p + "edge_j"], out[p + "edge_xy"] = i, j, x
    out["n_cases"] = np.array(ci)
    out["n_edge_cases"] = np.array(len(ecases))
    np.savez_compressed(HERE / "golden_trees.npz", **out)
    print(f"wrote {ci} face cases and {len(ecases)} edge cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
