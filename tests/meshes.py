"""Small seeded meshes shared by the parity tests."""

import pathlib

import numpy as np

from numba_celltree_gb300 import synthetic as syn

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def golden_data():
    return np.load(GOLDEN / "reference_data.npz")


def meshes():
    d = golden_data()
    out = {
        "triplot": (d["xy"], d["triangles"]),
        "voronoi": (d["voronoi_xy"], d["voronoi"]),
        "tri20": syn.triangle_mesh(20, seed=0),
        "tri150": syn.triangle_mesh(150, seed=3),
        "quad40": syn.quad_mesh(40, seed=4),
        "mixed60": syn.mixed_mesh(60, seed=5),
        "utm80": syn.triangle_mesh(80, seed=6, extent=(80.0, 80.0), offset=(5.0e5, 4.2e6)),
        "rot_quads": syn.quad_mesh(30, seed=7, extent=(100.0, 100.0), rotate_deg=7.0),
    }
    return out
