"""Types and constants (constants.py of the upstream package, 23-151)."""

from typing import NamedTuple

import numpy as np

IntDType = np.intp
FloatDType = np.float64

MAX_N_VERTEX = 32  # constants.py:134
FILL_VALUE = -1  # constants.py:135
MIN_TOLERANCE = 1e-15  # constants.py:146
TOLERANCE_FACTOR = 1e-12  # constants.py:147
MAX_N_BUCKETS = 32  # the GPU builder keeps per-bucket state in one warp

# NodeDType constants.py:92-106 (packed, 41 bytes)
NodeDType = np.dtype(
    [
        ("child", IntDType),
        ("Lmax", FloatDType),
        ("Rmin", FloatDType),
        ("ptr", IntDType),
        ("size", IntDType),
        ("dim", bool),
    ]
)


class CellTreeData(NamedTuple):
    """constants.py:82-89 -- host (numpy) view of a tree."""

    elements: np.ndarray
    vertices: np.ndarray
    nodes: np.ndarray
    bb_indices: np.ndarray
    bb_coords: np.ndarray
    bbox: np.ndarray
    cells_per_leaf: int
