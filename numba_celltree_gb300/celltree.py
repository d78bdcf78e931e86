"""CellTree2d on the GPU -- drop-in for numba_celltree.CellTree2d
(celltree.py:37-351 upstream)."""

from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import _device, _lib
from .cast import cast_faces, cast_vertices, is_cuda_tensor
from .celltree_base import CellTree2dBase, _GpuTree, _validate_params, validate_elements


def _as_output(t, like_cuda: bool):
    return t if like_cuda else t.cpu().numpy()


class CellTree2d(CellTree2dBase):
    """
    Construct a cell tree from 2D vertices and a faces indexing array.

    Parameters
    ----------
    vertices: ndarray of floats with shape ``(n_point, 2)``
        Corner coordinates (x, y) of the cells.  A CUDA tensor is used in place.
    faces: ndarray of integers with shape ``(n_face, n_max_vert)``
        For every face the indices of its corner nodes; shorter faces are
        padded with ``fill_value``.
    fill_value: int
        Fill value marking empty nodes in ``faces``.
    n_buckets: int, optional, default: 4
        Buckets used in tree construction, 2 <= n_buckets <= 32.
    cells_per_leaf: int, optional, default: 2
        Number of cells in the leaf nodes.

    Results are identical to the upstream package: the same ``nodes`` and
    ``bb_indices`` arrays, the same cells for every query.  Queries given numpy
    arrays return numpy arrays; queries given CUDA tensors return CUDA tensors.
    ``precision`` selects the point-location form: ``"fp32"`` (float32
    traversal and leaf filter with exact float64 fallback, the default) or
    ``"fp64"`` (plain float64); both return identical indices.
    """

    _elements_name = "faces"

    def __init__(self, vertices, faces, fill_value: int, n_buckets: int = 4, cells_per_leaf: int = 2):
        _validate_params(n_buckets, cells_per_leaf)
        device = _device.require_cuda()
        torch = _device.torch()
        vertices = cast_vertices(vertices, copy=True)
        faces = cast_faces(faces, fill_value)
        v_d = _device.to_device(vertices, torch.float64, device)
        f_d = _device.to_device(faces, torch.int64, device)
        if f_d.shape[1] < 3 and f_d.shape[0] > 0:
            raise ValueError("faces must have at least 3 columns")
        if f_d.shape[0] == 0:
            raise ValueError("zero-size array to reduction operation minimum which has no identity")
        validate_elements(f_d, int(v_d.shape[0]), 3, "faces")
        lib = _lib.load()
        st = _device.stream()
        n, K = int(f_d.shape[0]), int(f_d.shape[1])
        # counter_clockwise geometry_utils.py:541-561, build_face_bboxes 443-456
        _lib.check(lib.ct_counter_clockwise(_device.ptr(v_d), _device.ptr(f_d), n, K, st), "counter_clockwise")
        bb = _device.empty((n, 4), torch.float64, device)
        _lib.check(lib.ct_face_bboxes(_device.ptr(v_d), _device.ptr(f_d), n, K, _device.ptr(bb), st), "face_bboxes")
        self._tree = _GpuTree(device, f_d, v_d, bb, n_buckets, cells_per_leaf)
        self._host = {}
        self.n_buckets = n_buckets
        self.cells_per_leaf = cells_per_leaf
        self.precision = "fp32"

    @property
    def faces(self) -> np.ndarray:
        return self._cached("faces", lambda: self._tree.elements.cpu().numpy())

    def default_tolerance(self) -> float:
        return self._tolerance(None)

    def launch_locate(self, points_dev, out_dev, tolerance: float, precision: str = "fp32") -> None:
        """Enqueue locate_points on the current stream for device-resident
        float64 points (n, 2) and an int64 output (n,); no synchronisation and
        no error-word check (for pipelines and timing loops)."""
        mode = _lib.CT_MODE_FP64 if precision == "fp64" else _lib.CT_MODE_FP32
        _lib.check(
            _lib.load().ct_locate_points(
                ctypes.byref(self._tree.desc), _device.ptr(points_dev), int(points_dev.shape[0]), float(tolerance),
                mode, _device.ptr(out_dev), _device.stream(),
            ),
            "locate_points",
        )

    def locate_points(self, points, tolerance: Optional[float] = None):
        """
        Find the index of a face that contains a point (query.py:110-117).

        Points that are very close near an edge of a face will also be
        identified as falling within that face.  Returns -1 for points that
        fall in no face.
        """
        tol = self._tolerance(tolerance)
        cuda_in = is_cuda_tensor(points)
        points = cast_vertices(points)
        t = self._tree
        torch = _device.torch()
        p_d = _device.to_device(points, torch.float64, t.device)
        n = int(p_d.shape[0])
        out = _device.empty((n,), torch.int64, t.device)
        mode = _lib.CT_MODE_FP64 if self.precision == "fp64" else _lib.CT_MODE_FP32
        t.reset_error()
        _lib.check(
            _lib.load().ct_locate_points(
                ctypes.byref(t.desc), _device.ptr(p_d), n, tol, mode, _device.ptr(out), _device.stream()
            ),
            "locate_points",
        )
        t.raise_on_device_error()
        return _as_output(out, cuda_in)
