"""The exported helpers of the upstream package that no query calls, as
batched GPU kernels (``csrc/ct_extra.cu``).

* ``liang_barsky_line_box_clip`` (algorithms/liang_barsky.py:10-64): the
  upstream scalar signature ``(a, b, box) -> (bool, Point, Point)``, and
  ``liang_barsky_line_box_clip_batch`` for arrays of segments and boxes;
* ``points_in_triangles`` (geometry_utils.py:273-289).
"""

from __future__ import annotations

from typing import NamedTuple

import numpy as np

from . import _device, _lib
from .cast import is_cuda_tensor


class Point(NamedTuple):  # constants.py Point
    x: float
    y: float


def _dev(x, dtype):
    torch = _device.torch()
    dev = _device.require_cuda()
    return _device.to_device(x, dtype, dev)


def liang_barsky_line_box_clip_batch(a, b, boxes):
    """Segments (a[i], b[i]) clipped by boxes[i] (xmin, xmax, ymin, ymax):
    ``(ok, c, d)`` with NaN points where ``ok`` is false.  CUDA tensors in,
    CUDA tensors out; numpy in, numpy out."""
    torch = _device.torch()
    cuda_in = is_cuda_tensor(a)
    a_d = _dev(np.asarray(a, dtype=np.float64) if not cuda_in else a, torch.float64).reshape(-1, 2).contiguous()
    b_d = _dev(np.asarray(b, dtype=np.float64) if not is_cuda_tensor(b) else b, torch.float64).reshape(-1, 2)
    x_d = _dev(np.asarray(boxes, dtype=np.float64) if not is_cuda_tensor(boxes) else boxes, torch.float64)
    b_d, x_d = b_d.contiguous(), x_d.reshape(-1, 4).contiguous()
    n = int(a_d.shape[0])
    if b_d.shape[0] != n or x_d.shape[0] != n:
        raise ValueError("a, b and boxes must have the same number of rows")
    ok = torch.empty((n,), dtype=torch.uint8, device=a_d.device)
    c = torch.empty((n, 2), dtype=torch.float64, device=a_d.device)
    d = torch.empty((n, 2), dtype=torch.float64, device=a_d.device)
    _lib.check(_lib.load().ct_liang_barsky_line_box_clip(_device.ptr(a_d), _device.ptr(b_d), _device.ptr(x_d), n,
                                                        _device.ptr(ok), _device.ptr(c), _device.ptr(d),
                                                        _device.stream()), "liang_barsky")
    ok = ok.bool()
    if cuda_in:
        return ok, c, d
    return ok.cpu().numpy(), c.cpu().numpy(), d.cpu().numpy()


def liang_barsky_line_box_clip(a, b, box):
    """liang_barsky_line_box_clip (liang_barsky.py:10-64) of one segment."""
    ok, c, d = liang_barsky_line_box_clip_batch(np.asarray([a], dtype=np.float64), np.asarray([b], dtype=np.float64),
                                                np.asarray([box], dtype=np.float64))
    return bool(ok[0]), Point(float(c[0, 0]), float(c[0, 1])), Point(float(d[0, 0]), float(d[0, 1]))


def points_in_triangles(points, face_indices, faces, vertices, tolerance: float):
    """points_in_triangles (geometry_utils.py:273-289): for every point,
    whether it lies in (or within ``tolerance`` of the edges of) triangle
    ``faces[face_indices[i]]``."""
    torch = _device.torch()
    cuda_in = is_cuda_tensor(points)
    p = _dev(points, torch.float64).reshape(-1, 2).contiguous()
    fi = _dev(face_indices, torch.int64).reshape(-1).contiguous()
    f = _dev(faces, torch.int64).contiguous()
    v = _dev(vertices, torch.float64).contiguous()
    n = int(p.shape[0])
    if fi.shape[0] != n:
        raise ValueError("one face index per point")
    out = torch.empty((n,), dtype=torch.uint8, device=p.device)
    err = torch.zeros((1,), dtype=torch.int32, device=p.device)
    _lib.check(_lib.load().ct_points_in_triangles(_device.ptr(p), _device.ptr(fi), n, _device.ptr(f), int(f.shape[1]),
                                                 int(f.shape[0]), _device.ptr(v), float(tolerance), _device.ptr(out),
                                                 _device.ptr(err), _device.stream()), "points_in_triangles")
    if int(err.item()):
        raise IndexError("face index out of range")
    out = out.bool()
    return out if cuda_in else out.cpu().numpy()
