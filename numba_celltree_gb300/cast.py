"""Input casting with the upstream rules (cast.py:14-54).

Host inputs (numpy arrays, lists) are cast with numpy exactly like upstream,
including the ValueError messages; CUDA tensors are cast on the device.
"""

from __future__ import annotations

import numpy as np

from .constants import FILL_VALUE, MAX_N_VERTEX, FloatDType, IntDType


def is_cuda_tensor(x) -> bool:
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor) and x.is_cuda


def cast_vertices(vertices, copy: bool = False):
    if is_cuda_tensor(vertices):
        import torch

        v = vertices.to(torch.float64)
        if copy and v.data_ptr() == vertices.data_ptr():
            v = v.clone()
        if v.ndim != 2 or v.shape[1] != 2:
            raise ValueError("vertices must have shape (n_points, 2)")
        return v.contiguous()
    if isinstance(vertices, np.ndarray):
        vertices = vertices.astype(FloatDType, copy=copy)
    else:
        vertices = np.ascontiguousarray(vertices, dtype=FloatDType)
    if vertices.ndim != 2 or vertices.shape[1] != 2:
        raise ValueError("vertices must have shape (n_points, 2)")
    return np.ascontiguousarray(vertices)


def cast_faces(faces, fill_value: int):
    if is_cuda_tensor(faces):
        import torch

        f = faces.to(torch.int64).clone()
        if f.ndim != 2:
            raise ValueError("faces must have shape (n_face, n_max_vert)")
        if f.shape[1] > MAX_N_VERTEX:
            raise ValueError(
                f"faces contains up to {f.shape[1]} vertices for a single face. "
                f"numba_celltree supports a maximum of {MAX_N_VERTEX} vertices."
            )
        if fill_value != FILL_VALUE:
            f[f == fill_value] = FILL_VALUE
        return f.contiguous()
    if isinstance(faces, np.ndarray):
        faces = faces.astype(IntDType, copy=True)
    else:
        faces = np.ascontiguousarray(faces, dtype=IntDType)
    if faces.ndim != 2:
        raise ValueError("faces must have shape (n_face, n_max_vert)")
    _, n_max_vert = faces.shape
    if n_max_vert > MAX_N_VERTEX:
        raise ValueError(
            f"faces contains up to {n_max_vert} vertices for a single face. "
            f"numba_celltree supports a maximum of {MAX_N_VERTEX} vertices. "
            f"Increase MAX_N_VERTEX in the source code, or alter the mesh."
        )
    if fill_value != FILL_VALUE:
        faces[faces == fill_value] = FILL_VALUE
    return np.ascontiguousarray(faces)


def cast_bboxes(bbox_coords):
    if is_cuda_tensor(bbox_coords):
        import torch

        b = bbox_coords.to(torch.float64).contiguous()
        if b.ndim != 2 or b.shape[1] != 4:
            raise ValueError("bbox_coords must have shape (n_box, 4)")
        return b
    bbox_coords = np.ascontiguousarray(bbox_coords, dtype=FloatDType)
    if bbox_coords.ndim != 2 or bbox_coords.shape[1] != 4:
        raise ValueError("bbox_coords must have shape (n_box, 4)")
    return bbox_coords


def cast_edges(edges):
    if is_cuda_tensor(edges):
        import torch

        e = edges.to(torch.float64).contiguous()
        if e.ndim != 3 or e.shape[1] != 2 or e.shape[2] != 2:
            raise ValueError("edges must have shape (n_edge, 2, 2)")
        return e
    edges = np.ascontiguousarray(edges, dtype=FloatDType)
    if edges.ndim != 3 or edges.shape[1] != 2 or edges.shape[2] != 2:
        raise ValueError("edges must have shape (n_edge, 2, 2)")
    return edges
