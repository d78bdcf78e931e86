"""Regridding with the intersection queries' output (no upstream
counterpart; the upstream example builds a dense weight matrix,
examples/spatial_indexing_2d_grids.py:245-313).

``WeightMatrix.from_intersections(i, j, area, n_rows, n_cols)`` takes the
query-major pairs of ``intersect_faces`` / ``intersect_boxes`` (row = query
face or box, column = tree face, weight = area of overlap) as a CSR matrix on
the GPU; ``mean(x)`` is the area-weighted mean of column values per row (NaN
where a row overlaps nothing), ``weight_sum`` the overlapping area per row.
"""

from __future__ import annotations

import numpy as np

from . import _device, _lib
from .cast import is_cuda_tensor


class WeightMatrix:
    def __init__(self, row_ptr, cols, weights, n_rows: int, n_cols: int):
        self.row_ptr = row_ptr
        self.cols = cols
        self.weights = weights
        self.n_rows = int(n_rows)
        self.n_cols = int(n_cols)

    @classmethod
    def from_intersections(cls, rows, cols, weights, n_rows: int, n_cols: int) -> "WeightMatrix":
        torch = _device.torch()
        dev = _device.require_cuda()
        r = _device.to_device(rows, torch.int64, dev).reshape(-1).contiguous()
        c = _device.to_device(cols, torch.int64, dev).reshape(-1).contiguous()
        w = _device.to_device(weights, torch.float64, dev).reshape(-1).contiguous()
        if not (r.shape[0] == c.shape[0] == w.shape[0]):
            raise ValueError("rows, cols and weights must have the same length")
        lib = _lib.load()
        row_ptr = torch.empty((int(n_rows) + 1,), dtype=torch.int64, device=dev)
        nbytes = int(lib.ct_csr_workspace_size(int(n_rows)))
        ws = torch.empty((nbytes,), dtype=torch.uint8, device=dev)
        err = torch.zeros((1,), dtype=torch.int32, device=dev)
        _lib.check(lib.ct_csr_row_ptr(_device.ptr(r), int(r.shape[0]), int(n_rows), _device.ptr(row_ptr),
                                      _device.ptr(ws), nbytes, _device.ptr(err), _device.stream()), "csr")
        e = int(err.item())
        if e & 1:
            raise ValueError("row index out of range")
        if e & 2:
            raise ValueError("rows must be non-decreasing (query-major pairs)")
        return cls(row_ptr, c, w, n_rows, n_cols)

    def _apply(self, x):
        torch = _device.torch()
        x_d = _device.to_device(x, torch.float64, self.row_ptr.device).reshape(-1).contiguous()
        if x_d.shape[0] != self.n_cols:
            raise ValueError(f"x must have {self.n_cols} values")
        mean = torch.empty((self.n_rows,), dtype=torch.float64, device=x_d.device)
        wsum = torch.empty((self.n_rows,), dtype=torch.float64, device=x_d.device)
        err = torch.zeros((1,), dtype=torch.int32, device=x_d.device)
        _lib.check(_lib.load().ct_csr_weighted_mean(
            _device.ptr(self.row_ptr), _device.ptr(self.cols), _device.ptr(self.weights), self.n_rows, self.n_cols,
            _device.ptr(x_d), _device.ptr(mean), _device.ptr(wsum), _device.ptr(err), _device.stream()), "mean")
        if int(err.item()):
            raise ValueError("column index out of range")
        return mean, wsum

    def mean(self, x):
        """Area-weighted mean of ``x`` (one value per column) for every row."""
        m, _ = self._apply(x)
        return m if is_cuda_tensor(x) else m.cpu().numpy()

    @property
    def weight_sum(self):
        torch = _device.torch()
        _, w = self._apply(torch.zeros((self.n_cols,), dtype=torch.float64, device=self.row_ptr.device))
        return w

    def to_scipy(self):
        """The matrix as ``scipy.sparse.csr_matrix`` (host)."""
        import scipy.sparse as sp

        return sp.csr_matrix((self.weights.cpu().numpy(), self.cols.cpu().numpy(), self.row_ptr.cpu().numpy()),
                             shape=(self.n_rows, self.n_cols))
