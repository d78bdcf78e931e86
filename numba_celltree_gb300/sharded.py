"""Several GPUs answering one query batch (no upstream counterpart; upstream
splits a batch into chunks for its threads, query.py:278-289).

Queries are independent, so a batch shards into contiguous ranges with no
exchange on the data path: every GPU holds a replica of the tree (built on
it from the same mesh -- replicas, not a distributed build) and answers its
own range; results are put back together in query order.  Per-query results
(cell index, barycentric weights) are concatenated; pair results (boxes,
faces, segments) are concatenated range by range with the query indices
shifted by the range start, which keeps upstream's query-major order.

* ``ShardedCellTree`` -- one process per GPU under ``torch.distributed``
  (NCCL on GPUs, gloo on CPUs): every rank calls the same method with the
  whole batch and gets the whole result; ranks exchange only their results
  (``_dist.gather_ordered`` / ``_dist.gather_pairs``).
* ``MultiDeviceCellTree`` -- one process driving several devices: each
  device's range runs on its own replica and stream, results are moved to
  the first device (or returned as numpy when the input was numpy).

Both wrap any object with the query methods of ``CellTree2d`` (the replica),
so the sharding and reassembly are independent of the kernels behind them.
"""

from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _dist


def split_ranges(n: int, parts: int) -> List[Tuple[int, int]]:
    """Contiguous ranges [start, end) of n queries for `parts` workers (sizes
    differ by at most one)."""
    return [_dist.shard(n, k, parts) for k in range(parts)]


def _torch():
    import torch

    return torch


def _as_tensor(x):
    torch = _torch()
    return x if isinstance(x, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(x))


def _like_input(x, like):
    """numpy when the query input was numpy, else a tensor."""
    torch = _torch()
    if isinstance(like, torch.Tensor):
        return x
    return x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


class ShardedCellTree:
    """A tree replicated on every rank of a torch.distributed job.

    ``tree`` is this rank's replica (e.g. ``CellTree2d`` built on the rank's
    GPU); every rank must call each query method with the same arguments.
    """

    def __init__(self, tree):
        self.tree = tree

    @classmethod
    def build(cls, vertices, faces, fill_value: int, n_buckets: int = 4, cells_per_leaf: int = 2):
        """Initialise the process group from the launcher's environment (if
        needed), select this rank's GPU and build the replica on it."""
        from .celltree import CellTree2d

        torch = _torch()
        _, _, local = _dist.setup()
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        return cls(CellTree2d(vertices, faces, fill_value, n_buckets, cells_per_leaf))

    @staticmethod
    def _range(n: int) -> Tuple[int, int]:
        ws, rank, _ = _dist.world()
        return _dist.shard(n, rank, ws)

    def _per_query(self, fn, queries, *args):
        n = int(queries.shape[0])
        s, e = self._range(n)
        local = fn(queries[s:e], *args)
        if isinstance(local, tuple):
            return tuple(_like_input(_dist.gather_ordered(_as_tensor(x), n), queries) for x in local)
        return _like_input(_dist.gather_ordered(_as_tensor(local), n), queries)

    def _pairs(self, fn, queries, *args):
        n = int(queries.shape[0])
        s, e = self._range(n)
        res = fn(queries[s:e], *args)
        out = _dist.gather_pairs(_as_tensor(res[0]), [_as_tensor(x) for x in res[1:]], s)
        return tuple(_like_input(x, queries) for x in out)

    def locate_points(self, points, tolerance: Optional[float] = None):
        return self._per_query(self.tree.locate_points, points, tolerance)

    def compute_barycentric_weights(self, points, tolerance: Optional[float] = None):
        return self._per_query(self.tree.compute_barycentric_weights, points, tolerance)

    def locate_boxes(self, bbox_coords):
        return self._pairs(self.tree.locate_boxes, bbox_coords)

    def intersect_boxes(self, bbox_coords):
        return self._pairs(self.tree.intersect_boxes, bbox_coords)

    def intersect_edges(self, edge_coords):
        return self._pairs(self.tree.intersect_edges, edge_coords)

    def intersect_faces(self, vertices, faces, fill_value: int):
        return self._pairs(lambda f: self.tree.intersect_faces(vertices, f, fill_value), faces)

    def locate_faces(self, vertices, faces):
        """Like upstream, a numpy ``faces`` argument is reoriented in place
        (every rank receives the whole reoriented array)."""
        n = int(faces.shape[0])
        s, e = self._range(n)
        mine = faces[s:e].copy() if isinstance(faces, np.ndarray) else faces[s:e].clone()
        res = self.tree.locate_faces(vertices, mine)
        out = _dist.gather_pairs(_as_tensor(res[0]), [_as_tensor(res[1])], s)
        oriented = _dist.gather_ordered(_as_tensor(mine), n)
        if isinstance(faces, np.ndarray):
            faces[...] = oriented.cpu().numpy().astype(faces.dtype, copy=False)
        else:
            faces.copy_(oriented.to(faces.device, faces.dtype))
        return tuple(_like_input(x, faces) for x in out)


class MultiDeviceCellTree:
    """Replicas of one tree on several devices of this process; every query
    batch is split into contiguous ranges, one per replica, which run on
    their own devices and streams at the same time."""

    def __init__(self, replicas: Sequence, devices: Sequence):
        if len(replicas) != len(devices) or not replicas:
            raise ValueError("one replica per device")
        self.replicas = list(replicas)
        self.devices = list(devices)

    @classmethod
    def build(cls, vertices, faces, fill_value: int, devices: Sequence = None, n_buckets: int = 4,
              cells_per_leaf: int = 2):
        """Build one replica per device (default: every visible GPU)."""
        from .celltree import CellTree2d

        torch = _torch()
        if devices is None:
            devices = list(range(torch.cuda.device_count()))
        devs = [torch.device("cuda", d) if isinstance(d, int) else torch.device(d) for d in devices]
        reps = []
        for d in devs:
            with torch.cuda.device(d):
                reps.append(CellTree2d(vertices, faces, fill_value, n_buckets, cells_per_leaf))
        return cls(reps, devs)

    def _run(self, name, queries, *args):
        """Each replica's range on its device and stream; results of each in
        range order (moved to the first device)."""
        torch = _torch()
        n = int(queries.shape[0])
        parts = []
        for (s, e), rep, d in zip(split_ranges(n, len(self.replicas)), self.replicas, self.devices):
            with torch.cuda.device(d):
                q = queries[s:e]
                if isinstance(q, torch.Tensor):
                    q = q.to(d)
                parts.append((s, getattr(rep, name)(q, *args)))
        return parts

    def _gather(self, x):
        torch = _torch()
        return x.to(self.devices[0]) if isinstance(x, torch.Tensor) else _as_tensor(x)

    def _per_query(self, name, queries, *args):
        torch = _torch()
        parts = self._run(name, queries, *args)
        if isinstance(parts[0][1], tuple):
            k = len(parts[0][1])
            res = tuple(torch.cat([self._gather(p[1][j]) for p in parts]) for j in range(k))
            return tuple(_like_input(r, queries) for r in res)
        return _like_input(torch.cat([self._gather(p[1]) for p in parts]), queries)

    def _pairs(self, name, queries, *args):
        torch = _torch()
        parts = self._run(name, queries, *args)
        k = len(parts[0][1])
        out = [torch.cat([self._gather(res[0]) + s for s, res in parts])]
        out += [torch.cat([self._gather(res[j]) for _, res in parts]) for j in range(1, k)]
        return tuple(_like_input(x, queries) for x in out)

    def locate_points(self, points, tolerance: Optional[float] = None):
        return self._per_query("locate_points", points, tolerance)

    def compute_barycentric_weights(self, points, tolerance: Optional[float] = None):
        return self._per_query("compute_barycentric_weights", points, tolerance)

    def locate_boxes(self, bbox_coords):
        return self._pairs("locate_boxes", bbox_coords)

    def intersect_boxes(self, bbox_coords):
        return self._pairs("intersect_boxes", bbox_coords)

    def intersect_edges(self, edge_coords):
        return self._pairs("intersect_edges", edge_coords)
