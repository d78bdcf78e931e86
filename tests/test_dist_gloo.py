"""The multi-GPU host path on the CPU: two gloo ranks run the product's
ShardedCellTree (numba_celltree_gb300/sharded.py) -- the query sharding and
the ordered reassembly of per-query and pair results -- with a small numpy
stand-in answering each rank's range where a GPU replica would; the
reassembled results must equal the stand-in's answers for the whole batch
in one process.  Also: barrier and max-over-ranks of the timing."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class StandInTree:
    """Brute-force numpy answers with the shapes and ordering contracts of
    CellTree2d's queries (query-major pairs, -1 for no cell); no GPU."""

    def __init__(self, xy, faces):
        self.xy = np.asarray(xy, dtype=np.float64)
        self.faces = np.asarray(faces, dtype=np.int64)
        v = self.xy[self.faces]
        self.bb = np.stack([v[..., 0].min(1), v[..., 0].max(1), v[..., 1].min(1), v[..., 1].max(1)], 1)

    def _inside(self, p):
        a, b, c = (self.xy[self.faces[:, k]] for k in range(3))
        p = np.asarray(p, dtype=np.float64)
        ins = np.zeros((len(p), len(self.faces)), dtype=bool)
        for lo in range(0, len(p), 512):
            q = p[lo:lo + 512, None, :]
            s1 = (b[None, :, 0] - a[None, :, 0]) * (q[..., 1] - a[None, :, 1]) - \
                 (b[None, :, 1] - a[None, :, 1]) * (q[..., 0] - a[None, :, 0])
            s2 = (c[None, :, 0] - b[None, :, 0]) * (q[..., 1] - b[None, :, 1]) - \
                 (c[None, :, 1] - b[None, :, 1]) * (q[..., 0] - b[None, :, 0])
            s3 = (a[None, :, 0] - c[None, :, 0]) * (q[..., 1] - c[None, :, 1]) - \
                 (a[None, :, 1] - c[None, :, 1]) * (q[..., 0] - c[None, :, 0])
            ins[lo:lo + 512] = (s1 >= 0) & (s2 >= 0) & (s3 >= 0)
        return ins

    def locate_points(self, points, tolerance=None):
        ins = self._inside(points)
        return np.where(ins.any(1), ins.argmax(1), -1).astype(np.int64)

    def compute_barycentric_weights(self, points, tolerance=None):
        idx = self.locate_points(points)
        w = np.zeros((len(points), 3))
        w[idx >= 0, 0] = 1.0
        return idx, w

    def _box_pairs(self, boxes):
        boxes = np.asarray(boxes, dtype=np.float64)
        hit = ((boxes[:, None, 0] < self.bb[None, :, 1]) & (self.bb[None, :, 0] < boxes[:, None, 1]) &
               (boxes[:, None, 2] < self.bb[None, :, 3]) & (self.bb[None, :, 2] < boxes[:, None, 3]))
        return np.nonzero(hit)

    def locate_boxes(self, boxes):
        i, j = self._box_pairs(boxes)
        return i.astype(np.int64), j.astype(np.int64)

    def intersect_boxes(self, boxes):
        i, j = self.locate_boxes(boxes)
        b = np.asarray(boxes)[i]
        c = self.bb[j]
        area = ((np.minimum(b[:, 1], c[:, 1]) - np.maximum(b[:, 0], c[:, 0])) *
                (np.minimum(b[:, 3], c[:, 3]) - np.maximum(b[:, 2], c[:, 2])))
        return i, j, area

    def intersect_edges(self, edges):
        e = np.asarray(edges, dtype=np.float64)
        boxes = np.stack([e[:, :, 0].min(1), e[:, :, 0].max(1), e[:, :, 1].min(1), e[:, :, 1].max(1)], 1)
        i, j = self.locate_boxes(boxes)
        return i, j, e[i]

    def intersect_faces(self, vertices, faces, fill_value):
        v = np.asarray(vertices)[np.asarray(faces)]
        boxes = np.stack([v[..., 0].min(1), v[..., 0].max(1), v[..., 1].min(1), v[..., 1].max(1)], 1)
        return self.intersect_boxes(boxes)

    def locate_faces(self, vertices, faces):
        faces[...] = faces[:, ::-1]  # stands in for the in-place reorientation
        v = np.asarray(vertices)[faces]
        boxes = np.stack([v[..., 0].min(1), v[..., 0].max(1), v[..., 1].min(1), v[..., 1].max(1)], 1)
        return self.locate_boxes(boxes)


def _inputs():
    from numba_celltree_gb300 import synthetic as syn

    xy, f = syn.triangle_mesh(20, seed=1, extent=(20.0, 20.0))
    pts = syn.uniform_points(3001, xy.min(0) - 1, xy.max(0) + 1, seed=2)
    boxes = syn.random_boxes(777, xy.min(0), xy.max(0), 0.1, 5.0, seed=3)
    segs = syn.random_segments(301, xy.min(0), xy.max(0), seed=4)
    qxy, qf = syn.triangle_mesh(9, seed=5, extent=(20.0, 20.0))
    return xy, f, pts, boxes, segs, qxy, qf


def _answers(tree, pts, boxes, segs, qxy, qf):
    qf2 = qf.copy()
    out = {
        "locate_points": (tree.locate_points(pts),),
        "barycentric": tree.compute_barycentric_weights(pts),
        "locate_boxes": tree.locate_boxes(boxes),
        "intersect_boxes": tree.intersect_boxes(boxes),
        "intersect_edges": tree.intersect_edges(segs),
        "intersect_faces": tree.intersect_faces(qxy, qf, -1),
        "locate_faces": tree.locate_faces(qxy, qf2),
        "oriented_faces": (qf2,),
    }
    return {k: tuple(np.asarray(x) for x in v) for k, v in out.items()}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from numba_celltree_gb300 import _dist
    from numba_celltree_gb300.sharded import ShardedCellTree

    _dist.setup("gloo")
    xy, f, pts, boxes, segs, qxy, qf = _inputs()
    tree = ShardedCellTree(StandInTree(xy, f))
    res = _answers(tree, pts, boxes, segs, qxy, qf)
    mx = _dist.max_over_ranks(float(rank) + 0.5)
    _dist.barrier()
    q.put((rank, res, mx))
    dist.destroy_process_group()


def test_two_gloo_ranks_reassemble_single_process_results():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    xy, f, pts, boxes, segs, qxy, qf = _inputs()
    expected = _answers(StandInTree(xy, f), pts, boxes, segs, qxy, qf)
    for rank, res, mx in got:
        assert mx == 1.5
        for k, v in expected.items():
            assert len(res[k]) == len(v), k
            for a, b in zip(res[k], v):
                assert a.shape == b.shape and np.array_equal(a, b), (rank, k)


def test_split_ranges_cover_in_order():
    from numba_celltree_gb300 import _dist
    from numba_celltree_gb300.sharded import split_ranges

    for n in (0, 1, 7, 10, 1001):
        for ws in (1, 2, 3, 8):
            r = [_dist.shard(n, k, ws) for k in range(ws)]
            assert r == split_ranges(n, ws)
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(r[k][1] == r[k + 1][0] for k in range(ws - 1))
            assert max(e - s for s, e in r) - min(e - s for s, e in r) <= 1


def test_single_process_sharding_is_the_identity():
    """World size 1 (no process group): the sharded tree returns its replica's
    answers unchanged."""
    from numba_celltree_gb300.sharded import ShardedCellTree

    xy, f, pts, boxes, segs, qxy, qf = _inputs()
    a = _answers(ShardedCellTree(StandInTree(xy, f)), pts, boxes, segs, qxy, qf)
    b = _answers(StandInTree(xy, f), pts, boxes, segs, qxy, qf)
    for k in b:
        for x, y in zip(a[k], b[k]):
            assert np.array_equal(x, y), k
