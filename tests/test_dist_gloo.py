"""The N > 1 host path on the CPU: two gloo ranks shard a batch of point and
box queries, each answers its range (the oracle stands in for the per-GPU
kernels), and the ordered gathers reassemble exactly the single-process
results; barrier and max-over-ranks of the timing."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


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
    from numba_celltree_gb300 import synthetic as syn
    from oracle import oracle as O

    _dist.setup("gloo")
    xy, f = syn.triangle_mesh(30, seed=1, extent=(30.0, 30.0))
    tree = O.OracleCellTree2d(xy, f, -1)
    pts = syn.uniform_points(10001, xy.min(0) - 1, xy.max(0) + 1, seed=2)
    boxes = syn.random_boxes(777, xy.min(0), xy.max(0), 0.1, 5.0, seed=3)
    a, b = _dist.shard(len(pts), rank, ws)
    full = _dist.gather_ordered(torch.as_tensor(tree.locate_points(pts[a:b])), len(pts))
    a, b = _dist.shard(len(boxes), rank, ws)
    bi, bj = tree.locate_boxes(boxes[a:b])
    gi, gj = _dist.gather_pairs(torch.as_tensor(bi), [torch.as_tensor(bj)], a)
    mx = _dist.max_over_ranks(float(rank) + 0.5)
    _dist.barrier()
    if rank == 0:
        q.put((full.numpy(), gi.numpy(), gj.numpy(), mx))
    dist.destroy_process_group()


def test_two_gloo_ranks_reassemble_single_process_results():
    import torch.multiprocessing as mp

    from numba_celltree_gb300 import _dist
    from numba_celltree_gb300 import synthetic as syn
    from oracle import oracle as O

    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, gi, gj, mx = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    xy, f = syn.triangle_mesh(30, seed=1, extent=(30.0, 30.0))
    tree = O.OracleCellTree2d(xy, f, -1)
    pts = syn.uniform_points(10001, xy.min(0) - 1, xy.max(0) + 1, seed=2)
    boxes = syn.random_boxes(777, xy.min(0), xy.max(0), 0.1, 5.0, seed=3)
    assert np.array_equal(full, tree.locate_points(pts))
    ri, rj = tree.locate_boxes(boxes)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    assert mx == 1.5


def test_shard_ranges_cover_in_order():
    from numba_celltree_gb300 import _dist

    for n in (0, 1, 7, 10, 1001):
        for ws in (1, 2, 3, 8):
            r = [_dist.shard(n, k, ws) for k in range(ws)]
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(r[k][1] == r[k + 1][0] for k in range(ws - 1))
            assert max(e - s for s, e in r) - min(e - s for s, e in r) <= 1
