"""Replicas on several devices of one process (MultiDeviceCellTree): two
replicas on the one GPU of this machine each answer half of every batch;
the reassembled results must equal a single CellTree2d's, for every query
kind, with numpy and with CUDA inputs."""

import numpy as np
import pytest

from numba_celltree_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_two_replicas_reassemble_single_tree_results():
    import torch

    from numba_celltree_gb300 import CellTree2d
    from numba_celltree_gb300.sharded import MultiDeviceCellTree, ShardedCellTree

    xy, f = syn.mixed_mesh(80, seed=101, extent=(80.0, 80.0))
    one = CellTree2d(xy, f, -1)
    multi = MultiDeviceCellTree.build(xy, f, -1, devices=[0, 0])
    lo, hi = xy.min(0), xy.max(0)
    pts = syn.uniform_points(100_001, lo, hi, seed=102, margin=0.02)
    boxes = syn.random_boxes(5_001, lo, hi, 0.1, 6.0, seed=103)
    segs = syn.random_segments(2_001, lo, hi, seed=104)
    for tree in (multi, ShardedCellTree(one)):
        for inp in (pts, torch.as_tensor(pts, device="cuda")):
            got = tree.locate_points(inp)
            assert isinstance(got, type(inp))
            assert np.array_equal(np.asarray(got.cpu() if hasattr(got, "cpu") else got), one.locate_points(pts))
        for a, b in zip(tree.compute_barycentric_weights(pts), one.compute_barycentric_weights(pts)):
            assert np.array_equal(a, b)
        for a, b in zip(tree.locate_boxes(boxes), one.locate_boxes(boxes)):
            assert np.array_equal(a, b)
        for a, b in zip(tree.intersect_boxes(boxes), one.intersect_boxes(boxes)):
            assert np.array_equal(a, b)
        for a, b in zip(tree.intersect_edges(segs), one.intersect_edges(segs)):
            assert np.array_equal(a, b, equal_nan=True)
