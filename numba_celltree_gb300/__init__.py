"""GB300-native cell tree: a drop-in for numba_celltree's CellTree2d and
EdgeCellTree2d whose construction and queries run as hand-written sm_103a
CUDA kernels (libcelltree_gb300.so)."""

from .batch import CellTreeBatch
from .celltree import CellTree2d
from .edge_celltree import EdgeCellTree2d
from .sharded import MultiDeviceCellTree, ShardedCellTree

__version__ = "0.2.0"

__all__ = ("CellTree2d", "CellTreeBatch", "EdgeCellTree2d", "MultiDeviceCellTree", "ShardedCellTree")
