"""Device plumbing: PyTorch supplies device memory (caching allocator) and the
current CUDA stream; all compute is done by libcelltree_gb300."""

from __future__ import annotations

import numpy as np


def torch():
    import torch as _torch

    return _torch


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("numba_celltree_gb300 needs a CUDA GPU (sm_103a); none is available")
    return t.device("cuda", t.cuda.current_device())


def stream() -> int:
    return torch().cuda.current_stream().cuda_stream


def empty(shape, dtype, device):
    return torch().empty(shape, dtype=dtype, device=device)


def to_device(x, dtype, device):
    """numpy / list / tensor -> contiguous CUDA tensor of `dtype`."""
    t = torch()
    if isinstance(x, t.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    arr = np.ascontiguousarray(x)
    h = t.from_numpy(arr)
    return h.to(device=device, dtype=dtype, non_blocking=False).contiguous()


def ptr(x) -> int:
    return 0 if x is None else int(x.data_ptr())
