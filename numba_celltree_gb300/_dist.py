"""Host-side plumbing for one process per GPU (torch.distributed).

Queries are independent, so a batch shards into contiguous ranges with no
collective on the data path: every rank holds a replica of the tree and
queries its own range.  The only exchanges are for reassembling results in
query order -- an all-gather of the per-rank result blocks, and for
multi-result queries (pairs) first of the per-rank pair counts -- and the
barrier / max-over-ranks of timing.  NCCL when CUDA is available, gloo
otherwise (the CPU tests run two gloo ranks).
"""

from __future__ import annotations

import os
from typing import Tuple


def world() -> Tuple[int, int, int]:
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def setup(backend: str = None) -> Tuple[int, int, int]:
    """Initialise the process group when world_size > 1 (MASTER_ADDR /
    MASTER_PORT from the environment)."""
    import torch
    import torch.distributed as dist

    ws, rank, local = world()
    if ws > 1 and not dist.is_initialized():
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend, rank=rank, world_size=ws)
    return ws, rank, local


def _device():
    import torch
    import torch.distributed as dist

    if dist.is_initialized() and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(v: float) -> float:
    import torch
    import torch.distributed as dist

    if not dist.is_initialized() or dist.get_world_size() == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(n: int, rank: int, world_size: int) -> Tuple[int, int]:
    """Contiguous range [start, end) of n queries for `rank` (sizes differ by
    at most one)."""
    base, extra = divmod(n, world_size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_ordered(local, n: int):
    """Concatenate every rank's block of a per-query result (rank order =
    query order).  `local` is this rank's block (torch tensor, first dim =
    its shard length); every rank returns the full result."""
    import torch
    import torch.distributed as dist

    if not dist.is_initialized() or dist.get_world_size() == 1:
        return local
    ws = dist.get_world_size()
    dev = _device()
    m = max(shard(n, r, ws)[1] - shard(n, r, ws)[0] for r in range(ws))
    pad = torch.zeros((m,) + tuple(local.shape[1:]), dtype=local.dtype, device=dev)
    pad[: local.shape[0]] = local.to(dev)
    parts = [torch.empty_like(pad) for _ in range(ws)]
    dist.all_gather(parts, pad)
    out = [parts[r][: shard(n, r, ws)[1] - shard(n, r, ws)[0]] for r in range(ws)]
    return torch.cat(out)


def gather_pairs(ii_local, others, start: int):
    """Multi-result queries: this rank's pairs (query indices relative to its
    shard `start`, query-major) and parallel arrays `others`; returns the
    pairs of all ranks with global query indices, query-major.  One
    all-gather of the pair counts, one of the (padded) pair blocks."""
    import torch
    import torch.distributed as dist

    ii = ii_local + start
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return (ii,) + tuple(others)
    ws = dist.get_world_size()
    dev = _device()
    cnt = torch.tensor([ii.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.empty_like(cnt) for _ in range(ws)]
    dist.all_gather(counts, cnt)
    counts = [int(c.item()) for c in counts]
    m = max(max(counts), 1)
    res = []
    for a in (ii,) + tuple(others):
        pad = torch.zeros((m,) + tuple(a.shape[1:]), dtype=a.dtype, device=dev)
        pad[: a.shape[0]] = a.to(dev)
        parts = [torch.empty_like(pad) for _ in range(ws)]
        dist.all_gather(parts, pad)
        res.append(torch.cat([parts[r][: counts[r]] for r in range(ws)]))
    return tuple(res)
