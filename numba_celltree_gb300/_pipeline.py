"""Host-resident query batches: chunked, double-buffered host <-> device
streaming around a device query.

A batch of host points is cut into chunks.  Chunk c is copied to the device
on an upload stream, queried on the caller's current stream and its result
copied back on a download stream, so the upload of chunk c+1 and the
download of chunk c-1 overlap the query of chunk c.  Results land in pinned
host memory (the CUDA runtime copies into pageable memory through a single
staging thread, an order of magnitude slower than a DMA into pinned memory);
the returned numpy array is a view of that pinned block, which goes back to
PyTorch's pinned-block cache when the array is dropped.

Points in ordinary (pageable) memory are page-locked in place chunk by
chunk (``ct_host_register``; chunk boundaries moved onto page boundaries so
that every chunk owns its pages) just before their upload is enqueued, so
the registration of chunk c overlaps the upload and query of chunk c-1, and
all chunks are released after the last upload.  Registering 4 GB measured
7 to 21 ms on a Grace host against 35 ms for copying it into pinned memory,
and the upload then runs at the pinned rate.  Where registration is refused
(or the array is small, or not 16-byte aligned) the points are copied by
the host, all intra-op threads at once, into one of two pinned staging
blocks and uploaded from there; the host copy of chunk c+1 overlaps the
upload and query of chunk c.  Uploading straight from unregistered pageable
memory is as fast on the first call on a Grace host, but repeated calls on
the same array slowed down twenty-fold in measurements (the driver's
handling of pages the GPU has already read).
"""

from __future__ import annotations

import mmap
import warnings

import numpy as np

from . import _device

CHUNK_POINTS = 1 << 25  # largest chunk (512 MiB of float64 pairs)
FIRST_CHUNK = 1 << 22   # the first (and the last) chunks are small: the GPU starts
                        # after a short upload and the last download is short


def chunk_bounds(n: int, chunk: int, first: int = None):
    """Chunk boundaries [(s, e), ...]: sizes ramp up by doubling from `first`
    to `chunk`, stay at `chunk`, and ramp down by halving at the end."""
    first = min(FIRST_CHUNK if first is None else first, chunk)
    if n <= 0:
        return []
    sizes = []
    m = first
    rest = n
    while rest > 0 and m < chunk:
        take = min(m, rest)
        sizes.append(take)
        rest -= take
        m *= 2
    tail = []
    while rest > 2 * chunk:
        sizes.append(chunk)
        rest -= chunk
    # the last <= 2 chunks: halve down to `first`
    while rest > first:
        half = rest // 2
        tail.append(rest - half)
        rest = half
    if rest > 0:
        tail.append(rest)
    return_sizes = sizes + tail
    out, s = [], 0
    for k in return_sizes:
        out.append((s, s + k))
        s += k
    return out


REGISTER_MIN_BYTES = 64 << 20  # smaller arrays go through the staging copy


def page_cuts(addr: int, itemsize: int, bounds, page: int = mmap.PAGESIZE):
    """Chunk bounds with every cut between two chunks moved up to the next
    row that starts on a page boundary of the host block at `addr` (rows of
    `itemsize` bytes), so that each chunk owns whole pages apart from the
    block's first and last page; None when no row starts on a page boundary."""
    if not bounds:
        return []
    if page % itemsize or addr % itemsize:
        return None
    step = page // itemsize
    s0 = ((-addr) % page) // itemsize  # rows whose start is page aligned: s0 + k * step
    n = bounds[-1][1]
    cuts = []
    for s, _ in bounds[1:]:
        c = s + ((s0 - s) % step)
        if 0 < c < n and (not cuts or c > cuts[-1]):
            cuts.append(c)
    edges = [0] + cuts + [n]
    return list(zip(edges[:-1], edges[1:]))


class InPlacePins:
    """Byte ranges of a host array page-locked in place (whole pages), all
    released together."""

    def __init__(self, read_only: bool):
        from . import _lib

        self.lib = _lib.load()
        self.read_only = int(bool(read_only))
        self.bases = []

    def pin(self, start: int, end: int, page: int = mmap.PAGESIZE) -> bool:
        a = start - start % page
        b = -(-end // page) * page
        if self.lib.ct_host_register(a, b - a, self.read_only) != 0:
            return False
        self.bases.append(a)
        return True

    def release(self) -> None:
        for a in self.bases:
            self.lib.ct_host_unregister(a)
        self.bases = []


def pinned_empty(shape, dtype):
    """Pinned host tensor (PyTorch's cached pinned allocator)."""
    torch = _device.torch()
    return torch.empty(shape, dtype=dtype, pin_memory=True)


COMPUTE_STREAMS = 2  # chunks queried on alternating streams
BUFFERS = 3  # device buffers (points and results) the chunks rotate through


def stream_points(points: np.ndarray, device, query, out_dtype, chunk=None) -> np.ndarray:
    """Run ``query(points_d, out_d, slot)`` over `points` (n, 2) float64 host
    array in chunks; returns the concatenated results as a numpy array over
    pinned memory.  ``query`` enqueues work on the current stream and must
    not synchronise; consecutive chunks run on COMPUTE_STREAMS streams in
    turn (slot = the stream's number), so that one chunk's kernels fill the
    tail of the previous chunk's -- calls with different slots may run at
    the same time and must not share scratch memory."""
    torch = _device.torch()
    chunk = CHUNK_POINTS if chunk is None else int(chunk)
    n = int(points.shape[0])
    out_h = pinned_empty((n,), out_dtype)
    if n == 0:
        return out_h.numpy()
    with warnings.catch_warnings():
        # a read-only array: the tensor over it is only ever read
        warnings.simplefilter("ignore", UserWarning)
        src = torch.from_numpy(points)
    compute = torch.cuda.current_stream(device)
    up = torch.cuda.Stream(device)
    down = torch.cuda.Stream(device)
    computes = [compute]
    for _ in range(COMPUTE_STREAMS - 1):
        cs = torch.cuda.Stream(device)
        cs.wait_stream(compute)  # work the caller enqueued before (e.g. the tree build)
        computes.append(cs)
    bounds = chunk_bounds(n, chunk)
    pin_in = src.is_pinned()
    pins = None
    addr = points.ctypes.data
    if not pin_in and points.nbytes >= REGISTER_MIN_BYTES and points.flags.c_contiguous:
        aligned = page_cuts(addr, 16, bounds)
        if aligned is not None:
            bounds = aligned
            pins = InPlacePins(read_only=not points.flags.writeable)
    m = max(e - s for s, e in bounds)
    nbuf = min(max(2, BUFFERS), len(bounds))
    p_d = [torch.empty((m, 2), dtype=torch.float64, device=device) for _ in range(nbuf)]
    o_d = [torch.empty((m,), dtype=out_dtype, device=device) for _ in range(nbuf)]
    stage = None  # pinned staging blocks, allocated when a chunk needs them
    staged = [None] * nbuf  # upload that last read staging block b
    done = [None] * nbuf  # query of the chunk that last used buffer b
    fetched = [None] * nbuf  # download of the chunk that last used buffer b
    registering = pins is not None
    try:
        for c, (s, e) in enumerate(bounds):
            b = c % nbuf
            k = e - s
            direct = pin_in
            if registering:
                direct = pins.pin(addr + 16 * s, addr + 16 * e)
                registering = direct  # once refused, the rest goes through the staging copy
            if not direct:
                if stage is None:
                    stage = [pinned_empty((m, 2), torch.float64) for _ in range(nbuf)]
                # host copy into the pinned staging block (its last upload must be done)
                if staged[b] is not None:
                    staged[b].synchronize()
                stage[b][:k].copy_(src[s:e])
                up_src = stage[b][:k]
            else:
                up_src = src[s:e]
            with torch.cuda.stream(up):
                if done[b] is not None:
                    up.wait_event(done[b])
                p_d[b][:k].copy_(up_src, non_blocking=True)
                uploaded = torch.cuda.Event()
                uploaded.record(up)
                staged[b] = uploaded
            slot = c % len(computes)
            cs = computes[slot]
            cs.wait_event(uploaded)
            if fetched[b] is not None:
                cs.wait_event(fetched[b])
            with torch.cuda.stream(cs):
                query(p_d[b][:k], o_d[b][:k], slot)
            ev = torch.cuda.Event()
            ev.record(cs)
            done[b] = ev
            with torch.cuda.stream(down):
                down.wait_event(ev)
                out_h[s:e].copy_(o_d[b][:k], non_blocking=True)
                ev2 = torch.cuda.Event()
                ev2.record(down)
                fetched[b] = ev2
        down.synchronize()
        for cs in computes:
            cs.synchronize()
            if cs is not compute:
                compute.wait_stream(cs)
    finally:
        if pins is not None:
            up.synchronize()  # no upload may still read a registered page
            pins.release()
    return out_h.numpy()
