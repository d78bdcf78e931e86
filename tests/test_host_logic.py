"""Host-side logic that needs no GPU: the chunk schedule of the host-batch
pipeline."""

from numba_celltree_gb300._pipeline import chunk_bounds


def test_chunk_bounds_cover_in_order_and_ramp():
    for chunk in (1000, 4096, 1 << 25):
        for n in (0, 1, 7, 999, 1000, 1001, 4_194_304, 10_000_000, 268_435_456, 100_000_001):
            b = chunk_bounds(n, chunk)
            if n == 0:
                assert b == []
                continue
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(len(b) - 1))
            sizes = [e - s for s, e in b]
            assert all(0 < k <= chunk for k in sizes)
    sizes = [e - s for s, e in chunk_bounds(268_435_456, 1 << 25)]
    assert sizes[0] == 1 << 22 and sizes[-1] <= 1 << 22 and max(sizes) == 1 << 25
