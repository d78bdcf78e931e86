"""Seeded synthetic meshes and query sets with the shapes of the benchmark
workloads (no external datasets exist for this domain).

All coordinates are float64 and all generators take a numpy seed, so the
same arguments always give the same arrays.
"""

from __future__ import annotations

import numpy as np


def jittered_grid(nx: int, ny: int = None, seed: int = 0, extent=(1.0, 1.0), offset=(0.0, 0.0),
                  jitter: float = 0.2):
    """Vertices of an (nx+1) x (ny+1) lattice on [0, ex] x [0, ey] + offset with
    interior vertices jittered uniformly by +-jitter cell widths."""
    ny = nx if ny is None else ny
    rng = np.random.default_rng(seed)
    hx, hy = extent[0] / nx, extent[1] / ny
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = i.ravel() * hx
    y = j.ravel() * hy
    inner = (i.ravel() > 0) & (i.ravel() < nx) & (j.ravel() > 0) & (j.ravel() < ny)
    k = int(inner.sum())
    x[inner] += rng.uniform(-jitter * hx, jitter * hx, size=k)
    y[inner] += rng.uniform(-jitter * hy, jitter * hy, size=k)
    xy = np.stack([x + offset[0], y + offset[1]], axis=1)
    return xy


def _quads(nx: int, ny: int):
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    v0 = (j * (nx + 1) + i).ravel()
    return np.stack([v0, v0 + 1, v0 + nx + 2, v0 + nx + 1], axis=1)


def triangle_mesh(nx: int, ny: int = None, seed: int = 0, extent=(1.0, 1.0), offset=(0.0, 0.0), jitter=0.2):
    """Jittered grid with every quad split into two triangles (int64, K=3)."""
    ny = nx if ny is None else ny
    xy = jittered_grid(nx, ny, seed, extent, offset, jitter)
    q = _quads(nx, ny)
    tri = np.empty((2 * q.shape[0], 3), dtype=np.int64)
    tri[0::2] = q[:, [0, 1, 2]]
    tri[1::2] = q[:, [0, 2, 3]]
    return xy, tri


def quad_mesh(nx: int, ny: int = None, seed: int = 0, extent=(1.0, 1.0), offset=(0.0, 0.0), jitter=0.2,
              rotate_deg: float = 0.0):
    ny = nx if ny is None else ny
    xy = jittered_grid(nx, ny, seed, extent, (0.0, 0.0), jitter)
    if rotate_deg:
        a = np.deg2rad(rotate_deg)
        c, s = np.cos(a), np.sin(a)
        cx, cy = extent[0] / 2, extent[1] / 2
        x, y = xy[:, 0] - cx, xy[:, 1] - cy
        xy = np.stack([c * x - s * y + cx, s * x + c * y + cy], axis=1)
    xy = xy + np.asarray(offset, dtype=np.float64)
    return xy, _quads(nx, ny).astype(np.int64)


def _convex(poly_xy: np.ndarray) -> bool:
    n = len(poly_xy)
    s = 0
    for k in range(n):
        a, b, c = poly_xy[k], poly_xy[(k + 1) % n], poly_xy[(k + 2) % n]
        cr = (b[0] - a[0]) * (c[1] - b[1]) - (b[1] - a[1]) * (c[0] - b[0])
        if cr < 0:
            return False
        s += cr > 0
    return s >= 3


def mixed_mesh(nx: int, ny: int = None, seed: int = 0, extent=(1.0, 1.0), split_frac=0.3, merge_frac=0.1):
    """Mixed polygon mesh (K=6, fill -1): a jittered quad grid in which a
    fraction of quads is split into two triangles and a fraction of
    horizontally adjacent quad pairs is merged into convex hexagons (or a
    triangle + quad into a pentagon) when the merge is convex."""
    ny = nx if ny is None else ny
    rng = np.random.default_rng(seed + 1000)
    xy = jittered_grid(nx, ny, seed, extent)
    q = _quads(nx, ny)
    nq = q.shape[0]
    used = np.zeros(nq, dtype=bool)
    faces = []
    # merges: quad (i, j) with its right neighbour (i+1, j)
    cand = rng.permutation(nq)[: int(merge_frac * nq)]
    for c in cand:
        i = c % nx
        if i == nx - 1 or used[c] or used[c + 1]:
            continue
        a, b = q[c], q[c + 1]
        # a: v0 v1 v2 v3 ; b: w0=v1 w1 w2 w3=v2  ->  hexagon v0 v1 w1 w2 v2 v3
        hexa = [a[0], a[1], b[1], b[2], a[2], a[3]]
        if rng.random() < 0.5:
            # pentagon: triangle (v0 v2 v3) removed -> keep v0 v1 w1 w2 v2 and triangle v0 v2 v3
            penta = [a[0], a[1], b[1], b[2], a[2]]
            if _convex(xy[penta]):
                faces.append(penta + [-1])
                faces.append([a[0], a[2], a[3], -1, -1, -1])
                used[c] = used[c + 1] = True
                continue
        if _convex(xy[hexa]):
            faces.append(hexa)
            used[c] = used[c + 1] = True
    rest = np.nonzero(~used)[0]
    split = rng.random(len(rest)) < split_frac
    for c, s in zip(rest, split):
        v = q[c]
        if s:
            faces.append([v[0], v[1], v[2], -1, -1, -1])
            faces.append([v[0], v[2], v[3], -1, -1, -1])
        else:
            faces.append([v[0], v[1], v[2], v[3], -1, -1])
    faces = np.asarray(faces, dtype=np.int64)
    order = rng.permutation(len(faces))
    return xy, faces[order]


def uniform_points(n: int, lo, hi, seed: int = 0, margin: float = 0.0):
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    span = hi - lo
    return rng.uniform(lo - margin * span, hi + margin * span, size=(n, 2))


def near_edge_points(xy, faces, n: int, dist: float, seed: int = 0):
    """Points within `dist` of random face edges and vertices."""
    rng = np.random.default_rng(seed)
    f = faces[rng.integers(0, len(faces), size=n)]
    k = rng.integers(0, 3, size=n)
    a = xy[f[np.arange(n), k]]
    b = xy[f[np.arange(n), (k + 1) % 3]]
    t = rng.random(n)
    t[rng.random(n) < 0.2] = 0.0  # on vertices
    p = a + t[:, None] * (b - a)
    p += rng.uniform(-dist, dist, size=(n, 2))
    return p


def random_boxes(n: int, lo, hi, side_lo: float, side_hi: float, seed: int = 0, log_uniform: bool = False):
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    c = rng.uniform(lo, hi, size=(n, 2))
    if log_uniform:
        s = np.exp(rng.uniform(np.log(side_lo), np.log(side_hi), size=(n, 2)))
    else:
        s = rng.uniform(side_lo, side_hi, size=(n, 2))
    return np.stack([c[:, 0], c[:, 0] + s[:, 0], c[:, 1], c[:, 1] + s[:, 1]], axis=1)


def random_segments(n: int, lo, hi, seed: int = 0):
    rng = np.random.default_rng(seed)
    return rng.uniform(np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64), size=(n, 2, 2))
