"""Launch-shape autotuner (no upstream counterpart).

The library's kernels take a few launch shapes that change their speed but
never their results: how finely the batched point location sorts its queries
(``sort_bits``), the occupancy the candidate-list kernel is compiled for
(``cells_bpsm``), the grid of the open-query traversal (``fast_bpsm``), the
block size and work ordering of the box and segment traversals, the stack of
the plain float64 form, and the density of the start-node grid and candidate
lists built with a tree (``grid_density``).  The best choice depends on the
GPU, on the mesh (size, cells per leaf) and on the batch, so a tuner times
the candidates on a sample of a real call the first time a problem of that
size class is seen, and keeps the fastest in a small JSON cache keyed by GPU
and problem bucket (log2 of the cell and query counts):

* ``NUMBA_CELLTREE_GB300_TUNING`` -- path of the cache file (default
  ``~/.cache/numba_celltree_gb300/tuning.json``);
* ``NUMBA_CELLTREE_GB300_AUTOTUNE`` -- ``1`` (default) tunes at first use,
  ``0`` uses cached entries and the library defaults only.

``cells_per_leaf`` and ``n_buckets`` shape the tree itself (its ``nodes`` and
``bb_indices``, which must equal the upstream package's for the same
arguments), so they are tuned only when the caller asks for it:
``CellTree2d(..., cells_per_leaf="auto")`` picks the leaf size whose tree
locates a sample of query points fastest (see ``tune_leaf_size``).
"""

from __future__ import annotations

import itertools
import json
import math
import os
import pathlib
import statistics
import tempfile
import threading
from typing import Callable, Dict, Iterable, List, Optional

CACHE_ENV = "NUMBA_CELLTREE_GB300_TUNING"
MODE_ENV = "NUMBA_CELLTREE_GB300_AUTOTUNE"
FORMAT = 1

# the library defaults (what a call uses without a cache entry)
DEFAULTS: Dict[str, dict] = {
    "locate": {"sort_bits": None, "cells_bpsm": 6, "fast_bpsm": 16},
    "fp64": {"stack": 0},
    "boxes": {"threads": 256, "work_order": None, "job_cells": 0},
    "segments": {"threads": 128, "work_order": None, "split": None},
    "index": {"grid_density": 1.0},
}

# candidate values per knob
SPACE: Dict[str, Dict[str, list]] = {
    "locate": {"sort_bits": [0, 8, 16, 24], "cells_bpsm": [4, 6, 8], "fast_bpsm": [8, 16, 32]},
    "fp64": {"stack": [0, 512]},
    "boxes": {"threads": [64, 128, 256], "work_order": [False, True]},
    "segments": {"threads": [64, 128], "work_order": [False, True]},
    "index": {"grid_density": [0.5, 1.0, 2.0]},
}

# batches from which a call tunes itself at first use (smaller ones run the
# defaults: tuning them would cost more than it saves)
TUNE_MIN = {"locate": 1 << 20, "fp64": 1 << 20, "boxes": 1 << 16, "segments": 1 << 16}
# queries of the sample a tuning run times
SAMPLE_MAX = {"locate": 1 << 22, "fp64": 1 << 20, "boxes": 1 << 16, "segments": 1 << 15}


def enabled() -> bool:
    return os.environ.get(MODE_ENV, "1").strip() not in ("0", "false", "no", "off")


def bucket(n: int) -> int:
    """Size class of a count: log2 rounded to the nearest integer (0 for n <= 1)."""
    n = int(n)
    return 0 if n <= 1 else int(round(math.log2(n)))


def cache_key(kind: str, gpu: str, cells: int, queries: int, **extra) -> str:
    parts = [kind, gpu, f"c{bucket(cells)}", f"q{bucket(queries)}"]
    parts += [f"{k}{extra[k]}" for k in sorted(extra)]
    return "|".join(parts)


def gpu_name(device=None) -> str:
    """GPU model, SM count and compute capability of `device` (the current
    CUDA device by default)."""
    import torch

    p = torch.cuda.get_device_properties(device if device is not None else torch.cuda.current_device())
    return f"{p.name}|sm{p.multi_processor_count}|cc{p.major}.{p.minor}"


def candidates(kind: str, fixed: Optional[dict] = None) -> List[dict]:
    """Every combination of the knobs of `kind` (knobs in `fixed` held)."""
    space = dict(SPACE[kind])
    for k, v in (fixed or {}).items():
        space[k] = [v]
    names = sorted(space)
    return [dict(zip(names, vals)) for vals in itertools.product(*(space[k] for k in names))]


class TuningCache:
    """JSON file of tuned launch shapes: {"format": 1, "entries": {key: {...}}}.
    Reads tolerate a missing or damaged file (it is then rewritten); writes
    replace the file atomically, merging with entries other processes wrote."""

    def __init__(self, path=None):
        self.path = pathlib.Path(path or os.environ.get(CACHE_ENV) or
                                 pathlib.Path.home() / ".cache" / "numba_celltree_gb300" / "tuning.json")
        self._lock = threading.Lock()
        self._mem: Optional[Dict[str, dict]] = None

    def _read(self) -> Dict[str, dict]:
        try:
            d = json.loads(self.path.read_text())
            if isinstance(d, dict) and d.get("format") == FORMAT and isinstance(d.get("entries"), dict):
                return {k: v for k, v in d["entries"].items() if isinstance(v, dict)}
        except (OSError, ValueError):
            pass
        return {}

    def entries(self) -> Dict[str, dict]:
        with self._lock:
            if self._mem is None:
                self._mem = self._read()
            return dict(self._mem)

    def get(self, key: str) -> Optional[dict]:
        return self.entries().get(key)

    def put(self, key: str, value: dict) -> None:
        with self._lock:
            merged = self._read()
            merged[key] = value
            self._mem = merged
            try:
                self.path.parent.mkdir(parents=True, exist_ok=True)
                fd, tmp = tempfile.mkstemp(prefix=".tuning", dir=str(self.path.parent))
                with os.fdopen(fd, "w") as f:
                    json.dump({"format": FORMAT, "entries": merged}, f, indent=1, sort_keys=True)
                os.replace(tmp, self.path)
            except OSError:
                pass  # a read-only home: keep the result for this process only


_cache: Optional[TuningCache] = None


def cache() -> TuningCache:
    global _cache
    want = os.environ.get(CACHE_ENV)
    if _cache is None or (want and pathlib.Path(want) != _cache.path):
        _cache = TuningCache()
    return _cache


def pick(timings: Iterable[tuple]) -> tuple:
    """(config, ms) with the smallest time; ties keep the first."""
    best = None
    for cfg, ms in timings:
        if best is None or ms < best[1]:
            best = (cfg, ms)
    if best is None:
        raise ValueError("no candidate timed")
    return best


def time_gpu(fn: Callable[[], None], reps: int = 3) -> float:
    """Median milliseconds of `fn` (which enqueues GPU work on the current
    stream) over `reps` runs after one warm-up, CUDA events on that stream."""
    import torch

    st = torch.cuda.current_stream()
    fn()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def tune(kind: str, key: str, run: Callable[[dict], None], cands: List[dict], reps: int = 3,
         store: bool = True, default: Optional[dict] = None) -> dict:
    """Time `run(cfg)` for every candidate and return (and cache) the fastest:
    {"config": cfg, "ms": t, "default_ms": t0, "candidates": n}; `default`
    is the configuration a call would use untuned (its time is reported)."""
    timed = [(c, time_gpu(lambda c=c: run(c), reps)) for c in cands]
    best, ms = pick(timed)
    dflt = default if default is not None else DEFAULTS[kind]
    d_ms = next((t for c, t in timed if all(c.get(k) == dflt.get(k) for k in c)), None)
    entry = {"config": best, "ms": round(ms, 4), "default_ms": None if d_ms is None else round(d_ms, 4),
             "candidates": len(cands)}
    if store:
        cache().put(key, entry)
    return entry


def lookup(kind: str, key: str) -> dict:
    """Cached configuration for `key` merged over the defaults of `kind`."""
    cfg = dict(DEFAULTS[kind])
    e = cache().get(key)
    if e and isinstance(e.get("config"), dict):
        cfg.update({k: v for k, v in e["config"].items() if k in cfg})
    return cfg
