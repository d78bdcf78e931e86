"""Minimal stand-in for the ``numba`` package.

It lets the pure-Python (JIT disabled) mode of the upstream package run in an
environment without numba: ``njit`` returns the function unchanged and
``prange`` is ``range``.  Only the names the upstream sources import are
provided.  Used by ``make_golden.py`` to generate golden fixtures.
"""

import os

os.environ.setdefault("NUMBA_DISABLE_JIT", "1")

from . import core, extending, types  # noqa: E402,F401


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(f):
        return f

    return wrap


jit = njit
prange = range


def get_num_threads():
    return 1


def int32(x):
    return int(x)


def carray(ptr, shape, dtype=None):  # pragma: no cover - JIT-only path
    raise NotImplementedError
