int64 = "int64"


def CPointer(t):  # pragma: no cover - JIT-only path
    return t
