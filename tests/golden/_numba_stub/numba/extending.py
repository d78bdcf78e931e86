def intrinsic(f):  # pragma: no cover - JIT-only path
    return f
