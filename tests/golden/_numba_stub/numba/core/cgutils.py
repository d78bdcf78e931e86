def alloca_once(*args, **kwargs):  # pragma: no cover - JIT-only path
    raise NotImplementedError
