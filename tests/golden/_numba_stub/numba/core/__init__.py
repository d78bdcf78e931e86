from . import cgutils  # noqa: F401
