from . import geometry, vbd  # noqa: F401
