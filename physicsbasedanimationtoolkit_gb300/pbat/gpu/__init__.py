from . import vbd  # noqa: F401
