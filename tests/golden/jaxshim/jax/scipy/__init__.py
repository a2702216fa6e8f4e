from . import linalg, integrate  # noqa: F401
