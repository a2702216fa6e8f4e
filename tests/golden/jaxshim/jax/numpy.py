"""jax.numpy restated on NumPy with float64 as the default float type."""
import builtins as _bi

import numpy as _np
from numpy import *  # noqa: F401,F403
from numpy import linalg  # noqa: F401

float64 = _np.float64
float32 = _np.float64       # the golden run is FP64 throughout
int32 = _np.int32
ndarray = _np.ndarray


def array(obj, dtype=None):
    if isinstance(obj, (list, tuple)):
        parts = [_np.asarray(o) for o in obj]
        if _bi.any(_np.iscomplexobj(p) for p in parts):
            return _np.array([_np.asarray(p, dtype=_np.complex128) for p in parts], dtype=dtype)
    a = _np.array(obj, dtype=dtype)
    if dtype is None and a.dtype == _np.float32:
        a = a.astype(_np.float64)
    return a


def asarray(obj, dtype=None):
    return array(obj, dtype=dtype)


def clip(a, a_min=None, a_max=None, min=None, max=None):
    lo = a_min if a_min is not None else min
    hi = a_max if a_max is not None else max  # noqa: A001
    return _np.clip(a, lo, hi)


def fabs(x):
    return _np.abs(x)


def where(c, x=None, y=None):
    if x is None:
        return _np.where(c)
    return _np.where(c, x, y)


def take_jax(a, idx):
    idx = _np.asarray(idx)
    return _np.asarray(a)[_np.where(idx < 0, idx + len(a), idx)]
