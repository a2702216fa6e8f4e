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


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v):
        out = _np.array(self.arr, copy=True).view(JArray)
        out[self.idx] = v
        return out

    def add(self, v):
        out = _np.array(self.arr, copy=True).view(JArray)
        out[self.idx] += v
        return out

    def get(self):
        return _np.asarray(self.arr)[self.idx]


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


class JArray(_np.ndarray):
    """An ndarray with JAX's functional update syntax, x.at[idx].set(v) / .add(v)."""

    @property
    def at(self):
        return _At(self)


def zeros(shape, dtype=None):
    return _np.zeros(shape, dtype=dtype if dtype is not None else _np.float64).view(JArray)


def zeros_like(a, dtype=None):
    return _np.zeros_like(_np.asarray(a), dtype=dtype).view(JArray)
