"""Key-seeded NumPy draws standing in for jax.random; every draw is logged."""
import numpy as _np

DRAWS = []


def PRNGKey(seed):
    return _np.array([0, int(seed) & 0xFFFFFFFF], dtype=_np.uint32)


def _rng(key):
    k = _np.asarray(key, dtype=_np.uint64)
    return _np.random.default_rng(_np.random.SeedSequence([int(k[0]), int(k[1])]))


def split(key, num=2):
    k = _np.asarray(key)
    st = _np.random.SeedSequence([int(k[0]), int(k[1]), 7]).generate_state(2 * num)
    return st.reshape(num, 2).astype(_np.uint32)


def normal(key, shape=(), dtype=None):
    v = _rng(key).standard_normal(shape)
    DRAWS.append(("normal", tuple(int(x) for x in _np.asarray(key)), v))
    return v


def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
    v = minval + (maxval - minval) * _rng(key).random(shape)
    DRAWS.append(("uniform", tuple(int(x) for x in _np.asarray(key)), v))
    return v
