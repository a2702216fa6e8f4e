"""A NumPy (float64) restatement of the JAX primitives that the reference's
model-evaluation modules call, used only to execute those modules in a
container without JAX and record golden vectors.

Semantics restated (JAX 0.7.2 as pinned by the reference's README):
  jit                identity (no tracing)
  vmap               a Python loop over the mapped axis, outputs stacked
  grad               exact derivative by the complex-step method,
                     d f / d x_i = Im f(x + i h e_i) / h with h = 1e-30, which
                     is exact to rounding for the analytic potentials used here
  lax.scan / map     Python loops; lax.cond / switch evaluate the chosen branch
  ops.segment_sum    scatter-add that drops ids outside [0, num_segments)
  random.*           keys are uint32 pairs; draws come from NumPy generators
                     seeded by the key and every draw is logged in
                     ``random.DRAWS`` so the golden script can hand the same
                     numbers to the oracle (threefry itself is not restated)
"""
import numpy as _np

from . import numpy, lax, ops, random, scipy, nn, debug  # noqa: F401


def jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _index(x, i, ax):
    if ax is None:
        return x
    if isinstance(x, dict):
        return {k: _index(v, i, ax) for k, v in x.items()}
    if isinstance(x, (tuple, list)):
        return type(x)(_index(v, i, ax) for v in x)
    return _np.take(_np.asarray(x), i, axis=ax)


def _size(x, ax):
    if isinstance(x, dict):
        return _size(next(iter(x.values())), ax)
    if isinstance(x, (tuple, list)):
        return _size(x[0], ax)
    return _np.asarray(x).shape[ax]


def _stack(outs):
    first = outs[0]
    if isinstance(first, dict):
        return {k: _stack([o[k] for o in outs]) for k in first}
    if isinstance(first, (tuple, list)):
        return type(first)(_stack([o[i] for o in outs]) for i in range(len(first)))
    return _np.stack([_np.asarray(o) for o in outs])


def vmap(fun, in_axes=0, out_axes=0):
    def wrapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        axes = list(axes) + [None] * (len(args) - len(axes))
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _size(a, ax)
                break
        outs = [fun(*[_index(a, i, ax) for a, ax in zip(args, axes)]) for i in range(n)]
        return _stack(outs)
    return wrapped


_H = 1e-30


def grad(fun, argnums=0):
    """Complex-step gradient of a scalar function of a 1-D argument.

    All len(x) perturbed copies are evaluated in one call, column j of the
    stacked argument being x + i h e_j; the reference's potentials act
    elementwise on their coordinates, so fun returns one value per column."""
    def g(x, *rest):
        x = _np.asarray(x, dtype=_np.float64)
        n = x.shape[0]
        xc = x[:, None] + 1j * _H * _np.eye(n)
        val = _np.asarray(fun(xc, *rest))
        return _np.imag(val) / _H
    return g
