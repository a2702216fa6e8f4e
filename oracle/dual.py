"""Forward-mode derivatives for the oracle.

The reference takes the acceleration as ``-jax.grad`` of the total potential
(model.py:152-157).  The oracle gets the same mathematical gradient by
evaluating the potential on dual numbers carrying three tangents (d/dx, d/dy,
d/dz), vectorised over points.  Plain ndarrays pass through unchanged, so one
potential routine serves values and gradients.
"""
import numpy as np


class Dual:
    __slots__ = ("v", "d")

    def __init__(self, v, d):
        self.v = v          # values, shape S
        self.d = d          # tangents, shape (k,) + S

    # -- arithmetic -------------------------------------------------------
    def __add__(self, o):
        if isinstance(o, Dual):
            return Dual(self.v + o.v, self.d + o.d)
        return Dual(self.v + o, self.d)

    __radd__ = __add__

    def __sub__(self, o):
        if isinstance(o, Dual):
            return Dual(self.v - o.v, self.d - o.d)
        return Dual(self.v - o, self.d)

    def __rsub__(self, o):
        return Dual(o - self.v, -self.d)

    def __neg__(self):
        return Dual(-self.v, -self.d)

    def __mul__(self, o):
        if isinstance(o, Dual):
            return Dual(self.v * o.v, self.d * o.v + o.d * self.v)
        return Dual(self.v * o, self.d * o)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, Dual):
            q = self.v / o.v
            return Dual(q, (self.d - o.d * q) / o.v)
        return Dual(self.v / o, self.d / o)

    def __rtruediv__(self, o):
        q = o / self.v
        return Dual(q, -self.d * (q / self.v))

    def __pow__(self, p):
        if isinstance(p, Dual):
            raise TypeError("dual exponent not supported")
        if p == 2:
            return self * self
        if p == 3:
            return self * self * self
        vp = self.v ** p
        return Dual(vp, self.d * (p * self.v ** (p - 1)))


def seed(*vals):
    """Return Duals for independent variables with unit tangents."""
    k = len(vals)
    out = []
    for i, v in enumerate(vals):
        v = np.asarray(v, dtype=np.float64)
        d = np.zeros((k,) + v.shape)
        d[i] = 1.0
        out.append(Dual(v, d))
    return out


def sqrt(x):
    if isinstance(x, Dual):
        s = np.sqrt(x.v)
        return Dual(s, x.d * (0.5 / s))
    return np.sqrt(x)


def log(x):
    if isinstance(x, Dual):
        return Dual(np.log(x.v), x.d / x.v)
    return np.log(x)


def exp(x):
    if isinstance(x, Dual):
        e = np.exp(x.v)
        return Dual(e, x.d * e)
    return np.exp(x)


def value(x):
    return x.v if isinstance(x, Dual) else x
