"""Gauss-Hermite basis and h -> (V, sigma) (ghmoments.py:6-78)."""
import math

import numpy as np

SQ2 = math.sqrt(2.0)


def gauss(v, v0, s):
    """ghmoments.py:6-9: y = (v - v0)/s, alpha = (2 pi)^-1/2 / s exp(-y^2/2)."""
    y = (v - v0) / s
    return y, (2 * math.pi) ** -0.5 / s * np.exp(-0.5 * y ** 2)


def hermite(y):
    """Orthonormal H0..H4 by the recurrence of ghmoments.py:11-36."""
    H0 = 1.0 + y * 0
    H1 = SQ2 * y
    H2 = (SQ2 * y * H1 - 1.0 * H0) / math.sqrt(2.0)
    H3 = (SQ2 * y * H2 - math.sqrt(2.0) * H1) / math.sqrt(3.0)
    H4 = (SQ2 * y * H3 - math.sqrt(3.0) * H2) / math.sqrt(4.0)
    return H0, H1, H2, H3, H4


def h_to_V_sigma(h1, h2, v0, s, h3=0.0, h4=0.0):
    """ghmoments.py:53-78."""
    dv = math.sqrt(2.0) * h1 + math.sqrt(3.0) * h3
    V = v0 + s * dv
    s2 = 1.0 + 2.0 * math.sqrt(2.0) * h2 + 2.0 * math.sqrt(6.0) * h4 - dv ** 2
    return V, s * np.sqrt(np.maximum(s2, 1e-10))
