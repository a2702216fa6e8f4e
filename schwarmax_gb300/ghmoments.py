"""Gauss-Hermite helpers on torch tensors (ghmoments.py:6-78)."""
import math

import torch


def gauss(x, v, s):
    y = (x - v) / s
    return y, (2 * math.pi) ** -0.5 / s * torch.exp(-0.5 * y ** 2)


def hermite(y):
    """Orthonormal H0..H4 of van der Marel & Franx (ghmoments.py:11-36)."""
    s2 = math.sqrt(2.0)
    H0 = torch.ones_like(y)
    H1 = s2 * y
    H2 = (s2 * y * H1 - H0) / math.sqrt(2.0)
    H3 = (s2 * y * H2 - math.sqrt(2.0) * H1) / math.sqrt(3.0)
    H4 = (s2 * y * H3 - math.sqrt(3.0) * H2) / 2.0
    return H0, H1, H2, H3, H4


def h_to_V_sigma(h1, h2, v0, s, h3=0.0, h4=0.0):
    dv = math.sqrt(2.0) * h1 + math.sqrt(3.0) * h3
    s2 = 1.0 + 2.0 * math.sqrt(2.0) * h2 + 2.0 * math.sqrt(6.0) * h4 - dv ** 2
    return v0 + s * dv, s * torch.sqrt(torch.clamp(s2, min=1e-10))
