"""Axisymmetric Jeans initial velocities (jeans.py:8-93).

Per particle at (x*, y*, z*):
  sigma_z^2 = (1/nu) * trapz_{|z*|..10, 1000 pts} rho(x*, y*, z') dPhi/dz(x*, y*, z')
  P(r)      = trapz_{|z*|..10} rho(r, 0, z') dPhi/dz(r, 0, z')
  v_phi^2   = b sigma_z^2 + (R/nu) b (P(R+h) - P(R-h))/(2h) + R dPhi/dR(R, 0, z*)
  v_stream  = sqrt(max(v_phi^2 - sigma_R^2, 0)),  sigma_R = sigma_phi = sqrt(b) sigma_z
with dPhi/dz, dPhi/dR central differences of step 5e-3 and h = 5e-3.
Velocities: vR = g1 sigma_R, vz = g2 sigma_z, vphi = v_stream + g3 sigma_phi,
mapped by the clockwise cylindrical convention (utils.py:144-162).  The
normal draws g1, g2, g3 are explicit inputs (the reference uses threefry keys
42, 109, 2026).
"""
import numpy as np

from . import orbits
from . import potential as pot

N_QUAD = 1000
Z_TOP = 10.0
FD = 5e-3


def _dphi_dz(x, y, z, P):
    return (pot.phi(x, y, z + FD, P) - pot.phi(x, y, z - FD, P)) / (2 * FD)


def _trapz_column(x, y, zabs, P):
    """trapezoid of rho * dPhi/dz on linspace(|z|, 10, 1000); x, y, zabs: (n,)."""
    t = np.linspace(0.0, 1.0, N_QUAD)
    pts = zabs[:, None] + (Z_TOP - zabs)[:, None] * t[None, :]
    # jnp.linspace(a, b, n) ends exactly at b
    pts[:, -1] = Z_TOP
    X = np.broadcast_to(x[:, None], pts.shape)
    Y = np.broadcast_to(y[:, None], pts.shape)
    f = pot.rho(X, Y, pts, P) * _dphi_dz(X, Y, pts, P)
    dz = np.diff(pts, axis=1)
    return np.sum(0.5 * (f[:, 1:] + f[:, :-1]) * dz, axis=1)


def jeans_moments(x, y, z, P, anisotropy_b=1.0, chunk=512):
    n = x.shape[0]
    out = np.zeros((4, n))
    for s in range(0, n, chunk):
        sl = slice(s, s + chunk)
        xs, ys, zs = x[sl], y[sl], z[sl]
        R = np.sqrt(xs ** 2 + ys ** 2)
        za = np.abs(zs)
        integ = _trapz_column(xs, ys, za, P)
        nu = pot.rho(xs, ys, zs, P)
        sz2 = np.maximum(integ / nu, 0.0)
        sz = np.sqrt(sz2)
        sR2 = anisotropy_b * sz2
        sR = np.sqrt(sR2)
        zero = np.zeros_like(R)
        Pp = _trapz_column(R + FD, zero, za, P)
        Pm = _trapz_column(R - FD, zero, za, P)
        dP = anisotropy_b * (Pp - Pm) / (2 * FD)
        dphidR = (pot.phi(R + FD, zero, zs, P) - pot.phi(R - FD, zero, zs, P)) / (2 * FD)
        vphi2 = sR2 + (R / nu) * dP + R * dphidR
        vstream = np.sqrt(np.maximum(vphi2 - sR ** 2, 0.0))
        ok = nu > 0
        out[0, sl] = np.where(ok, vstream, 0.0)
        out[1, sl] = np.where(ok, sR, 0.0)
        out[2, sl] = np.where(ok, sz, 0.0)
        out[3, sl] = np.where(ok, sR, 0.0)
    return out


def w0_new(w0, normals, P):
    """w0: (n, 3) positions; normals: (3, n) standard normal draws -> (n, 6)."""
    x, y, z = w0[:, 0], w0[:, 1], w0[:, 2]
    v_rot, sR, sz, sphi = jeans_moments(x, y, z, P)
    vR = normals[0] * sR
    vz = normals[1] * sz
    vphi = v_rot + normals[2] * sphi
    R = np.sqrt(x ** 2 + y ** 2)
    X, Y, VX, VY = orbits.cyl_to_cart_clockwise(R, np.arctan2(y, x), vR, vphi)
    return np.stack([X, Y, z, VX, VY, vz], -1)
