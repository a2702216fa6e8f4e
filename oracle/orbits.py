"""Per-particle set-up of the orbit library (oracle restatement).

makeRotationMatrix     utils.py:164-179
cylindrical -> xy      utils.py:144-162
T_orb, V_c             utils.py:182-273 (central differences, dR = 1e-3)
jitter                 model.py:127-148 (uniform draws are explicit inputs)
Jacobi energy          integrates.py:29-35
"""
import math

import numpy as np

from . import potential as pot


def rotation_matrix(alpha_deg, beta_deg, gamma_deg):
    """(Rz(g) Rx(b) Rz(a))^T with angles in degrees; X = R @ x."""
    a, b, g = (math.radians(v) for v in (alpha_deg, beta_deg, gamma_deg))

    def Rz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    def Rx(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])

    return (Rz(g) @ Rx(b) @ Rz(a)).T


def cyl_to_cart_clockwise(R, phi, vR, vphi):
    c, s = np.cos(phi), np.sin(phi)
    return R * c, R * s, vR * c + vphi * s, vR * s - vphi * c


def _dphi_dR(R, z, P, dR):
    Rs = np.maximum(np.abs(R), 2 * dR)
    zero = np.zeros_like(Rs)
    d = (pot.phi(Rs + dR, zero, z, P) - pot.phi(Rs - dR, zero, z, P)) / (2.0 * dR)
    return Rs, d


def orbital_timescale(R, z, P, dR=1e-3):
    Rs, d = _dphi_dR(R, z, P, dR)
    om2 = np.maximum(np.abs(d) / Rs, 1e-20)
    return 2 * np.pi / np.sqrt(om2)


def rotation_curve(R, z, P, dR=1e-3):
    Rs, d = _dphi_dR(R, z, P, dR)
    return np.sqrt(np.maximum(Rs * d, 0.0))


def jitter(w0_new, Vc, uniforms):
    """w0_new: (n, 6); Vc: (n,); uniforms: (6, n, n_real) in [0, 1).

    Returns (n, n_real, 6) = w0_new + (u - 0.5) * scale, scale 0.1 kpc for
    positions and clip(0.1 Vc, 1, 15) kpc/Gyr for velocities."""
    d_scale = 0.1 * np.ones_like(Vc)
    v_scale = np.clip(0.1 * Vc, 1, 15)
    sc = [d_scale, d_scale, d_scale, v_scale, v_scale, v_scale]
    noise = np.stack([(uniforms[i] - 0.5) * sc[i][:, None] for i in range(6)], -1)
    return w0_new[:, None, :] + noise


def jacobi_energy(w, P, Omega):
    x, y, z, vx, vy, vz = (w[..., i] for i in range(6))
    ek = 0.5 * (vx ** 2 + vy ** 2 + vz ** 2)
    phi = pot.phi_acc(x, y, z, P)[0] if P.get("cylspline") is not None else pot.phi(x, y, z, P)
    return ek + phi - Omega * (x * vy - y * vx)
