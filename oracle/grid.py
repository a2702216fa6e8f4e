"""Regular-grid cell assignment (utils.py:10-42) and the projection of a
phase-space sample onto the Rzphi grid and the sky grid (integrates.py:115-147).

The arithmetic runs in the dtype of the inputs, one IEEE-rounded operation at
a time and in a fixed order, so the float32 path reproduces the integer cell
indices of a float32 kernel that uses the same order without FMA contraction:

  normalised = (p - lo) / (hi - lo);  k = floor(normalised * n)
  clip k to [0, n-1];  flat = sum_d k_d * stride_d
  any normalised >= 1 or < 0  ->  flat = prod(n)   (dropped later)
"""
import numpy as np


def assign_regular_grid(pos, lo, hi, nbins):
    """pos: (N, Dm) array; lo, hi, nbins: length-Dm sequences."""
    pos = np.asarray(pos)
    dt = pos.dtype
    n = np.asarray(nbins, dtype=np.int64)
    lo = np.asarray(lo, dtype=dt)
    hi = np.asarray(hi, dtype=dt)
    span = (hi - lo).astype(dt)
    norm = ((pos - lo).astype(dt) / span).astype(dt)
    k = np.floor((norm * n.astype(dt)).astype(dt)).astype(np.int64)
    k = np.clip(k, 0, n - 1)
    strides = np.concatenate([[1], np.cumprod(n[:-1])])
    flat = (k * strides).sum(axis=-1)
    oob = np.any((norm >= 1.0) | (norm < 0.0), axis=-1)
    return np.where(oob, int(np.prod(n)), flat).astype(np.int64)


SIGN_SYM = np.array([
    [1, 1, 1, 1, 1, 1],
    [1, 1, -1, 1, 1, -1],
    [-1, -1, 1, -1, -1, 1],
    [-1, -1, -1, -1, -1, -1],
])  # integrates.py:74-79


def sample_cells(x, y, z, vx, vy, vz, rot, rzphi_lo, rzphi_hi, n_rzphi,
                 xy_lo, xy_hi, n_xy, bin_mapping):
    """Cell indices and line-of-sight velocity (kpc/Gyr) of samples.

    Returns (rz_cell, vbin, vlos) with rz_cell in [0, prod(n_rzphi)] and
    vbin = bin_mapping[pixel] (-1 = outside any aperture).  rot is the 3x3
    matrix X = rot @ x (utils.py:176-179); the rotated coordinate is formed as
    (r0*x + r1*y) + r2*z.
    """
    dt = np.asarray(x).dtype
    R = np.sqrt((x * x + y * y).astype(dt)).astype(dt)
    ph = np.arctan2(y, x).astype(dt)
    rz_cell = assign_regular_grid(np.stack([R, z, ph], -1), rzphi_lo, rzphi_hi, n_rzphi)
    r = np.asarray(rot, dtype=dt)
    X = ((r[0, 0] * x + r[0, 1] * y).astype(dt) + r[0, 2] * z).astype(dt)
    Y = ((r[1, 0] * x + r[1, 1] * y).astype(dt) + r[1, 2] * z).astype(dt)
    vl = ((r[2, 0] * vx + r[2, 1] * vy).astype(dt) + r[2, 2] * vz).astype(dt)
    pix = assign_regular_grid(np.stack([X, Y], -1), xy_lo, xy_hi, n_xy)
    vbin = np.asarray(bin_mapping)[pix]
    return rz_cell, vbin, vl
