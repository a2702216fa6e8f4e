"""Post-analysis restated on the CPU (test infrastructure: checks the device
kernels of schwarmax_gb300.analysis; nothing in the product imports it).

* ``build_Lcirc_of_E`` follows utils.py:275-341: log-spaced radii, midplane
  potential and its central difference along x, sort, removal of repeated
  energies, and scipy's interp1d(kind='cubic') with the end values as fill.
* ``compute_transfer_matrix`` follows utils.py:413-485: fine grid, pixel map,
  scipy.ndimage.gaussian_filter(mode='constant') of every bin's indicator image,
  per-bin sums, column normalisation.
"""
import numpy as np

from . import potential as op


def lcirc_table(P, R_min=1e-2, R_max=1e2, n_grid=2000, dR=1e-3):
    R = np.logspace(np.log10(R_min), np.log10(R_max), n_grid)
    zero = np.zeros_like(R)
    ph = op.phi(R, zero, zero, P)
    dphi = (op.phi(R + dR, zero, zero, P) - op.phi(R - dR, zero, zero, P)) / (2.0 * dR)
    vc2 = np.maximum(R * dphi, 0.0)
    return ph + 0.5 * vc2, R * np.sqrt(vc2)


def build_Lcirc_of_E(P, R_min=1e-2, R_max=1e2, n_grid=2000, dR=1e-3):
    from scipy.interpolate import interp1d
    E, L = lcirc_table(P, R_min, R_max, n_grid, dR)
    i = np.argsort(E)
    E, L = E[i], L[i]
    keep = np.diff(E, prepend=-np.inf) > 0
    E, L = E[keep], L[keep]
    return interp1d(E, L, kind="cubic", bounds_error=False, fill_value=(L[0], L[-1])), E, L


def circularity(points, P, interp):
    """lambda_z, R, E of phase-space points (6, N), velocities in kpc/Gyr."""
    x, y, z, vx, vy, vz = points
    E = 0.5 * (vx * vx + vy * vy + vz * vz) + op.phi(x, y, z, P)
    Lz = -(x * vy - y * vx)
    return Lz / (np.asarray(interp(E)) + 1e-10), np.sqrt(x * x + y * y), E


def compute_transfer_matrix(sigma_psf, nX, nY, X_minmax, Y_minmax, bin_mapping, total_bins, grid_res=500):
    from scipy.ndimage import gaussian_filter
    bm = np.asarray(bin_mapping)
    if len(bm) == nX * nY + 1:
        bm = bm[:-1]
    if sigma_psf == 0:
        return np.eye(total_bins)
    X_min, X_max = X_minmax
    Y_min, Y_max = Y_minmax
    xe = np.linspace(X_min, X_max, grid_res + 1)
    ye = np.linspace(Y_min, Y_max, grid_res + 1)
    XX, YY = np.meshgrid(0.5 * (xe[:-1] + xe[1:]), 0.5 * (ye[:-1] + ye[1:]))
    ix = np.clip(np.floor((XX.ravel() - X_min) / (X_max - X_min) * nX).astype(int), 0, nX - 1)
    iy = np.clip(np.floor((YY.ravel() - Y_min) / (Y_max - Y_min) * nY).astype(int), 0, nY - 1)
    fine = bm[ix + iy * nX].reshape(grid_res, grid_res)
    sigma_pix = sigma_psf / (xe[1] - xe[0])
    P = np.zeros((total_bins, total_bins))
    flat = fine.ravel()
    for j in range(total_bins):
        conv = gaussian_filter((fine == j).astype(float), sigma=sigma_pix, mode="constant").ravel()
        P[:, j] = np.bincount(flat[flat >= 0], weights=conv[flat >= 0], minlength=total_bins)[:total_bins]
    cs = P.sum(axis=0)
    return P / np.where(cs > 0, cs, 1.0)[None, :]
