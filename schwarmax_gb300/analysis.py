"""Post-analysis of an evaluation on the GPU, with the reference's names.

* ``build_Lcirc_of_E`` (utils.py:275-341): the circular-orbit table E_circ(R),
  L_circ(R) of the canonical potential is computed by ``smx_lcirc_table``; sorting,
  de-duplication and the not-a-knot cubic spline of interp1d(kind='cubic') are formed
  on the host (a table of n_grid points), and the returned interpolator evaluates on
  the device (``smx_spline_eval``).
* ``circularity``: lambda_z = L_z / L_circ(E) of stored samples (the model-side
  circularity of example/example_analysis.ipynb) through ``smx_circularity``, and
  ``histogram2d``, np.histogram2d's binning with exact fixed-point sums.
* ``compute_transfer_matrix`` (utils.py:413-485): the PSF transfer matrix through
  ``smx_psf_transfer``; ``apply_psf`` applies it to the sky rows of a library.
"""
import ctypes

import numpy as np
import torch

from . import kernels
from ._lib import SmxPotential, call
from .kernels import _check, _prec, _ptr, _stream
from .potentials import potential_struct, require_canonical


def not_a_knot_spline(x, y):
    """Piecewise-cubic coefficients (4, n-1) (powers of x - x_j, highest first) of the
    not-a-knot cubic spline through (x, y), the interpolant of
    scipy.interpolate.interp1d(kind='cubic').  Second derivatives M_i from the
    tridiagonal system of the interior knots, with M_0 and M_{n-1} eliminated by the
    not-a-knot conditions (third derivative continuous at x_1 and x_{n-2})."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = x.size
    if n < 4:
        raise ValueError("a cubic spline needs at least 4 points")
    h = np.diff(x)
    d = np.diff(y) / h
    r = 6.0 * (d[1:] - d[:-1])                       # interior equations i = 1 .. n-2
    k = n - 2
    lo = np.zeros(k)
    di = 2.0 * (h[:-1] + h[1:])
    up = np.zeros(k)
    lo[1:] = h[1:-1]
    up[:-1] = h[1:-1]
    # M_0 = M_1 - h0 (M_2 - M_1) / h1  -> folds into the first equation
    di[0] += h[0] + h[0] * h[0] / h[1]
    up[0] -= h[0] * h[0] / h[1]
    # M_{n-1} = M_{n-2} + h_{n-2} (M_{n-2} - M_{n-3}) / h_{n-3}
    di[-1] += h[-1] + h[-1] * h[-1] / h[-2]
    lo[-1] -= h[-1] * h[-1] / h[-2]
    # Thomas algorithm
    c = np.zeros(k)
    g = np.zeros(k)
    c[0] = up[0] / di[0]
    g[0] = r[0] / di[0]
    for i in range(1, k):
        den = di[i] - lo[i] * c[i - 1]
        c[i] = up[i] / den if i < k - 1 else 0.0
        g[i] = (r[i] - lo[i] * g[i - 1]) / den
    Mi = np.zeros(k)
    Mi[-1] = g[-1]
    for i in range(k - 2, -1, -1):
        Mi[i] = g[i] - c[i] * Mi[i + 1]
    M = np.empty(n)
    M[1:-1] = Mi
    M[0] = Mi[0] - h[0] * (Mi[1] - Mi[0]) / h[1]
    M[-1] = Mi[-1] + h[-1] * (Mi[-1] - Mi[-2]) / h[-2]
    coef = np.empty((4, n - 1))
    coef[0] = (M[1:] - M[:-1]) / (6.0 * h)
    coef[1] = M[:-1] / 2.0
    coef[2] = d - h * (2.0 * M[:-1] + M[1:]) / 6.0
    coef[3] = y[:-1]
    return coef


class LcircInterp:
    """L_circ(E) on the device: the cubic spline with interp1d's fill values."""

    def __init__(self, E, L, device="cuda"):
        self.E = np.asarray(E, dtype=np.float64)
        self.L = np.asarray(L, dtype=np.float64)
        self.coef = not_a_knot_spline(self.E, self.L)
        self.knots_d = torch.as_tensor(self.E, device=device).contiguous()
        self.coef_d = torch.as_tensor(self.coef, device=device).contiguous()
        self.below, self.above = float(self.L[0]), float(self.L[-1])

    def __call__(self, E):
        host = not isinstance(E, torch.Tensor)
        x = torch.as_tensor(np.asarray(E, dtype=np.float64) if host else E, dtype=torch.float64,
                            device=self.knots_d.device).contiguous()
        out = torch.empty_like(x)
        call("smx_spline_eval", _ptr(self.knots_d), _ptr(self.coef_d), int(self.E.size), self.below, self.above,
             _ptr(x), x.numel(), _ptr(out), _stream())
        return out.cpu().numpy() if host else out


def build_Lcirc_of_E(potential_fn, potential_args=(), R_min=1e-2, R_max=1e2, n_grid=2000, dR=1e-3, bulge_mass=None):
    """utils.py:275-341 for the canonical potential: potential_fn is
    ``potential_func`` and potential_args its (params_baryon, params_halo).
    Returns (Lcirc_interp, E_circ, L_circ) with the reference's sorting and removal of
    repeated energies; Lcirc_interp takes NumPy arrays (returns NumPy) or device
    tensors (returns device tensors)."""
    require_canonical(None, potential_fn)
    params_baryon, params_halo = potential_args
    pot = potential_struct(params_baryon, params_halo, bulge_mass, **potential_fn.types)
    E = torch.empty(int(n_grid), dtype=torch.float64, device="cuda")
    L = torch.empty_like(E)
    call("smx_lcirc_table", ctypes.byref(pot), float(R_min), float(R_max), int(n_grid), float(dR), _ptr(E), _ptr(L),
         _stream())
    E = E.cpu().numpy()
    L = L.cpu().numpy()
    order = np.argsort(E)
    E, L = E[order], L[order]
    keep = np.diff(E, prepend=-np.inf) > 0
    E, L = E[keep], L[keep]
    return LcircInterp(E, L), E, L


def circularity(points, params_baryon, params_halo, lcirc: LcircInterp, bulge_mass=None):
    """lambda_z, R and E of the phase-space points (6, N) (positions in kpc,
    velocities in kpc/Gyr; float or double CUDA tensor)."""
    pot = potential_struct(params_baryon, params_halo, bulge_mass)
    dt = points.dtype
    N = points.shape[1]
    _check(points, "points", dt, (6, N))
    lam = torch.empty(N, dtype=dt, device=points.device)
    R = torch.empty_like(lam)
    E = torch.empty_like(lam)
    call("smx_circularity", ctypes.byref(pot), _prec(dt), _ptr(points), N, _ptr(lcirc.knots_d), _ptr(lcirc.coef_d),
         int(lcirc.E.size), lcirc.below, lcirc.above, _ptr(lam), _ptr(R), _ptr(E), _stream())
    return lam, R, E


def histogram2d(a, b, bins, range, weights=None, weight_scale=None):
    """np.histogram2d(a, b, bins=(na, nb), range=range, weights=weights) on the
    device; returns the (na, nb) counts as a double tensor."""
    na, nb = (bins, bins) if np.isscalar(bins) else bins
    dt = a.dtype
    n = a.numel()
    _check(a, "a", dt, (n,))
    _check(b, "b", dt, (n,))
    if weights is not None:
        _check(weights, "weights", dt, (n,))
    ea = torch.as_tensor(np.linspace(range[0][0], range[0][1], int(na) + 1), device=a.device)
    eb = torch.as_tensor(np.linspace(range[1][0], range[1][1], int(nb) + 1), device=a.device)
    if weight_scale is None:
        if weights is None:
            weight_scale = 1.0               # counts: every add is exactly 2^40 units
        else:                                # every bin sum below 2^20 weight_scale
            weight_scale = max(float(weights.abs().max().item()) if n else 1.0, 1e-300) * max(1.0, float(n)) / 2 ** 20
    scratch = torch.empty(int(na) * int(nb), dtype=torch.int64, device=a.device)
    out = torch.empty(int(na), int(nb), dtype=torch.float64, device=a.device)
    call("smx_histogram2d", _prec(dt), _ptr(a), _ptr(b), _ptr(weights), n, _ptr(ea), int(na), _ptr(eb), int(nb),
         float(weight_scale), _ptr(scratch), _ptr(out), _stream())
    return out


def gaussian_kernel1d(sigma, truncate=4.0):
    """Normalised Gaussian taps exp(-x^2 / 2 sigma^2), x = -r .. r, r = int(truncate sigma + 0.5)
    (the kernel of scipy.ndimage.gaussian_filter)."""
    r = int(truncate * float(sigma) + 0.5)
    x = np.arange(-r, r + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    return phi / phi.sum(), r


def compute_transfer_matrix(sigma_psf, nX, nY, X_minmax, Y_minmax, bin_mapping, total_bins, grid_res=500):
    """utils.py:413-485 on the device.  Returns P (total_bins, total_bins) as a double
    CUDA tensor (identity for sigma_psf == 0)."""
    if sigma_psf == 0:
        return torch.eye(int(total_bins), dtype=torch.float64, device="cuda")
    bm = np.asarray(bin_mapping.cpu() if isinstance(bin_mapping, torch.Tensor) else bin_mapping)
    if len(bm) == nX * nY + 1:
        bm = bm[:-1]
    X_min, X_max = (float(v) for v in X_minmax)
    Y_min, Y_max = (float(v) for v in Y_minmax)
    pixel = np.linspace(X_min, X_max, grid_res + 1)
    sigma_pix = sigma_psf / (pixel[1] - pixel[0])
    kw, r = gaussian_kernel1d(sigma_pix)
    kw_d = torch.as_tensor(kw[::-1].copy(), device="cuda")
    bm_d = torch.as_tensor(bm.astype(np.int32), device="cuda")
    nbytes = ctypes.c_size_t(0)
    call("smx_psf_transfer_workspace_size", int(grid_res), int(total_bins), int(r), ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
    P = torch.empty(int(total_bins), int(total_bins), dtype=torch.float64, device="cuda")
    call("smx_psf_transfer", _ptr(kw_d), int(r), int(nX), int(nY), X_min, X_max, Y_min, Y_max, _ptr(bm_d),
         int(total_bins), int(grid_res), _ptr(P), _ptr(ws), ws.numel(), _stream())
    return P


def apply_psf(library, P, n_cells, n_bins):
    """The PSF transfer applied to the sky rows of a library (n, rows): every row block
    [xy | h0 .. h4] of the apertures becomes P @ block (flux and its
    Gauss-Hermite-weighted sums are redistributed alike).  Returns a new library."""
    out = library.clone()
    Pd = P.to(library.dtype)
    for k in range(6):
        sl = slice(n_cells + k * n_bins, n_cells + (k + 1) * n_bins)
        out[:, sl] = library[:, sl] @ Pd.t()
    return out


__all__ = ["build_Lcirc_of_E", "circularity", "histogram2d", "compute_transfer_matrix", "apply_psf",
           "not_a_knot_spline", "LcircInterp", "SmxPotential", "kernels"]
