"""Precision model of the mixed NNLS, in FP64 NumPy on the CPU.

The split tensor-core products are exact for inputs cut to fixed point (31 bits
below each row's largest magnitude for 4 slices, 39 bits for 5), so their error is
that of the cut inputs.  On an orbit-like library (epicyclic orbits binned by the
oracle, 100 bootstraps, 200 ADMM iterations of nnls.py:68-166) this test compares,
against the plain FP64 ADMM, the bootstrap chi^2 moved by
  * U = library x row scale rounded to float,
  * U cut to 31 bits per row,
  * U cut to 39 bits per row,
and pins their order: float rounding >> 31 bits >> 39 bits.  (The mixed solver
builds U in double and slices it; float rounding of U was the dominant term.)"""
import math

import numpy as np
import pytest

from oracle import integrate as oi, nnls as onnls

pytestmark = pytest.mark.slow


def _library(rng, n, K=160, n_pix=40, n_bins=120):
    kms = 1.0 / 0.9777922216807892
    Rg = rng.gamma(2.0, 2.5, n) + 0.2
    e = rng.uniform(0, 0.5, n)
    Z = rng.exponential(0.3, n)
    vc = 220 * kms * (1 - np.exp(-Rg / 1.5))
    Om = vc / Rg
    t = np.linspace(0, 20 * np.pi, K)[None, :]
    ph0, ps, ch = rng.uniform(0, 2 * np.pi, (3, n, 1))
    R = Rg[:, None] * (1 + e[:, None] * np.cos(1.4 * t + ps))
    phi = ph0 + t
    z = Z[:, None] * np.cos(2.5 * t + ch)
    ys = np.stack([R * np.cos(phi), R * np.sin(phi), z, -vc[:, None] * np.sin(phi), vc[:, None] * np.cos(phi),
                   -Z[:, None] * 2.5 * Om[:, None] * np.sin(2.5 * t + ch)], -1).transpose(1, 0, 2)
    half = n_pix * 0.5 * (50e3 * math.pi / (180 * 3600)) / 2
    pix = np.stack(np.meshgrid(np.arange(n_pix), np.arange(n_pix), indexing="xy"), -1).reshape(-1, 2)
    gen = pix[rng.choice(len(pix), n_bins, replace=False)]
    bm = np.argmin(((pix[:, None, :] - gen[None]) ** 2).sum(-1), 1)
    npb = np.bincount(bm, minlength=n_bins).astype(float) + 1
    a, b, g = (math.radians(v) for v in (30, 60, 45))

    def rz(x):
        c, s = math.cos(x), math.sin(x)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])

    def rx(x):
        c, s = math.cos(x), math.sin(x)
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])

    geo = oi.BinGeometry((rz(g) @ rx(b) @ rz(a)).T, [[0, 10], [-3, 3], [-np.pi, np.pi]], [20, 16, 10],
                         [[-half, half], [-half, half]], [n_pix, n_pix], np.concatenate([bm, [-1]]), npb,
                         np.zeros(n_bins), np.full(n_bins, 150.0))
    acc = oi.Accumulator(n, geo)
    acc.add(ys, np.ones((K, n)))
    Rz_, surf, h, _ = oi.normalise(acc, np.ones(n), np.ones(n), np.full(n, 100.0), np.full(n, 100.0))
    return oi.realisation_mean(Rz_, surf, h, np.ones(n), n, 1)


def _trunc_rows(M, bits):
    mx = np.abs(M).max(1, keepdims=True)
    e = np.ceil(np.log2(np.where(mx > 0, mx, 1.0)))
    sc = np.exp2(bits - e)
    return np.rint(M * sc) / sc


def test_float_rounding_of_the_design_matrix_dominates_the_slicing():
    rng = np.random.default_rng(7)
    n, B, lam, iters = 768, 100, 1.0, 200
    A_rz, A_xy, A_h = _library(rng, n)
    nb = A_xy.shape[0]
    w_true = rng.dirichlet(np.full(n, 0.3)) * n
    y_rz = A_rz @ w_true + 1e-6
    y_xy = (A_xy @ w_true) * (1 + 0.05 * rng.normal(size=nb)) + 1e-9
    gamma = A_xy @ w_true + 1e-9
    yh = [A_h[k] @ w_true / gamma + 0.02 * rng.normal(size=nb) for k in range(1, 5)]
    sig_rz, sig_xy = 0.1 * y_rz, 0.1 * y_xy
    sh = [np.full(nb, 0.03) for _ in range(4)]
    W = dict(w_rzphi=math.sqrt(5.0), w_xy=math.sqrt(5.0), w_h=1.0)
    U = onnls.design(A_rz, A_xy, *A_h[1:], gamma, sig_rz, sig_xy, *sh, **W)
    keep = np.abs(U).max(1) > 0
    U = U[keep]
    Y = np.array([onnls.rhs_vector(y_rz, y_xy + (sig_xy * rng.normal(size=nb) if b else 0),
                                   *[yh[k] + (sh[k] * rng.normal(size=nb) if b else 0) for k in range(4)],
                                   sig_rz, sig_xy, *sh, **W)[keep] for b in range(B)])
    w0 = np.sum(y_rz) / n

    def chi2(Uc):
        Z = onnls.admm(Uc, Y, w0, lam, iters)
        R = Z @ U.T - Y
        return np.sum(R * R, 1)

    ref = chi2(U)
    scale = np.median(ref)
    moved = {name: np.abs(chi2(Uc) - ref).max() / scale
             for name, Uc in (("float", U.astype(np.float32).astype(np.float64)), ("31", _trunc_rows(U, 31)),
                              ("39", _trunc_rows(U, 39)))}
    assert moved["float"] > 5 * moved["31"] > 0
    assert moved["31"] > 20 * moved["39"]
