"""ADMM non-negative least squares (nnls.py:6-166), FP64.

U rows, in order: Rzphi, xy, h1..h4, each divided by (sigma + 1e-8); the
kinematic rows also by gamma_kin (floored at 1e-8 in magnitude).  Weighted by
w_rzphi, w_xy, w_h.  Q = U^T U + (lambda/n) I, rho = tr(Q)/n,
L = chol(Q + rho I), c = -U^T y.  From w = z = sum(y_Rzphi)/n, u = 0, each of
maxiter iterations does
  w = (LL^T)^-1 (rho (z - u) - c);  w^ = 1.6 w - 0.6 z;  z = max(0, w^ + u);
  u = u + w^ - z
and z is returned.  There is no convergence test.
"""
import numpy as np
import scipy.linalg as sla

EPS = 1e-8
ALPHA = 1.6


def design(A_rz, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, sig_rz, sig_xy, s1, s2, s3, s4,
           w_rzphi=1.0, w_xy=1.0, w_h=1.0):
    g = np.where(np.abs(gamma_kin) > EPS, gamma_kin, EPS)
    blocks = [w_rzphi * A_rz / (sig_rz[:, None] + EPS), w_xy * A_xy / (sig_xy[:, None] + EPS)]
    for A, s in ((A_h1, s1), (A_h2, s2), (A_h3, s3), (A_h4, s4)):
        blocks.append(w_h * A / (g[:, None] * (s[:, None] + EPS)))
    return np.vstack(blocks)


def rhs_vector(y_rz, y_xy, y1, y2, y3, y4, sig_rz, sig_xy, s1, s2, s3, s4,
               w_rzphi=1.0, w_xy=1.0, w_h=1.0):
    return np.concatenate([w_rzphi * y_rz / (sig_rz + EPS), w_xy * y_xy / (sig_xy + EPS),
                           w_h * y1 / (s1 + EPS), w_h * y2 / (s2 + EPS),
                           w_h * y3 / (s3 + EPS), w_h * y4 / (s4 + EPS)])


def admm(U, Y, w_init_val, lambda_reg, maxiter, return_state=False):
    """U: (m, n); Y: (B, m) right-hand sides.  Returns Z (B, n)."""
    n = U.shape[1]
    Q = U.T @ U + (lambda_reg / n) * np.eye(n)
    rho = np.trace(Q) / n
    cf = sla.cho_factor(Q + rho * np.eye(n), lower=True)
    c = -(Y @ U)                       # (B, n)
    B = Y.shape[0]
    w = np.full((B, n), w_init_val)
    z = w.copy()
    u = np.zeros((B, n))
    for _ in range(maxiter):
        rhs = rho * (z - u) - c
        w = sla.cho_solve(cf, rhs.T).T
        wh = ALPHA * w + (1.0 - ALPHA) * z
        z = np.maximum(0.0, wh + u)
        u = u + wh - z
    if return_state:
        return z, dict(w=w, u=u, rho=rho, Q=Q)
    return z


def solve_nnls_admm(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4,
                    y_Rzphi, y_xy, gamma_kin, y_h1, y_h2, y_h3, y_h4,
                    sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3, sig_A4,
                    lambda_reg=1.0, maxiter=200, w_rzphi=1.0, w_xy=1.0, w_h=1.0):
    U = design(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, sig_Rzphi, sig_xy,
               sig_A1, sig_A2, sig_A3, sig_A4, w_rzphi, w_xy, w_h)
    y = rhs_vector(y_Rzphi, y_xy, y_h1, y_h2, y_h3, y_h4, sig_Rzphi, sig_xy,
                   sig_A1, sig_A2, sig_A3, sig_A4, w_rzphi, w_xy, w_h)
    n = U.shape[1]
    return admm(U, y[None, :], np.sum(y_Rzphi) / n, lambda_reg, maxiter)[0]


def solve_nnls_admm_bootstrap(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4,
                              y_Rzphi, y_xy, gamma_kin,
                              y_xy_boot, y_h1_boot, y_h2_boot, y_h3_boot, y_h4_boot,
                              sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3, sig_A4,
                              lambda_reg=1.0, maxiter=200, w_rzphi=1.0, w_xy=1.0, w_h=1.0):
    U = design(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, sig_Rzphi, sig_xy,
               sig_A1, sig_A2, sig_A3, sig_A4, w_rzphi, w_xy, w_h)
    B = y_xy_boot.shape[0]
    Y = np.stack([rhs_vector(y_Rzphi, y_xy_boot[b], y_h1_boot[b], y_h2_boot[b], y_h3_boot[b],
                             y_h4_boot[b], sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3, sig_A4,
                             w_rzphi, w_xy, w_h) for b in range(B)])
    n = U.shape[1]
    return admm(U, Y, np.sum(y_Rzphi) / n, lambda_reg, maxiter)
