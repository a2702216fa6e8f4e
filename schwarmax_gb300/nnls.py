"""ADMM NNLS with the reference's argument lists (nnls.py:6-166).

The A blocks are (rows, n_orb) as in the reference; they are packed into an
orbit-major library (n_orb, rows) and solved by ``smx_nnls_admm`` (Woodbury
form, Cholesky of the rows x rows system).  ``mixed=False`` is the FP64 path.
"""
import torch

from . import kernels
from .potentials import as_cuda

EPS = 1e-8


def _pack(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, dtype):
    blocks = [as_cuda(A, dtype) for A in (A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4)]
    lib = torch.cat([b.t() for b in blocks], dim=1).contiguous()
    return lib, torch.arange(lib.shape[1], dtype=torch.int32, device="cuda")


def _scales(A_Rzphi, A_xy, gamma_kin, sig_Rzphi, sig_xy, sigs, w_rzphi, w_xy, w_h):
    g = as_cuda(gamma_kin, torch.float64)
    g = torch.where(g.abs() > EPS, g, torch.full_like(g, EPS))
    rs = [w_rzphi / (as_cuda(sig_Rzphi, torch.float64) + EPS), w_xy / (as_cuda(sig_xy, torch.float64) + EPS)]
    rs += [w_h / (g * (as_cuda(s, torch.float64) + EPS)) for s in sigs]
    return torch.cat(rs).contiguous()


def _rhs(y_rz, y_xy, yh, sig_Rzphi, sig_xy, sigs, w_rzphi, w_xy, w_h):
    parts = [w_rzphi * as_cuda(y_rz, torch.float64) / (as_cuda(sig_Rzphi, torch.float64) + EPS),
             w_xy * as_cuda(y_xy, torch.float64) / (as_cuda(sig_xy, torch.float64) + EPS)]
    parts += [w_h * as_cuda(y, torch.float64) / (as_cuda(s, torch.float64) + EPS) for y, s in zip(yh, sigs)]
    return torch.cat(parts, dim=-1)


def solve_nnls_admm(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4,
                    y_Rzphi, y_xy, gamma_kin, y_h1, y_h2, y_h3, y_h4,
                    sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3, sig_A4,
                    lambda_reg=1, maxiter=200, w_rzphi=1.0, w_xy=1.0, w_h=1.0, mixed=False):
    """nnls.py:6-66; returns z (n_orb,) as a CUDA float64 tensor."""
    return solve_nnls_admm_bootstrap(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, y_Rzphi, y_xy, gamma_kin,
                                     as_cuda(y_xy, torch.float64)[None], as_cuda(y_h1, torch.float64)[None],
                                     as_cuda(y_h2, torch.float64)[None], as_cuda(y_h3, torch.float64)[None],
                                     as_cuda(y_h4, torch.float64)[None], sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3,
                                     sig_A4, lambda_reg, maxiter, w_rzphi, w_xy, w_h, mixed)[0]


def solve_nnls_admm_bootstrap(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4,
                              y_Rzphi, y_xy, gamma_kin,
                              y_xy_boot, y_h1_boot, y_h2_boot, y_h3_boot, y_h4_boot,
                              sig_Rzphi, sig_xy, sig_A1, sig_A2, sig_A3, sig_A4,
                              lambda_reg=1, maxiter=200, w_rzphi=1.0, w_xy=1.0, w_h=1.0, mixed=False):
    """nnls.py:68-166; returns weights (N_boot, n_orb) as a CUDA float64 tensor."""
    dtype = torch.float32 if mixed else torch.float64
    lib, rm = _pack(A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, dtype)
    sigs = (sig_A1, sig_A2, sig_A3, sig_A4)
    rs = _scales(A_Rzphi, A_xy, gamma_kin, sig_Rzphi, sig_xy, sigs, float(w_rzphi), float(w_xy), float(w_h))
    yb = as_cuda(y_xy_boot, torch.float64)
    B = yb.shape[0]
    y_rz = as_cuda(y_Rzphi, torch.float64)
    Y = _rhs(y_rz[None].expand(B, -1), yb, [as_cuda(v, torch.float64) for v in (y_h1_boot, y_h2_boot, y_h3_boot,
                                                                                y_h4_boot)],
             sig_Rzphi, sig_xy, sigs, float(w_rzphi), float(w_xy), float(w_h)).contiguous()
    n = lib.shape[0]
    w_init = float(y_rz.sum().item()) / n
    return kernels.nnls_admm(lib, rm, rs, Y, int(maxiter), float(lambda_reg), w_init, mixed)
