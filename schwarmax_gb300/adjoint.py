"""Differentiable projection + NNLS: gradients of chi^2 with respect to the
viewing angles (alpha, beta, gamma) and a line-of-sight velocity scale.

There is no reference counterpart: the reference stops gradients at its NNLS
(nnls.py:66,165).  The stored orbit samples of one evaluation are the input
(the integration does not depend on the viewing angles).  The model is

  A(theta)   library whose sky rows [xy | h0..h4] come from smx_soft_project
             (soft aperture assignment: a Gaussian of sigma pixels integrated
             over each pixel) and whose Rzphi rows are the hard ones;
  U(theta)   the scaled NNLS design rows of A (engine.nnls_inputs, row_map);
  w*(theta)  the NNLS solution for the unperturbed data row y: ADMM
             (smx_nnls_admm, FP64) refined on its free set F by the exact KKT
             system (U_F^T U_F + (lambda/n) I) w_F = U_F^T y  (active-set steps
             drop negative entries);
  chi^2      the likelihood's chi^2 of A w* for the unperturbed data
             (likelihood.py:214-226: Rzphi, xy with sigma = 0.1 y, h1..h4).

The gradient is the adjoint of that chain: the direct term dchi^2/dA at fixed
w, plus implicit differentiation of the KKT system,
  mu_F = H_FF^-1 (A^T dchi^2/dmodel)_F,   dchi^2/dU += -(r mu^T + (U mu) w*^T),
  r = U w* - y,
mapped back to the library rows and contracted with dA/dtheta by
smx_soft_project_adjoint, which recomputes the rotated samples.
"""
import ctypes
import math

import numpy as np
import torch

from . import engine, kernels
from ._lib import SMX_FP64, call

KMS = 0.9777922216807892


def rotation_and_derivatives(alpha, beta, gamma):
    """R = (Rz(g) Rx(b) Rz(a))^T (utils.py:164-179, angles in radians) and dR/d(alpha, beta, gamma)."""
    def Rz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    def dRz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[-s, -c, 0.0], [c, -s, 0.0], [0.0, 0.0, 0.0]])

    def Rx(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])

    def dRx(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[0.0, 0.0, 0.0], [0.0, -s, -c], [0.0, c, -s]])

    a, b, g = float(alpha), float(beta), float(gamma)
    R = (Rz(g) @ Rx(b) @ Rz(a)).T
    dR = np.stack([(Rz(g) @ Rx(b) @ dRz(a)).T, (Rz(g) @ dRx(b) @ Rz(a)).T, (dRz(g) @ Rx(b) @ Rz(a)).T])
    return R, dR


class SoftProblem:
    """Everything of one evaluation that the soft chi^2 needs, on the device, in double.

    bufs: integrator buffers of the evaluation (samples are converted to double),
    geo: its binning geometry (smx_binning), library: the hard library (n, rows),
    d: engine.data_terms output, dd: DeviceData, row_scale / y: scaled NNLS rows and
    the unperturbed data row (m,), lum: mean mass per orbit times L/M.
    """

    def __init__(self, bufs, t_total, geo, library, d, dd, row_scale, y, lum, sigma_pix=0.5, sigma_amplify=1.0,
                 regularization=1.0, admm_iters=200):
        self.samples = bufs.samples.double().contiguous()
        self.n_stored = bufs.n_stored
        self.slots = bufs.slots
        self.info = bufs.info.double().contiguous()
        self.t_total = t_total.double().contiguous()
        self.geo = geo
        self.library = library.double().contiguous()
        self.n, self.rows = self.library.shape
        self.nc = geo.nR * geo.nz * geo.nphi
        self.nb = geo.n_bins
        self.dd = dd
        self.d = d
        self.row_map = engine.row_map(self.nc, self.nb)
        self.row_scale = row_scale
        self.y = y.contiguous()
        self.lum = float(lum)
        self.sigma_pix = float(sigma_pix)
        self.amp = float(sigma_amplify)
        self.lam = float(regularization)
        self.admm_iters = int(admm_iters)
        s_min = float(dd.s.min())
        if not (math.isfinite(s_min) and s_min >= 0.01):
            raise ValueError(f"soft projection needs finite dispersions >= 0.01 km/s, got min {s_min}")
        self.h_data = dd.h.double()                # (4, nb) observed h1..h4 (bootstrap 0)
        self.sig_h = (dd.h_err + engine.EPSILON).double()

    # --------------------------------------------------------------- pieces
    def soft_library(self, theta):
        """Library with soft sky rows at theta = (alpha, beta, gamma [rad], vscale)."""
        a, b, g, vs = (float(t) for t in theta)
        R, _ = rotation_and_derivatives(a, b, g)
        for i in range(9):
            self.geo.rot[i] = float(R.reshape(-1)[i])
        lib = self.library.clone()
        call("smx_soft_project", ctypes.byref(self.geo), SMX_FP64, self.sigma_pix, vs,
             kernels._ptr(self.samples), kernels._ptr(self.n_stored), self.slots, kernels._ptr(self.info),
             kernels._ptr(self.t_total), kernels._ptr(self.dd.bin_mapping), kernels._ptr(self.dd.num_per_bin),
             kernels._ptr(self.dd.v0), kernels._ptr(self.dd.s), kernels._ptr(lib), kernels._stream())
        return lib

    def design(self, lib):
        return (lib[:, self.row_map.long()] * self.row_scale[None, :]).t().contiguous()   # (m, n)

    def solve(self, lib, U):
        """NNLS solution: ADMM, then Lawson-Hanson active-set steps to the exact KKT point of
        min |U w - y|^2 + (lambda/n) |w|^2, w >= 0.  Starting from the ADMM iterate
        (feasible, w >= 0) with its positive entries as the free set F: solve on F; if
        some entries come out <= 0, move from the current w towards that solution only as
        far as the first entry reaches zero and drop the entries at zero (so w stays
        feasible and the objective decreases); once the solution on F is positive, add the
        quarter of the inactive entries whose gradient is most negative, until the KKT
        conditions hold to 1e-8 of |U^T y| (at most 50 rounds; `kkt_settled` records
        whether they did).  An entry dropped right after it was added sits out one round.
        The fewer ADMM iterations (`admm_iters`), the farther the start and the more rounds."""
        n = self.n
        w_init = float((self.d["y_rz"].sum() / n).item())
        W0 = kernels.nnls_admm(lib, self.row_map, self.row_scale, self.y[None, :].contiguous(), self.admm_iters,
                               self.lam, w_init, mixed=False)[0]
        lam_n = self.lam / n
        Uty = U.t() @ self.y
        # a KKT violation below 1e-8 of |U^T y| is rounding of the free-set solve, not a
        # missing orbit: counting it would keep adding and dropping the same entries
        tol = 1e-8 * float(Uty.abs().max())
        free = W0 > 0
        w = torch.where(free, W0, torch.zeros_like(W0))
        eye = lambda k: torch.eye(k, dtype=torch.float64, device=U.device)   # noqa: E731
        self.kkt_settled = False
        added = torch.zeros_like(free)
        for outer in range(50):
            dropped = torch.zeros_like(free)
            while True:   # each pass drops at least one entry, so this ends
                idx = torch.nonzero(free).flatten()
                UF = U[:, idx]
                L = torch.linalg.cholesky(UF.t() @ UF + lam_n * eye(idx.numel()))
                wF = torch.cholesky_solve(Uty[idx][:, None], L)[:, 0]
                neg = wF <= 0
                if not bool(neg.any()):
                    break
                cur = w[idx]
                alpha = float(torch.min(cur[neg] / (cur[neg] - wF[neg])))
                cur = cur + alpha * (wF - cur)
                w[idx] = cur
                drop = idx[cur <= 1e-14 * float(cur.abs().max())]
                w[drop] = 0.0
                free[drop] = False
                dropped[drop] = True
            w.zero_()
            w[idx] = wF
            grad = U.t() @ (U @ w) - Uty + lam_n * w          # gradient of the objective / 2
            viol = (~free) & (grad < -tol)
            if not bool(viol.any()):
                self.kkt_settled = True
                return w, idx, L
            cand = torch.nonzero(viol & ~(dropped & added)).flatten()
            if cand.numel() == 0:
                cand = torch.nonzero(viol).flatten()
            k = max(1, cand.numel() // 4)
            add = cand[torch.argsort(grad[cand])[:k]]
            added.zero_()
            added[add] = True
            free[add] = True
        # not settled within the rounds: the last solve on its free set is returned
        # (kkt_settled stays False); its remaining violations are below the ones added
        return w, idx, L

    def chi2_of_model(self, mp):
        """chi^2 of the unperturbed data (likelihood.py:214-226) for model rows mp (rows,)."""
        nc, nb, amp = self.nc, self.nb, self.amp
        y_rz = self.d["y_rz"]
        t_rz = ((mp[:nc] - y_rz) / (0.1 * y_rz * amp)) ** 2
        surf = mp[nc:nc + nb] * self.lum
        t_xy = ((surf - self.dd.xy) / (0.1 * self.dd.xy * amp)) ** 2
        gam = self.d["gamma"]
        gam = torch.where(gam.abs() > 1e-8, gam, torch.full_like(gam, 1e-8))
        h = (mp[nc + 2 * nb: nc + 6 * nb].reshape(4, nb) / gam[None, :]).clamp(-10.0, 10.0)
        t_h = ((h - self.h_data) / (self.sig_h * amp)) ** 2
        return sum(torch.nansum(t) for t in (t_rz, t_xy, t_h))

    # --------------------------------------------------------------- chi^2 and gradient
    def chi2(self, theta):
        lib = self.soft_library(theta)
        U = self.design(lib)
        w, _, _ = self.solve(lib, U)
        return float(self.chi2_of_model(lib.t() @ w))

    def chi2_and_grad(self, theta, timings=None):
        import time

        def tick(key, t0):
            if timings is not None:
                torch.cuda.synchronize()
                timings[key] = timings.get(key, 0.0) + time.time() - t0
            return time.time()
        t = time.time()
        lib = self.soft_library(theta)
        t = tick("soft_project_s", t)
        U = self.design(lib)
        w, idx, L = self.solve(lib, U)
        t = tick("nnls_kkt_s", t)
        # direct term: chi^2(mp), mp = A^T w (grad mode on: this may run inside an autograd Function)
        with torch.enable_grad():
            mp = (lib.t() @ w).detach().requires_grad_(True)
            c2 = self.chi2_of_model(mp)
            (gmp,) = torch.autograd.grad(c2, mp)
        cot = torch.outer(w, gmp)                                  # dchi^2/dA at fixed w, (n, rows)
        # implicit term through the KKT system on the free set
        gw = lib @ gmp                                             # dchi^2/dw (n,)
        mu = torch.zeros_like(w)
        mu[idx] = torch.cholesky_solve(gw[idx][:, None], L)[:, 0]
        r = U @ w - self.y
        dU = -(torch.outer(r, mu) + torch.outer(U @ mu, w))         # (m, n)
        dA_rows = (dU * self.row_scale[:, None]).t()               # (n, m): d/dA[:, row_map]
        cot.index_add_(1, self.row_map.long(), dA_rows)
        t = tick("implicit_s", t)
        grad = self.project_adjoint(theta, cot)
        tick("adjoint_s", t)
        if timings is not None:
            timings["free_set"] = int(idx.numel())
        return float(c2.detach()), grad

    def project_adjoint(self, theta, cot):
        """dL/dtheta (4,) for a cotangent dL/dlibrary (n, rows) of the soft library."""
        a, b, g, vs = (float(t) for t in theta)
        R, dR = rotation_and_derivatives(a, b, g)
        for i in range(9):
            self.geo.rot[i] = float(R.reshape(-1)[i])
        drot = (ctypes.c_double * 27)(*(float(v) for v in dR.reshape(-1)))     # host array
        grad = torch.zeros(4, dtype=torch.float64, device=self.library.device)
        cot = cot.contiguous()
        kernels._check(cot, "cotangent", torch.float64, (self.n, self.rows))
        call("smx_soft_project_adjoint", ctypes.byref(self.geo), SMX_FP64, self.sigma_pix, vs, ctypes.addressof(drot),
             kernels._ptr(self.samples), kernels._ptr(self.n_stored), self.slots, kernels._ptr(self.info),
             kernels._ptr(self.t_total), kernels._ptr(self.dd.bin_mapping), kernels._ptr(self.dd.num_per_bin),
             kernels._ptr(self.dd.v0), kernels._ptr(self.dd.s), kernels._ptr(cot), kernels._ptr(grad),
             kernels._stream())
        return grad

    def geometry_dict(self):
        """Sky geometry for the dense reference (oracle.soft_projection)."""
        g = self.geo
        return dict(xlo=g.X_lo, ylo=g.Y_lo, dx=(g.X_hi - g.X_lo) / g.nX, dy=(g.Y_hi - g.Y_lo) / g.nY, nX=g.nX,
                    nY=g.nY, n_bins=g.n_bins, n_part=g.n_part, n_real=g.n_real, bin_mapping=self.dd.bin_mapping,
                    num_per_bin=self.dd.num_per_bin, v0=self.dd.v0, s=self.dd.s, area=self.dd.area_pixel)


class SoftChi2(torch.autograd.Function):
    """chi2 = SoftChi2.apply(theta, problem): theta (4,) double = (alpha, beta, gamma [rad], vscale)."""

    @staticmethod
    def forward(ctx, theta, problem):
        c2, grad = problem.chi2_and_grad(theta.detach().cpu().numpy())
        ctx.save_for_backward(grad.to(theta.device, theta.dtype))
        return torch.tensor(c2, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None


def problem_from_evaluation(theta12, dict_data, num_Vbin, Rzphi_n_tot, settings=None, sigma_pix=0.5,
                            precision="fp64"):
    """Builds the orbits of one evaluation (model_likelihood's ICs and integration)
    and returns (SoftProblem, theta0) with theta0 the evaluation's (alpha, beta,
    gamma [rad], 1.0)."""
    from .likelihood import grid_of, unpack_params
    from .potentials import potential_struct
    st = engine.settings_from(settings, precision=precision)
    halo, bary = unpack_params(theta12)
    pot = potential_struct(bary, halo, st.bulge_mass)
    dd = engine.device_data(dict_data, st.n_real)
    grid = grid_of(dict_data)
    libd = engine.build_library(pot, bary, dd, grid, st)
    n = libd["library"].shape[0]
    y_rz_raw = kernels.density_target(pot, st.dtype, dd.R_grid, dd.z_grid, dd.phi_grid, dd.dR, dd.dz, dd.dphi,
                                      dd.sample)
    d = engine.data_terms(dd, bary, y_rz_raw, n)
    row_scale, Y = engine.nnls_inputs(d, dd, grid.n_cells, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    lum = float(d["mmpo"].item()) * d["l2m"]
    prob = SoftProblem(libd["bufs"], libd["ic"]["t_total"], libd["geo"], libd["library"], d, dd, row_scale, Y[0],
                       lum, sigma_pix=sigma_pix)
    theta0 = np.array([math.radians(float(bary[k])) for k in ("alpha", "beta", "gamma")] + [1.0])
    return prob, theta0
