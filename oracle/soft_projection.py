"""Dense FP64 PyTorch reference of the differentiable projection + NNLS chi^2.

Test infrastructure only (tests/ import it to check
smx_soft_project, smx_soft_project_adjoint and schwarmax_gb300.adjoint).  The
reference has no such path (it stops gradients at its NNLS, nnls.py:66,165);
what this restates is the hard binning of integrates.py:115-174 with each
sample image spread over the pixels by a pixel-integrated Gaussian, the
per-realisation normalisation of integrates.py:207-238,287-298, the NNLS KKT
system on a fixed free set (the solution of nnls.py:68-166 once converged) and
the chi^2 terms of likelihood.py:214-226.  Every step is a differentiable
torch operation, so torch.autograd gives the reference gradient.
"""
import math

import torch

KMS = 0.9777922216807892
EPS = 1e-12
WIN = 3


def rotation(theta):
    """R = (Rz(g) Rx(b) Rz(a))^T from theta = (alpha, beta, gamma) (radians, tensors)."""
    a, b, g = theta[0], theta[1], theta[2]
    one, zero = torch.ones_like(a), torch.zeros_like(a)

    def Rz(t):
        c, s = torch.cos(t), torch.sin(t)
        return torch.stack([torch.stack([c, -s, zero]), torch.stack([s, c, zero]), torch.stack([zero, zero, one])])

    def Rx(t):
        c, s = torch.cos(t), torch.sin(t)
        return torch.stack([torch.stack([one, zero, zero]), torch.stack([zero, c, -s]), torch.stack([zero, s, c])])

    return (Rz(g) @ Rx(b) @ Rz(a)).T


def realisation_scales(info, t_total, n_part, n_real, symmetry=True):
    """Sample weight scale per orbit: valid_r / ((sum_r valid_r + 0.1) T_r)."""
    T, EJ0, EJ, WSUM = info[0], info[1], info[2], info[3]
    ok = ((EJ / EJ0 - 1).abs() < 0.1) & (T > t_total / 10)
    v = ok.double().reshape(n_part, n_real)
    nv = v.sum(1, keepdim=True)
    Ti = (4.0 if symmetry else 1.0) * WSUM.reshape(n_part, n_real) + EPS
    return (v / ((nv + 0.1) * Ti)).reshape(-1)


def soft_sky_rows(samples, n_stored, info, t_total, geo, theta, sigma_pix):
    """Sky rows (n_part, 6 nb) = [xy | h0..h4] with soft apertures at theta = (alpha, beta, gamma, vscale).

    samples (7, n_orb, slots) double; geo: dict with xlo, ylo, dx, dy, nX, nY, n_bins,
    n_part, n_real, bin_mapping (nX nY + 1,), num_per_bin, v0, s, area (pixel area x 1e6)."""
    n_part, n_real, nb = geo["n_part"], geo["n_real"], geo["n_bins"]
    n_orb = n_part * n_real
    slots = samples.shape[2]
    dev = samples.device
    R = rotation(theta[:3])
    vs = theta[3]
    sc = realisation_scales(info, t_total, n_part, n_real)
    j = torch.arange(slots, device=dev)
    keep = (j[None, :] < n_stored[:, None].long()) & (samples[6] != 0) & (sc[:, None] != 0)
    o_idx, s_idx = torch.nonzero(keep, as_tuple=True)
    w = samples[6][o_idx, s_idx] * sc[o_idx]
    q = samples[:6][:, o_idx, s_idx]                       # (6, N)
    part = o_idx // n_real
    xs, ws, ps = [], [], []
    for sxy, sz in ((1.0, 1.0), (1.0, -1.0), (-1.0, 1.0), (-1.0, -1.0)):
        sgn = torch.tensor([sxy, sxy, sz], dtype=q.dtype, device=dev)
        xs.append(torch.cat([q[:3] * sgn[:, None], q[3:] * sgn[:, None]]))
        ws.append(w)
        ps.append(part)
    Q = torch.cat(xs, 1)
    w = torch.cat(ws)
    part = torch.cat(ps)
    X = R[0] @ Q[:3]
    Y = R[1] @ Q[:3]
    vl = vs * (R[2] @ Q[3:]) * KMS
    u = (X - geo["xlo"]) / geo["dx"]
    v = (Y - geo["ylo"]) / geo["dy"]
    isig = 1.0 / (math.sqrt(2.0) * sigma_pix)

    def axis(c, n):
        first = torch.floor(c.detach().clamp(-16, n + 16)).long() - WIN
        k = torch.arange(2 * WIN + 1, device=dev)
        idx = first[:, None] + k[None, :]
        lo = (idx.double() - c[:, None]) * isig
        wgt = 0.5 * (torch.erf(lo + isig) - torch.erf(lo))
        inside = (idx >= 0) & (idx < n)
        return torch.where(inside, wgt, torch.zeros_like(wgt)), idx.clamp(0, n - 1), inside

    wx, ix, inx = axis(u, geo["nX"])
    wy, iy, iny = axis(v, geo["nY"])
    W = wx[:, None, :] * wy[:, :, None]                    # (N, 7y, 7x)
    pix = ix[:, None, :] + geo["nX"] * iy[:, :, None]
    b = geo["bin_mapping"].long()[pix]
    valid = inx[:, None, :] & iny[:, :, None] & (b >= 0) & (b < nb)
    bcl = b.clamp(0, nb - 1)
    s_b = geo["s"][bcl]
    yv = (vl[:, None, None] - geo["v0"][bcl]) / s_b
    g = torch.exp(-0.5 * yv * yv) / (math.sqrt(2.0 * math.pi) * s_b)
    sq2, sq3 = math.sqrt(2.0), math.sqrt(3.0)
    H = [torch.ones_like(yv), sq2 * yv]
    H.append((sq2 * yv * H[1] - 1.0) / sq2)
    H.append((sq2 * yv * H[2] - sq2 * H[1]) / sq3)
    H.append((sq2 * yv * H[3] - sq3 * H[2]) / 2.0)
    contrib = torch.where(valid, w[:, None, None] * W, torch.zeros_like(W))
    flat = (part[:, None, None] * nb + bcl).reshape(-1)
    out = torch.zeros(6, n_part * nb, dtype=samples.dtype, device=dev)
    out[0] = out[0].index_add(0, flat, contrib.reshape(-1))
    for k in range(5):
        out[1 + k] = out[1 + k].index_add(0, flat, (contrib * g * H[k]).reshape(-1))
    out = out.reshape(6, n_part, nb).permute(1, 0, 2).reshape(n_part, 6 * nb)
    norm = torch.cat([geo["num_per_bin"] * geo["area"] + EPS, torch.ones(5 * nb, dtype=out.dtype, device=dev)])
    return out / norm[None, :]


def kkt_solution(U, y, lam_n, free):
    """w with w_F = (U_F^T U_F + lam_n I)^-1 U_F^T y on the fixed free set F, 0 elsewhere (differentiable)."""
    idx = torch.nonzero(free).flatten()
    UF = U[:, idx]
    H = UF.t() @ UF + lam_n * torch.eye(idx.numel(), dtype=U.dtype, device=U.device)
    wF = torch.linalg.solve(H, UF.t() @ y)
    w = torch.zeros(U.shape[1], dtype=U.dtype, device=U.device)
    return w.index_put((idx,), wF)


def active_set(U, y, lam_n, free0, max_steps=50):
    """Free set after dropping negative KKT entries (no gradient)."""
    free = free0.clone()
    with torch.no_grad():
        for _ in range(max_steps):
            w = kkt_solution(U, y, lam_n, free)
            bad = free & (w <= 0)
            if not bool(bad.any()):
                return free
            free &= ~bad
    raise RuntimeError("active set did not settle")


def chi2(mp, nc, nb, y_rz, y_xy, gamma, h_data, sig_h, lum, amp=1.0):
    """chi^2 of the unperturbed data for model rows mp (likelihood.py:214-226)."""
    t_rz = ((mp[:nc] - y_rz) / (0.1 * y_rz * amp)) ** 2
    t_xy = ((mp[nc:nc + nb] * lum - y_xy) / (0.1 * y_xy * amp)) ** 2
    g = torch.where(gamma.abs() > 1e-8, gamma, torch.full_like(gamma, 1e-8))
    h = (mp[nc + 2 * nb: nc + 6 * nb].reshape(4, nb) / g[None, :]).clamp(-10.0, 10.0)
    t_h = ((h - h_data) / (sig_h * amp)) ** 2
    return torch.nansum(t_rz) + torch.nansum(t_xy) + torch.nansum(t_h)
