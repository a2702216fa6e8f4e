"""Forward model with the reference's entry points (model.py:14-850).

``build_model``, ``get_model_with_orbit``, ``model_deltaChi2_jackknife`` and
``compute_model_single`` keep the reference's names and arguments so that a
caller of the reference can switch.  Differences, all additive:
  * ``density_func`` / ``potential_func`` must be the canonical descriptors of
    ``schwarmax_gb300.potentials`` (callables cannot cross the C ABI).
  * ``settings=`` (engine.Settings or dict) exposes the integrator constants the
    reference hard-codes (model.py:127, 163-169) and the precision
    ("mixed": FP32 orbits + TF32/FP64 NNLS, "fp64": everything in double).
  * Random draws come from dict_data ('jeans_normals', 'jitter_uniforms'), see
    engine.py.
Outputs are torch tensors on the GPU with the reference's keys and shapes.
"""
import math

import numpy as np
import torch

from . import engine, kernels
from .engine import KPCGYR_TO_KMS, Grid, device_data, settings_from, split_maps
from .potentials import model_types, potential_struct, require_canonical

_DEF_NGRID = (10, 6, 6)
_DEF_LIM = ((0, 10.0), (-3, 3), (-math.pi, math.pi))
_DEF_XYLIM = ((-10.0, 10.0), (-3.0, 3.0))
_DEF_XYN = (60, 40)


def _grid(Rzphi_n_grid, Rzphi_lim_grid, xy_lim_grid, xy_n_grid):
    def arr(v):
        if isinstance(v, torch.Tensor):
            v = v.detach().cpu().numpy()
        return np.asarray(v, dtype=np.float64)
    return Grid(tuple(int(v) for v in arr(Rzphi_n_grid)), arr(Rzphi_lim_grid), arr(xy_lim_grid),
                tuple(int(v) for v in arr(xy_n_grid)))


def compute_model_single(w, A_Rzphi, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, v0, s):
    """model.py:14-66 for one weight vector (torch tensors, any device)."""
    eps = 1e-8
    g = torch.where(gamma_kin.abs() > eps, gamma_kin, torch.full_like(gamma_kin, eps))
    d3 = A_Rzphi @ w
    d2 = A_xy @ w
    hs = [torch.clamp((A @ w) / g, -10.0, 10.0) for A in (A_h1, A_h2, A_h3, A_h4)]
    from .ghmoments import h_to_V_sigma
    V, sig = h_to_V_sigma(hs[0], hs[1], v0, s, h3=hs[2], h4=hs[3])
    return d3, d2, hs[0], hs[1], hs[2], hs[3], V, sig


def build_model(density_func, potential_func, params_halo_pot, params_disk_rho, dict_data, num_Vbin,
                Rzphi_n_tot=360, Rzphi_n_grid=_DEF_NGRID, Rzphi_lim_grid=_DEF_LIM, xy_lim_grid=_DEF_XYLIM,
                xy_n_grid=_DEF_XYN, nnls_maxiter=200, regularization=1.0, settings=None, return_library=False):
    """model.py:70-286 on the GPU.  Returns the reference's dict (torch tensors)."""
    require_canonical(density_func, potential_func)
    st = settings_from(settings)
    grid = _grid(Rzphi_n_grid, Rzphi_lim_grid, xy_lim_grid, xy_n_grid)
    if grid.n_cells != int(Rzphi_n_tot):
        raise ValueError(f"Rzphi_n_tot={Rzphi_n_tot} does not match the grid ({grid.n_cells} cells)")
    dd = device_data(dict_data, st.n_real)
    if int(num_Vbin) != dd.n_bins:
        raise ValueError(f"num_Vbin={num_Vbin} does not match dict_data ({dd.n_bins} bins)")
    pot = potential_struct(params_disk_rho, params_halo_pot, st.bulge_mass,
                           **model_types(density_func, potential_func))
    r = engine.evaluate(pot, params_disk_rho, dd, grid, st, nnls_maxiter, regularization)
    out = dict(density_3d=r["data"]["y_rz"])
    out.update(split_maps(r["maps"], r["n_cells"], r["n_bins"]))
    out["weights"] = r["W"]
    if return_library:
        out["_eval"] = r
    return out


def get_model_with_orbit(density_func, potential_func, params_halo_pot, params_disk_rho, dict_data, num_Vbin,
                         Rzphi_n_tot=360, Rzphi_n_grid=_DEF_NGRID, Rzphi_lim_grid=_DEF_LIM, xy_lim_grid=_DEF_XYLIM,
                         xy_n_grid=_DEF_XYN, nnls_maxiter=200, regularization=1.0, settings=None):
    """model.py:606-850: one realisation per particle, every attempt stored,
    no symmetry images, NNLS weights w = 1.  The jitter draws are
    dict_data['jitter_uniforms_traj'] (6, n, 1) when present."""
    require_canonical(density_func, potential_func)
    st = settings_from(settings)
    grid = _grid(Rzphi_n_grid, Rzphi_lim_grid, xy_lim_grid, xy_n_grid)
    dd = device_data(dict_data, st.n_real)
    pot = potential_struct(params_disk_rho, params_halo_pot, st.bulge_mass,
                           **model_types(density_func, potential_func))
    r = engine.evaluate(pot, params_disk_rho, dd, grid, st, nnls_maxiter, regularization, weights=(1.0, 1.0, 1.0),
                        trajectory=True)
    bufs = r["lib"]["bufs"]
    n, N = dd.n, bufs.slots
    traj = bufs.samples[:6].permute(1, 2, 0).reshape(n, 1, N, 6).clone()
    traj[..., 3:] *= KPCGYR_TO_KMS
    t_traj = torch.cumsum(bufs.samples[6], dim=1).reshape(n, 1, N)
    W = r["W"]
    out = dict(weights=W[0], weights_all_boot=W, y_traj=traj, t_traj=t_traj,
               rotation_matrix=torch.as_tensor(engine.rotation_matrix(params_disk_rho["alpha"], params_disk_rho["beta"],
                                                                       params_disk_rho["gamma"])),
               Omega_bar=params_disk_rho["Omega_bar"], n_particles=n, n_realizations=1,
               mass_per_orbit=r["data"]["mmpo"], density_3d=r["data"]["y_rz"])
    out.update(split_maps(r["maps"], r["n_cells"], r["n_bins"]))
    return out


def model_deltaChi2_jackknife(density_func, potential_func, chi2_func, params_halo_pot, params_disk_rho, dict_data,
                              num_Vbin, Rzphi_n_tot=360, Rzphi_n_grid=_DEF_NGRID, Rzphi_lim_grid=_DEF_LIM,
                              xy_lim_grid=_DEF_XYLIM, xy_n_grid=_DEF_XYN, nnls_maxiter=200, regularization=1.0,
                              n_groups=100, batch_size=50, settings=None):
    """model.py:290-603: replicate g sets sigma of the xy and h1..h4 rows of the
    bins with bin % n_groups == g to 1e20 and re-solves the NNLS; returns the
    standard deviation of chi2_func over the replicates.  ``chi2_func`` is
    called with torch tensors (the canonical one is likelihood.chi2_func)."""
    require_canonical(density_func, potential_func)
    st = settings_from(settings)
    grid = _grid(Rzphi_n_grid, Rzphi_lim_grid, xy_lim_grid, xy_n_grid)
    dd = device_data(dict_data, st.n_real)
    pot = potential_struct(params_disk_rho, params_halo_pot, st.bulge_mass,
                           **model_types(density_func, potential_func))
    libd = engine.build_library(pot, params_disk_rho, dd, grid, st)
    return jackknife_of_library(chi2_func, libd["library"], pot, params_disk_rho, dd, grid, st, nnls_maxiter,
                                regularization, n_groups)


def jackknife_of_library(chi2_func, lib, pot, params_disk_rho, dd, grid, st, nnls_maxiter=200, regularization=1.0,
                         n_groups=100):
    """The leave-group-out part of model_deltaChi2_jackknife (model.py:480-603) on a
    library that is already built (for instance one of a batch of parameter points).
    Mixed precision with groups of at most 8 bins: all replicates in one batched solve;
    otherwise one solve per replicate."""
    n = lib.shape[0]
    nc, nb = grid.n_cells, dd.n_bins
    y_rz_raw = kernels.density_target(pot, st.dtype, dd.R_grid, dd.z_grid, dd.phi_grid, dd.dR, dd.dz, dd.dphi,
                                      dd.sample)
    d = engine.data_terms(dd, params_disk_rho, y_rz_raw, n)
    w_init = float((d["y_rz"].sum() / n).item())
    lum = float(d["mmpo"].item()) * d["l2m"]
    rm = engine.row_map(nc, nb)
    grp = torch.arange(nb, device="cuda") % n_groups
    per_group = -(-nb // int(n_groups))
    if st.nnls_mixed and 5 * per_group <= 40 and int(n_groups) >= 1:
        return _jackknife_batched(chi2_func, lib, d, dd, nc, nb, int(n_groups), per_group, rm, w_init, lum,
                                  nnls_maxiter, regularization)
    chi2 = []
    zeros_b = torch.zeros(1, nb, dtype=torch.float64, device="cuda")
    for g in range(n_groups):
        drop = grp == g
        sxy = torch.where(drop, torch.full_like(d["sig_xy"], 1e20), d["sig_xy"])
        sh = torch.where(drop[None], torch.full_like(d["sh"], 1e20), d["sh"])
        row_scale, Y = engine.nnls_inputs(d, dd, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0), boot=False,
                                          sig_xy=sxy, sig_h=sh)
        W = kernels.nnls_admm(lib, rm, row_scale, Y, nnls_maxiter, regularization, w_init,
                              mixed=st.nnls_mixed)
        maps, _ = kernels.model_maps(lib, nc, nb, W, d["gamma"].contiguous(), dd.v0, dd.s, d["y_rz"].contiguous(),
                                     dd.xy, (dd.xy[None] + zeros_b).contiguous(),
                                     (dd.h[:, None, :]).contiguous(), (dd.h_err + 1e-12).contiguous(), lum)
        m = split_maps(maps, nc, nb)
        chi2.append(chi2_func(d["y_rz"], m["density_3d_model"][0], d["sig_rz"], d["y_xy"] * lum,
                              m["surface_density"][0], sxy * lum, dd.h[0], m["h1"][0], sh[0], dd.h[1], m["h2"][0],
                              sh[1], dd.h[2], m["h3"][0], sh[2], dd.h[3], m["h4"][0], sh[3]))
    c = torch.stack([torch.as_tensor(v, dtype=torch.float64, device="cuda") for v in chi2])
    return torch.std(c, unbiased=False)


def _jackknife_batched(chi2_func, lib, d, dd, nc, nb, n_groups, per_group, rm, w_init, lum, maxiter, lam):
    """All replicates in one batched solve (smx_nnls_jackknife): replicate g drops the
    design rows (xy, h1..h4) of the bins with bin % n_groups == g; the model maps of
    every replicate come from one product, and chi2_func is applied per replicate with
    the reference's masked sigmas (1e20 on the dropped bins)."""
    from .likelihood import chi2_func as canonical_chi2
    bins = torch.arange(nb, device="cuda")
    drop = torch.full((n_groups, 5 * per_group), -1, dtype=torch.int32, device="cuda")
    for q in range(per_group):
        b = torch.arange(n_groups, device="cuda") + q * n_groups
        ok = b < nb
        for k in range(5):
            drop[:, 5 * q + k] = torch.where(ok, nc + k * nb + b, torch.full_like(b, -1)).to(torch.int32)
    row_scale, Y = engine.nnls_inputs(d, dd, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0), boot=False)
    W = kernels.nnls_jackknife(lib, rm, row_scale, Y[0].contiguous(), drop.contiguous(), maxiter, lam, w_init)
    G = n_groups
    y_xy_b = dd.xy[None].expand(G, nb).contiguous()
    y_h_b = dd.h[:, None, :].expand(4, G, nb).contiguous()
    maps, _ = kernels.model_maps(lib, nc, nb, W, d["gamma"].contiguous(), dd.v0, dd.s, d["y_rz"].contiguous(), dd.xy,
                                 y_xy_b, y_h_b, (dd.h_err + 1e-12).contiguous(), lum)
    m = split_maps(maps, nc, nb)
    dropped = (bins[None, :] % n_groups) == torch.arange(G, device="cuda")[:, None]     # (G, nb)
    sh = torch.where(dropped[None], torch.full((4, G, nb), 1e20, dtype=torch.float64, device="cuda"),
                     d["sh"][:, None, :].expand(4, G, nb))
    if chi2_func is canonical_chi2:
        r = sum(torch.nansum(((dd.h[k][None] - m[f"h{k + 1}"]) / sh[k]) ** 2, dim=1) for k in range(4))
        c = -0.5 * r
    else:
        sxy = torch.where(dropped, torch.full((G, nb), 1e20, dtype=torch.float64, device="cuda"),
                          d["sig_xy"][None].expand(G, nb))
        c = torch.stack([torch.as_tensor(chi2_func(d["y_rz"], m["density_3d_model"][j], d["sig_rz"], d["y_xy"] * lum,
                                                   m["surface_density"][j], sxy[j] * lum, dd.h[0], m["h1"][j], sh[0, j],
                                                   dd.h[1], m["h2"][j], sh[1, j], dd.h[2], m["h3"][j], sh[2, j],
                                                   dd.h[3], m["h4"][j], sh[3, j]), dtype=torch.float64,
                                         device="cuda") for j in range(G)])
    return torch.std(c, unbiased=False)
