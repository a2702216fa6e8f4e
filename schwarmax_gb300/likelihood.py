"""Likelihood layer with the reference's entry points (likelihood.py:73-336).

``model_likelihood(params, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify)``
unpacks the 12-D theta exactly as likelihood.py:105-165 (including the
(logM_enc, log c) -> (logM, logRs) Newton solve), runs one model evaluation on
the GPU and returns the log-mean-exp over the bootstrap log-likelihoods.  The
chi^2 terms (likelihood.py:199-238) are reduced in double inside
``smx_model_maps``.  ``settings=`` selects the integrator constants and the
precision (see engine.Settings).
"""
import math

import torch

from . import engine
from .engine import Grid, device_data, settings_from
from .model import model_deltaChi2_jackknife
from .potentials import density_func, potential_func, potential_struct  # noqa: F401
from .utils import logMenc_logc_to_logM_logRs

__all__ = ["model_likelihood", "model_likelihood_batch", "calculate_delta_chi2", "chi2_func", "density_func",
           "potential_func", "unpack_params"]


def unpack_params(params):
    p = [float(v) for v in (params.tolist() if hasattr(params, "tolist") else params)]
    logM_halo, logRs_halo = logMenc_logc_to_logM_logRs(p[0], p[3], r_enc=10.0, Delta=200.0, rho_crit=277.54)
    L_bar = 10.0 ** p[6]
    Hs = 10.0 ** p[5]
    halo = dict(logM=logM_halo, Rs=10 ** logRs_halo, a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0,
                z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    bary = dict(logM_disc=p[1], Rs_disc=10 ** p[4], Hs_disc=Hs, logM_bar=p[2], L_bar=L_bar, a_bar=L_bar / 5.0,
                b_bar=Hs, mass_to_light_ratio=10 ** p[10], Omega_bar=10 ** p[11], x_origin=0.0, y_origin=0.0,
                z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0, alpha=p[7] * 180 / math.pi,
                beta=p[8] * 180 / math.pi, gamma=p[9] * 180 / math.pi)
    return halo, bary


def grid_of(dict_data):
    if isinstance(dict_data, engine.DeviceData):
        dict_data = dict_data.source

    def f(v):
        return [float(x) for x in (v.tolist() if hasattr(v, "tolist") else v)]
    nR = [int(v) for v in (dict_data["Rzphi_n_grid"].tolist() if hasattr(dict_data["Rzphi_n_grid"], "tolist")
                           else dict_data["Rzphi_n_grid"])]
    nXY = [int(v) for v in (dict_data["nX_nY"].tolist() if hasattr(dict_data["nX_nY"], "tolist")
                            else dict_data["nX_nY"])]
    return Grid(tuple(nR), [f(dict_data["R_minmax"]), f(dict_data["z_minmax"]), f(dict_data["phi_minmax"])],
                [f(dict_data["X_minmax"]), f(dict_data["Y_minmax"])], tuple(nXY))


def log_likelihoods(params, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None, nnls_maxiter=200,
                    cache=True, want_maps=False):
    """The bootstrap log-likelihoods logl_all (N_boot,) as a device tensor, and the evaluation."""
    st = settings_from(settings)
    halo, bary = unpack_params(params)
    grid = grid_of(dict_data)
    if grid.n_cells != int(Rzphi_n_tot):
        raise ValueError("Rzphi_n_tot does not match dict_data['Rzphi_n_grid']")
    dd = device_data(dict_data, st.n_real, cache=cache)
    if int(num_Vbin) != dd.n_bins:
        raise ValueError("num_Vbin does not match dict_data")
    pot = potential_struct(bary, halo, st.bulge_mass)
    r = engine.evaluate(pot, bary, dd, grid, st, nnls_maxiter, 1.0, sigma_amplify=sigma_amplify, want_maps=want_maps)
    return r["logl"], r


def log_likelihoods_batch(params_batch, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None,
                          nnls_maxiter=200, cache=True, max_points=None, blocks_per_sm=0, keep=False):
    """Bootstrap log-likelihoods (P, N_boot) of P parameter points evaluated as one batch."""
    st = settings_from(settings)
    grid = grid_of(dict_data)
    if grid.n_cells != int(Rzphi_n_tot):
        raise ValueError("Rzphi_n_tot does not match dict_data['Rzphi_n_grid']")
    dd = device_data(dict_data, st.n_real, cache=cache)
    if int(num_Vbin) != dd.n_bins:
        raise ValueError("num_Vbin does not match dict_data")
    pots, barys = [], []
    for th in params_batch:
        halo, bary = unpack_params(th)
        pots.append(potential_struct(bary, halo, st.bulge_mass))
        barys.append(bary)
    r = engine.evaluate_batch(pots, barys, dd, grid, st, nnls_maxiter, 1.0, sigma_amplify=sigma_amplify,
                              max_points=max_points, blocks_per_sm=blocks_per_sm, keep=keep)
    return r["logl"], r


def model_likelihood_batch(params_batch, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None,
                           nnls_maxiter=200, cache=True, max_points=None):
    """jax.vmap(model_likelihood) over the rows of params_batch (P, 12), as the
    reference's grid search and MCMC call it (example/example_schwarmax.ipynb
    cells 8 and 12).  Returns a NumPy array of the P marginal log-likelihoods."""
    logl, _ = log_likelihoods_batch(params_batch, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify, settings,
                                    nnls_maxiter, cache, max_points)
    m = torch.max(logl, dim=1, keepdim=True).values
    lme = m[:, 0] + torch.log(torch.mean(torch.exp(logl - m), dim=1))
    return lme.cpu().numpy()


def log_mean_exp(logl):
    m = torch.max(logl)
    return m + torch.log(torch.mean(torch.exp(logl - m)))


def model_likelihood(params, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None, nnls_maxiter=200,
                     cache=True):
    """likelihood.py:96-244.  Returns the marginal log-likelihood as a Python float."""
    logl, _ = log_likelihoods(params, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify, settings, nnls_maxiter, cache)
    return float(log_mean_exp(logl).item())


def chi2_func(y_Rzphi, y_Rzphi_model, sigma_Rzphi, y_xy, y_xy_model, sigma_xy,
              y_h1, y_h1_model, sigma_h1, y_h2, y_h2_model, sigma_h2,
              y_h3, y_h3_model, sigma_h3, y_h4, y_h4_model, sigma_h4):
    """likelihood.py:73-94 on torch tensors: only the h1..h4 terms are returned."""
    r = [torch.nansum(((a - b) / s) ** 2) for a, b, s in ((y_h1, y_h1_model, sigma_h1), (y_h2, y_h2_model, sigma_h2),
                                                            (y_h3, y_h3_model, sigma_h3), (y_h4, y_h4_model, sigma_h4))]
    return -0.5 * (r[0] + r[1] + r[2] + r[3])


def calculate_delta_chi2(params, dict_data, num_Vbin, Rzphi_n_tot, settings=None, nnls_maxiter=200):
    """likelihood.py:248-336 (leave-one-bin-out jackknife).  Returns a float."""
    halo, bary = unpack_params(params)
    g = grid_of(dict_data)
    d = model_deltaChi2_jackknife(density_func, potential_func, chi2_func, halo, bary, dict_data, num_Vbin,
                                  Rzphi_n_tot, g.n_rzphi, g.rzphi_lim, g.xy_lim, g.n_xy, nnls_maxiter=nnls_maxiter,
                                  regularization=1.0, n_groups=int(num_Vbin), batch_size=25, settings=settings)
    return float(d.item())
