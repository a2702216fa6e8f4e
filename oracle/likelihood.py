"""Likelihood layer (likelihood.py:73-336, utils.py:514-569), FP64 oracle."""
import math

import numpy as np

from . import model
from .constants import EPSILON


def logM_logRs_to_logMenc_logc(logM, logRs, r_enc=10.0, Delta=200.0, rho_crit=277.54):
    M, Rs = 10.0 ** logM, 10.0 ** logRs
    x = r_enc / Rs
    M_enc = M * (math.log(1.0 + x) - x / (1.0 + x))
    R_vir = (3.0 * M / (4.0 * math.pi * Delta * rho_crit)) ** (1.0 / 3.0)
    return math.log10(M_enc), math.log10(R_vir / Rs)


def logMenc_logc_to_logM_logRs(logM_enc, log_c, r_enc=10.0, Delta=200.0, rho_crit=277.54):
    """Six Newton steps from logM_enc + 0.5 (utils.py:526-569)."""
    M_enc = 10.0 ** logM_enc
    c = 10.0 ** log_c
    coeff = 4.0 * math.pi * Delta * rho_crit / 3.0
    ln10 = math.log(10.0)
    logM = logM_enc + 0.5
    for _ in range(6):
        M = 10.0 ** logM
        Rs = (M / coeff) ** (1.0 / 3.0) / c
        x = r_enc / Rs
        f_nfw = math.log(1.0 + x) - x / (1.0 + x)
        f = M * f_nfw - M_enc
        df = (f_nfw - x * x / (3.0 * (1.0 + x) ** 2)) * M * ln10
        logM = logM - f / df
    Rs = (10.0 ** logM / coeff) ** (1.0 / 3.0) / c
    return logM, math.log10(Rs)


def unpack_params(params):
    """12-D theta -> (params_halo_pot, params_baryon_rho) (likelihood.py:105-165)."""
    p = [float(v) for v in params]
    logM_halo, logRs_halo = logMenc_logc_to_logM_logRs(p[0], p[3])
    L_bar = 10.0 ** p[6]
    Hs = 10.0 ** p[5]
    halo = dict(logM=logM_halo, Rs=10 ** logRs_halo, a=1.0, b=1.0, c=1.0, x_origin=0.0,
                y_origin=0.0, z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    bary = dict(logM_disc=p[1], Rs_disc=10 ** p[4], Hs_disc=Hs, logM_bar=p[2], L_bar=L_bar,
                a_bar=L_bar / 5.0, b_bar=Hs, mass_to_light_ratio=10 ** p[10], Omega_bar=10 ** p[11],
                x_origin=0.0, y_origin=0.0, z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0,
                alpha=p[7] * 180 / math.pi, beta=p[8] * 180 / math.pi, gamma=p[9] * 180 / math.pi)
    return halo, bary


def grid_args(dict_data):
    Rm, zm, pm = dict_data["R_minmax"], dict_data["z_minmax"], dict_data["phi_minmax"]
    return dict(Rzphi_n_grid=np.asarray(dict_data["Rzphi_n_grid"]),
                Rzphi_lim_grid=np.array([Rm, zm, pm], dtype=np.float64),
                xy_lim_grid=np.array([dict_data["X_minmax"], dict_data["Y_minmax"]], dtype=np.float64),
                xy_n_grid=np.asarray(dict_data["nX_nY"]))


def chi2_terms(md, dict_data, sigma_amplify=1.0):
    """likelihood.py:192-238; returns logl_all (B,)."""
    y_rz = md["density_3d"]
    y_xy = np.asarray(dict_data["XY_density_data"], np.float64)
    yh = [np.asarray(dict_data[f"h{k}_data"], np.float64) for k in range(1, 5)]
    sxy_raw = np.asarray(dict_data["XY_density_data_err"], np.float64) + EPSILON
    sh_raw = [np.asarray(dict_data[f"h{k}_data_err"], np.float64) + EPSILON for k in range(1, 5)]
    y_xy_b = y_xy[None] + np.asarray(dict_data["XY_standard_normal"]) * sxy_raw[None]
    yh_b = [yh[k][None] + np.asarray(dict_data[f"h{k + 1}_standard_normal"]) * sh_raw[k][None] for k in range(4)]
    with np.errstate(divide="ignore", invalid="ignore"):
        s_rz = 0.1 * y_rz * sigma_amplify
        s_xy = 0.1 * y_xy * sigma_amplify
        res_rz = np.nansum(((md["density_3d_model"] - y_rz) / s_rz) ** 2)
        res_xy = np.nansum(((md["surface_density"] - y_xy_b) / s_xy) ** 2, axis=1)
        res_h = [np.nansum(((md[f"h{k + 1}"] - yh_b[k]) / (sh_raw[k] * sigma_amplify)) ** 2, axis=1)
                 for k in range(4)]
    return -0.5 * (res_h[0] + res_h[1] + res_h[2] + res_h[3] + res_xy + res_rz)


def log_mean_exp(l):
    m = np.max(l)
    return m + np.log(np.mean(np.exp(l - m)))


def model_likelihood(params, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None,
                     nnls_maxiter=200, return_model=False):
    halo, bary = unpack_params(params)
    md = model.build_model(halo, bary, dict_data, num_Vbin, Rzphi_n_tot, nnls_maxiter=nnls_maxiter,
                           regularization=1.0, settings=settings, **grid_args(dict_data))
    logl = chi2_terms(md, dict_data, sigma_amplify)
    out = log_mean_exp(logl)
    if return_model:
        return out, logl, md
    return out


def chi2_func(y_Rzphi, y_Rzphi_model, sigma_Rzphi, y_xy, y_xy_model, sigma_xy,
              y_h1, y_h1_model, sigma_h1, y_h2, y_h2_model, sigma_h2,
              y_h3, y_h3_model, sigma_h3, y_h4, y_h4_model, sigma_h4):
    """likelihood.py:73-94: only the h1-h4 terms enter the return value."""
    r = [np.nansum(((a - b) / s) ** 2) for a, b, s in ((y_h1, y_h1_model, sigma_h1), (y_h2, y_h2_model, sigma_h2),
                                                         (y_h3, y_h3_model, sigma_h3), (y_h4, y_h4_model, sigma_h4))]
    return -0.5 * (r[0] + r[1] + r[2] + r[3])


def calculate_delta_chi2(params, dict_data, num_Vbin, Rzphi_n_tot, settings=None, nnls_maxiter=200,
                         library=None):
    halo, bary = unpack_params(params)
    return model.model_deltaChi2_jackknife(chi2_func, halo, bary, dict_data, num_Vbin, Rzphi_n_tot,
                                           nnls_maxiter=nnls_maxiter, regularization=1.0,
                                           n_groups=num_Vbin, batch_size=25, settings=settings,
                                           library=library, **grid_args(dict_data))
