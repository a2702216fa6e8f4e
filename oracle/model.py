"""Forward model (model.py:14-850), FP64 oracle.

build_model            model.py:70-286
compute_model_single   model.py:14-68
model_deltaChi2_jackknife  model.py:290-603
get_model_with_orbit   model.py:606-850

Random draws are explicit: dict_data['jeans_normals'] (3, n) replaces the
threefry normals of keys 42/109/2026 and dict_data['jitter_uniforms']
(6, n, n_real) the uniforms of key 911.  Integrator settings default to the
reference's hard-coded values (model.py:163-169) and can be overridden through
`settings` (mode "sampled" is the uniform-time sampling used by the
benchmark configurations).
"""
import math

import numpy as np

from . import integrate, jeans, nnls, orbits, target
from . import potential as pot
from .constants import EPSILON
from .ghmoments import h_to_V_sigma

DEFAULT_SETTINGS = dict(n_real=4, mode="reference", n_attempts=5000, n_periods=50,
                        steps_per_period=100, atol=1e-7, rtol=1e-4, dt_min=1e-5, dt_max=0.3,
                        n_samples=1000, max_attempts=1_000_000, bulge_mass=None)


def compute_model_single(w, A_rz, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, v0, s):
    g = np.where(np.abs(gamma_kin) > 1e-8, gamma_kin, 1e-8)
    d3 = A_rz @ w
    d2 = A_xy @ w
    hs = [np.clip((A @ w) / g, -10.0, 10.0) for A in (A_h1, A_h2, A_h3, A_h4)]
    V, sig = h_to_V_sigma(hs[0], hs[1], v0, s, h3=hs[2], h4=hs[3])
    return d3, d2, hs[0], hs[1], hs[2], hs[3], V, sig


def compute_model_batch(W, A_rz, A_xy, A_h1, A_h2, A_h3, A_h4, gamma_kin, v0, s):
    """compute_model_single vmapped over the rows of W (B, n)."""
    g = np.where(np.abs(gamma_kin) > 1e-8, gamma_kin, 1e-8)
    d3 = W @ A_rz.T
    d2 = W @ A_xy.T
    hs = [np.clip((W @ A.T) / g[None, :], -10.0, 10.0) for A in (A_h1, A_h2, A_h3, A_h4)]
    V, sig = h_to_V_sigma(hs[0], hs[1], v0[None, :], s[None, :], h3=hs[2], h4=hs[3])
    return d3, d2, hs[0], hs[1], hs[2], hs[3], V, sig


def _settings(settings):
    s = dict(DEFAULT_SETTINGS)
    if settings:
        s.update(settings)
    return s


def library_inputs(params_halo_pot, params_disk_rho, dict_data, st, n_real):
    """ICs, V_c, T_orb and jittered start states (model.py:104-148)."""
    P = pot.canonical_params(params_disk_rho, params_halo_pot, st["bulge_mass"])
    w0 = np.asarray(dict_data["w0"], dtype=np.float64)
    w0n = jeans.w0_new(w0, np.asarray(dict_data["jeans_normals"], dtype=np.float64), P)
    R = np.sqrt(w0n[:, 0] ** 2 + w0n[:, 1] ** 2)
    z = w0n[:, 2]
    Vc = orbits.rotation_curve(R, z, P)
    Torb = orbits.orbital_timescale(R, z, P)
    uni = np.asarray(dict_data["jitter_uniforms"], dtype=np.float64)[:, :, :n_real]
    wb = orbits.jitter(w0n, Vc, uni)
    return P, w0n, Vc, Torb, wb


def build_library(params_halo_pot, params_disk_rho, dict_data, Rzphi_n_grid, Rzphi_lim_grid,
                  xy_lim_grid, xy_n_grid, settings=None, n_real=None, trajectory=False):
    st = _settings(settings)
    n_real = st["n_real"] if n_real is None else n_real
    P, w0n, Vc, Torb, wb = library_inputs(params_halo_pot, params_disk_rho, dict_data, st, n_real)
    rot = orbits.rotation_matrix(params_disk_rho["alpha"], params_disk_rho["beta"], params_disk_rho["gamma"])
    geo = integrate.BinGeometry(rot, Rzphi_lim_grid, Rzphi_n_grid, xy_lim_grid, xy_n_grid,
                                dict_data["bin_mapping"], dict_data["num_per_bin"],
                                dict_data["v0"], dict_data["s"])
    Om = float(params_disk_rho["Omega_bar"])
    kw = dict(n_periods=st["n_periods"], steps_per_period=st["steps_per_period"], atol=st["atol"],
              rtol=st["rtol"], dt_min=st["dt_min"], dt_max=st["dt_max"])
    if trajectory:
        lib = integrate.trajectory_library(wb, Torb, P, Om, geo, n_attempts=st["n_attempts"], **kw)
    else:
        lib = integrate.build_library(wb, Torb, P, Om, geo, mode=st["mode"], n_attempts=st["n_attempts"],
                                      n_samples=st["n_samples"], max_attempts=st["max_attempts"], **kw)
    lib.update(P=P, w0_new=w0n, Vc=Vc, T_orb=Torb, w0_batch=wb, rot=rot)
    return lib


def data_terms(dict_data, params_disk_rho, A_Rzphi, P):
    """Target, data scaling and gamma_kin (model.py:190-248)."""
    l2m = 1.0 / float(params_disk_rho["mass_to_light_ratio"])
    y_rz = target.density_target(np.asarray(dict_data["R_grid"]), np.asarray(dict_data["z_grid"]),
                                 np.asarray(dict_data["phi_grid"]), float(dict_data["dR"]),
                                 float(dict_data["dz"]), float(dict_data["dphi"]),
                                 np.asarray(dict_data["sample_for_integration"]), P)
    sig_rz = 0.02 * y_rz + 1e-10
    y_xy = np.asarray(dict_data["XY_density_data"], np.float64) / l2m
    sig_xy = (np.asarray(dict_data["XY_density_data_err"], np.float64) + EPSILON) / l2m
    yh = [np.asarray(dict_data[f"h{k}_data"], np.float64) for k in range(1, 5)]
    sh = [np.asarray(dict_data[f"h{k}_data_err"], np.float64) + EPSILON for k in range(1, 5)]
    mmpo = np.sum(y_rz) / A_Rzphi.shape[1]
    y_xy, sig_xy, y_rz, sig_rz = y_xy / mmpo, sig_xy / mmpo, y_rz / mmpo, sig_rz / mmpo
    X, Y, nXY = dict_data["X_minmax"], dict_data["Y_minmax"], dict_data["nX_nY"]
    area = ((X[1] - X[0]) / nXY[0]) * ((Y[1] - Y[0]) / nXY[1]) * 1e6
    M_b = y_xy * np.asarray(dict_data["num_per_bin"], np.float64) * area
    normGH = 1.0 + yh[3] * math.sqrt(6.0) / 4.0
    gamma_kin = M_b / (normGH * 2.0 * math.sqrt(math.pi) * np.asarray(dict_data["s"], np.float64) + EPSILON)
    return dict(y_rz=y_rz, sig_rz=sig_rz, y_xy=y_xy, sig_xy=sig_xy, yh=yh, sh=sh, mmpo=mmpo,
                gamma_kin=gamma_kin, l2m=l2m)


def build_model(params_halo_pot, params_disk_rho, dict_data, num_Vbin, Rzphi_n_tot=360,
                Rzphi_n_grid=(10, 6, 6), Rzphi_lim_grid=((0, 10.0), (-3, 3), (-math.pi, math.pi)),
                xy_lim_grid=((-10.0, 10.0), (-3.0, 3.0)), xy_n_grid=(60, 40),
                nnls_maxiter=200, regularization=1.0, settings=None, _trajectory=False):
    lib = build_library(params_halo_pot, params_disk_rho, dict_data, Rzphi_n_grid, Rzphi_lim_grid,
                        xy_lim_grid, xy_n_grid, settings,
                        n_real=1 if _trajectory else None, trajectory=_trajectory)
    A_rz, A_xy, A_h = lib["A_Rzphi"], lib["A_xy"], lib["A_h"]
    d = data_terms(dict_data, params_disk_rho, A_rz, lib["P"])
    boots = [d["y_xy"][None, :] + np.asarray(dict_data["XY_standard_normal"]) * d["sig_xy"][None, :]]
    for k in range(4):
        boots.append(d["yh"][k][None, :] + np.asarray(dict_data[f"h{k + 1}_standard_normal"]) * d["sh"][k][None, :])
    wts = dict(w_rzphi=1.0, w_xy=1.0, w_h=1.0) if _trajectory else \
        dict(w_rzphi=math.sqrt(5.0), w_xy=math.sqrt(5.0), w_h=1.0)
    W = nnls.solve_nnls_admm_bootstrap(A_rz, A_xy, A_h[1], A_h[2], A_h[3], A_h[4],
                                       d["y_rz"], d["y_xy"], d["gamma_kin"], *boots,
                                       d["sig_rz"], d["sig_xy"], *d["sh"],
                                       lambda_reg=regularization, maxiter=nnls_maxiter, **wts)
    v0 = np.asarray(dict_data["v0"], np.float64)
    s = np.asarray(dict_data["s"], np.float64)
    d3, d2, h1, h2, h3, h4, V, sig = compute_model_batch(W, A_rz, A_xy, A_h[1], A_h[2], A_h[3], A_h[4],
                                                         d["gamma_kin"], v0, s)
    d2 = d2 * d["mmpo"] * d["l2m"]
    out = dict(density_3d=d["y_rz"], density_3d_model=d3, surface_density=d2, h1=h1, h2=h2,
               h3=h3, h4=h4, V=V, sigma=sig, weights=W)
    out["_lib"] = lib
    out["_data"] = d
    return out


def get_model_with_orbit(params_halo_pot, params_disk_rho, dict_data, num_Vbin, Rzphi_n_tot=360,
                         Rzphi_n_grid=(10, 6, 6), Rzphi_lim_grid=((0, 10.0), (-3, 3), (-math.pi, math.pi)),
                         xy_lim_grid=((-10.0, 10.0), (-3.0, 3.0)), xy_n_grid=(60, 40),
                         nnls_maxiter=200, regularization=1.0, settings=None):
    r = build_model(params_halo_pot, params_disk_rho, dict_data, num_Vbin, Rzphi_n_tot, Rzphi_n_grid,
                    Rzphi_lim_grid, xy_lim_grid, xy_n_grid, nnls_maxiter, regularization, settings,
                    _trajectory=True)
    lib = r["_lib"]
    out = dict(weights=r["weights"][0], weights_all_boot=r["weights"], y_traj=lib["y_traj"],
               t_traj=lib["t_traj"], rotation_matrix=lib["rot"], Omega_bar=params_disk_rho["Omega_bar"],
               n_particles=lib["y_traj"].shape[0], n_realizations=1, mass_per_orbit=r["_data"]["mmpo"])
    for k in ("density_3d", "density_3d_model", "surface_density", "h1", "h2", "h3", "h4", "V", "sigma"):
        out[k] = r[k]
    out["_lib"] = lib
    return out


def model_deltaChi2_jackknife(chi2_func, params_halo_pot, params_disk_rho, dict_data, num_Vbin,
                              Rzphi_n_tot=360, Rzphi_n_grid=(10, 6, 6),
                              Rzphi_lim_grid=((0, 10.0), (-3, 3), (-math.pi, math.pi)),
                              xy_lim_grid=((-10.0, 10.0), (-3.0, 3.0)), xy_n_grid=(60, 40),
                              nnls_maxiter=200, regularization=1.0, n_groups=100, batch_size=50,
                              settings=None, library=None):
    """Leave-group-out jackknife (model.py:290-603): replicate g sets sigma of
    the xy and h1-h4 rows of bins with (bin % n_groups == g) to 1e20, re-solves
    the single-RHS NNLS and evaluates chi2_func; returns std over replicates."""
    lib = library or build_library(params_halo_pot, params_disk_rho, dict_data, Rzphi_n_grid,
                                   Rzphi_lim_grid, xy_lim_grid, xy_n_grid, settings)
    A_rz, A_xy, A_h = lib["A_Rzphi"], lib["A_xy"], lib["A_h"]
    d = data_terms(dict_data, params_disk_rho, A_rz, lib["P"])
    v0 = np.asarray(dict_data["v0"], np.float64)
    s = np.asarray(dict_data["s"], np.float64)
    nb = d["sig_xy"].shape[0]
    grp = np.arange(nb) % n_groups
    lum = d["mmpo"] * d["l2m"]
    chi2 = []
    for g in range(n_groups):
        drop = grp == g
        sxy = np.where(drop, 1e20, d["sig_xy"])
        sh = [np.where(drop, 1e20, x) for x in d["sh"]]
        w = nnls.solve_nnls_admm(A_rz, A_xy, A_h[1], A_h[2], A_h[3], A_h[4],
                                 d["y_rz"], d["y_xy"], d["gamma_kin"], *d["yh"],
                                 d["sig_rz"], sxy, *sh, lambda_reg=regularization,
                                 maxiter=nnls_maxiter, w_rzphi=math.sqrt(5.0), w_xy=math.sqrt(5.0), w_h=1.0)
        d3, d2, h1, h2, h3, h4, _, _ = compute_model_single(w, A_rz, A_xy, A_h[1], A_h[2], A_h[3], A_h[4],
                                                            d["gamma_kin"], v0, s)
        chi2.append(chi2_func(d["y_rz"], d3, d["sig_rz"], d["y_xy"] * lum, d2 * lum, sxy * lum,
                              d["yh"][0], h1, sh[0], d["yh"][1], h2, sh[1],
                              d["yh"][2], h3, sh[2], d["yh"][3], h4, sh[3]))
    return float(np.std(np.array(chi2)))
