"""Pin the FP64 oracle against golden vectors produced by the reference's own
modules (tests/golden/make_golden.py).  CPU only."""
import math

import numpy as np
import pytest

from conftest import golden, params_from_flat
from oracle import ghmoments, grid, integrate, jeans, likelihood, model, nnls, orbits
from oracle import potential as pot


@pytest.mark.parametrize("tag", ["a", "b"])
def test_potential_density_acceleration(tag):
    g = golden("potential")
    pb, ph = params_from_flat(g[f"{tag}_params"])
    P = pot.canonical_params(pb, ph)
    x, y, z = g[f"{tag}_x"], g[f"{tag}_y"], g[f"{tag}_z"]
    np.testing.assert_allclose(pot.phi(x, y, z, P), g[f"{tag}_phi"], rtol=1e-12)
    np.testing.assert_allclose(pot.rho(x, y, z, P), g[f"{tag}_rho"], rtol=1e-11)
    a = np.stack(pot.acc(x, y, z, P), -1)
    scale = np.abs(g[f"{tag}_acc"]).max(axis=1, keepdims=True)
    np.testing.assert_allclose(a / scale, g[f"{tag}_acc"] / scale, rtol=0, atol=1e-10)


def test_gh_basis_and_moments():
    g = golden("small_funcs")
    yv, gau = ghmoments.gauss(g["v"], g["v0"], g["s"])
    np.testing.assert_allclose(yv, g["gh_y"], rtol=1e-14)
    np.testing.assert_allclose(gau, g["gh_gau"], rtol=1e-13)
    np.testing.assert_allclose(np.stack(ghmoments.hermite(yv)), g["gh_H"], rtol=1e-12, atol=1e-14)
    h = g["h"]
    V, sig = ghmoments.h_to_V_sigma(h[0], h[1], g["v0"], g["s"], h3=h[2], h4=h[3])
    np.testing.assert_allclose(V, g["V"], rtol=1e-13)
    np.testing.assert_allclose(sig, g["sig"], rtol=1e-13)


def test_grid_assignment_exact():
    g = golden("small_funcs")
    idx = grid.assign_regular_grid(g["grid_pos"], g["grid_lo"], g["grid_hi"], g["grid_n"])
    np.testing.assert_array_equal(idx, g["grid_idx"])
    # boundary rules: the upper edge and negative offsets are out of range
    assert idx[-3] == np.prod(g["grid_n"]) and idx[-1] == np.prod(g["grid_n"])


def test_rotation_matrix():
    g = golden("small_funcs")
    for a, r in zip(g["angles"], g["rots"]):
        np.testing.assert_allclose(orbits.rotation_matrix(*a), r, rtol=0, atol=1e-15)


def test_halo_parameter_conversion():
    g = golden("small_funcs")
    for (me, lc), (lm, lrs), (me2, lc2) in zip(g["menc"], g["conv"], g["back"]):
        a, b = likelihood.logMenc_logc_to_logM_logRs(me, lc)
        assert abs(a - lm) < 1e-12 and abs(b - lrs) < 1e-12
        c, d = likelihood.logM_logRs_to_logMenc_logc(a, b)
        assert abs(c - me2) < 1e-12 and abs(d - lc2) < 1e-12


def test_orbital_timescale_and_vc():
    g = golden("small_funcs")
    pb, ph = params_from_flat(g["params"])
    P = pot.canonical_params(pb, ph)
    np.testing.assert_allclose(orbits.orbital_timescale(g["orb_R"], g["orb_z"], P), g["orb_T"], rtol=1e-9)
    np.testing.assert_allclose(orbits.rotation_curve(g["orb_R"], g["orb_z"], P), g["orb_Vc"], rtol=1e-9)


def test_jeans_initial_conditions():
    g = golden("jeans")
    pb, ph = params_from_flat(g["params"])
    P = pot.canonical_params(pb, ph)
    w = jeans.w0_new(g["w0"], g["normals"], P)
    np.testing.assert_allclose(w, g["w0_new"], rtol=1e-8, atol=1e-9)


def _geo(g, rot):
    return integrate.BinGeometry(rot, g["geo_Rzphi_lim"], g["geo_nRzphi"], np.array([g["geo_X"], g["geo_Y"]]),
                                 g["geo_nXY"], g["geo_bin_mapping"], g["geo_num_per_bin"], g["geo_v0"], g["geo_s"])


def test_chunked_library_integration():
    g = golden("integrate")
    pb, ph = params_from_flat(g["params"])
    P = pot.canonical_params(pb, ph)
    lib = integrate.library_from_states(g["w0"], g["T_total"], g["dt_init"], P, float(g["Omega_bar"]),
                                        _geo(g, g["rot"]), n_attempts=int(g["N_max"]), chunk=int(g["chunk"]))
    np.testing.assert_allclose(lib["n_valid"], g["n_valid"])
    # each reference output is (n_part, rows); oracle A matrices are (rows, n_part)
    np.testing.assert_allclose(lib["A_Rzphi"].T, g["Rzphi"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(lib["A_xy"].T, g["surface"], rtol=1e-9, atol=1e-20)
    for k in range(5):
        np.testing.assert_allclose(lib["A_h"][k].T, g[f"h{k}"], rtol=1e-8, atol=1e-14)


def test_trajectory_library():
    g = golden("withtraj")
    pb, ph = params_from_flat(g["params"])
    P = pot.canonical_params(pb, ph)
    lib = integrate.trajectory_library(g["w0"], None, P, float(g["Omega_bar"]), _geo(g, g["rot"]),
                                       n_attempts=int(g["N_max"]), T_total=g["T_total"], dt_init=g["dt_init"])
    np.testing.assert_allclose(lib["y_traj"], g["y_traj"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(lib["t_traj"], g["t_traj"], rtol=1e-11)
    np.testing.assert_allclose(lib["A_Rzphi"].T, g["Rzphi"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(lib["A_xy"].T, g["surface"], rtol=1e-9, atol=1e-20)
    for k in range(5):
        np.testing.assert_allclose(lib["A_h"][k].T, g[f"h{k}"], rtol=1e-8, atol=1e-14)


def test_nnls_admm():
    g = golden("nnls")
    A_h = list(g["A_h"])
    sig_h = list(g["sig_h"])
    W = nnls.solve_nnls_admm_bootstrap(g["A_rz"], g["A_xy"], *A_h, g["y_rz"], g["y_xy"], g["gamma"],
                                       g["y_xy_b"], *list(g["y_h_b"]), g["sig_rz"], g["sig_xy"], *sig_h,
                                       lambda_reg=1.0, maxiter=int(g["maxiter"]), w_rzphi=math.sqrt(5.0),
                                       w_xy=math.sqrt(5.0), w_h=1.0)
    np.testing.assert_allclose(W, g["W_boot"], rtol=1e-8, atol=1e-10)
    w1 = nnls.solve_nnls_admm(g["A_rz"], g["A_xy"], *A_h, g["y_rz"], g["y_xy"], g["gamma"], *list(g["y_h"]),
                              g["sig_rz"], g["sig_xy"], *sig_h, lambda_reg=0.5, maxiter=int(g["maxiter"]))
    np.testing.assert_allclose(w1, g["W_single"], rtol=1e-8, atol=1e-10)
    maps = model.compute_model_batch(g["W_boot"], g["A_rz"], g["A_xy"], *A_h, g["gamma"], g["v0"], g["s"])
    for i, m in enumerate(maps):
        np.testing.assert_allclose(m, g[f"map{i}"], rtol=1e-8, atol=1e-8)


def _tiny_dd(g):
    dd = {k[3:]: g[k] for k in g if k.startswith("dd_")}
    dd["total_bins"] = int(dd["total_bins"])
    dd["Rzphi_n_tot"] = int(dd["Rzphi_n_tot"])
    dd["jeans_normals"] = g["jeans_normals"]
    dd["jitter_uniforms"] = g["jitter_uniforms"]
    return dd


@pytest.mark.slow
def test_end_to_end_likelihood_build_model_jackknife():
    """model_likelihood, build_model and calculate_delta_chi2 on 2 particles x 4
    realisations x 5000 attempts.  The libraries are time averages over 50
    orbital periods, so rounding-level differences between the oracle's
    forward-mode gradient and the reference's grad grow along the orbits; the
    outputs still agree to ~1e-6 of their scale."""
    g = golden("end_to_end")
    dd = _tiny_dd(g)
    logl = likelihood.model_likelihood(g["theta"], dd, 4, 48, sigma_amplify=float(g["sigma_amplify"]))
    assert abs(logl - float(g["logL"])) <= 1e-6 * abs(float(g["logL"]))
    halo, bary = likelihood.unpack_params(g["theta"])
    bm = model.build_model(halo, bary, dd, 4, 48, nnls_maxiter=60, **likelihood.grid_args(dd))
    for k in ("density_3d", "density_3d_model", "surface_density", "h1", "h2", "h3", "h4", "V", "sigma", "weights"):
        ref = g["bm_" + k]
        np.testing.assert_allclose(bm[k], ref, rtol=0, atol=1e-5 * np.abs(ref).max(), err_msg=k)
    d = likelihood.calculate_delta_chi2(g["theta"], dd, 4, 48, library=bm["_lib"])
    assert abs(d - float(g["delta_chi2"])) <= 1e-5 * abs(float(g["delta_chi2"]))


@pytest.mark.slow
def test_get_model_with_orbit():
    g = golden("end_to_end")
    w = golden("with_orbit")
    dd = _tiny_dd(g)
    dd["jeans_normals"] = w["jeans_normals"]
    dd["jitter_uniforms"] = w["jitter_uniforms"]
    halo, bary = likelihood.unpack_params(g["theta"])
    mo = model.get_model_with_orbit(halo, bary, dd, 4, 48, nnls_maxiter=60, **likelihood.grid_args(dd))
    for k in ("t_traj", "y_traj", "weights_all_boot", "density_3d_model", "surface_density", "h1", "V", "sigma"):
        ref = w["mo_" + k]
        np.testing.assert_allclose(mo[k], ref, rtol=0, atol=1e-5 * np.abs(ref).max(), err_msg=k)
    assert abs(mo["mass_per_orbit"] - float(w["mo_mass_per_orbit"])) < 1e-12 * float(w["mo_mass_per_orbit"])


@pytest.mark.slow
def test_end_to_end_on_the_example_galaxy():
    """model_likelihood and build_model on the example galaxy's real IFU (609
    Voronoi apertures on 60 x 40 pixels of 0.24 kpc, 10 x 6 x 10 cells; 2 particles x 4
    realisations x 5000 attempts, 3 bootstraps), as the reference computed them.
    Rounding-level differences between the oracle's forward-mode gradient and the
    reference's grad move the orbits by about 1e-6 of their size, which moves a couple
    of the 160,000 samples across a pixel edge into a neighbouring aperture: those few
    apertures differ by a sample's weight (up to 0.3 % of the map's scale), the rest
    agree to 1e-5."""
    g = golden("example_end_to_end")
    dd = _tiny_dd(g)
    nb, nc = dd["total_bins"], dd["Rzphi_n_tot"]
    logl = likelihood.model_likelihood(g["theta"], dd, nb, nc, sigma_amplify=float(g["sigma_amplify"]))
    assert abs(logl - float(g["logL"])) <= 5e-6 * abs(float(g["logL"]))
    halo, bary = likelihood.unpack_params(g["theta"])
    bm = model.build_model(halo, bary, dd, nb, nc, nnls_maxiter=60, **likelihood.grid_args(dd))
    np.testing.assert_array_equal(bm["density_3d"], g["bm_density_3d"])
    for k in ("density_3d_model", "weights"):
        ref = g["bm_" + k]
        np.testing.assert_allclose(bm[k], ref, rtol=0, atol=1e-4 * np.abs(ref).max(), err_msg=k)
    for k in ("surface_density", "h1", "h2", "h3", "h4", "V", "sigma"):
        ref = g["bm_" + k]
        dev = np.abs(np.asarray(bm[k]) - ref) / np.abs(ref).max()
        assert np.median(dev) <= 1e-6, k
        assert np.quantile(dev, 0.99) <= 1e-4, k
        assert np.unique(np.nonzero(dev > 1e-4)[-1]).size <= 8, k      # apertures touched by edge samples


@pytest.mark.slow
def test_jackknife_on_the_example_galaxy():
    """calculate_delta_chi2 (leave-one-bin-out over 609 apertures, likelihood.py:248-336)
    on the example galaxy, as the reference computed it.  The few samples on pixel
    edges (see above) move it by about 1e-5."""
    g = golden("example_end_to_end")
    j = golden("example_jackknife")
    dd = _tiny_dd(g)
    d = likelihood.calculate_delta_chi2(j["theta"], dd, dd["total_bins"], dd["Rzphi_n_tot"])
    ref = float(j["delta_chi2"])
    assert abs(d - ref) <= 1e-4 * abs(ref), (d, ref)


@pytest.mark.parametrize("name", ["T1", "T2", "T3", "T4", "V1", "V2", "V3", "V4"])
def test_dehnen_models_match_reference(name):
    """Every Dehnen & Aly model of the reference (T1..T4, V1..V4): potential, density and
    -grad Phi against the reference's own functions (jax.grad by complex step)."""
    from oracle import dual as Dd, potential as op
    g = golden("dehnen_types")
    M, a, b, L, gam = g[name + "_params"]
    x, y, z = g[name + "_x"], g[name + "_y"], g[name + "_z"]
    code = op.DEHNEN_CODES[name]
    phi = op.DEHNEN_PHI[code](x, y, z, M, a, b, L, gam)
    rho = op.DEHNEN_RHO[code](x, y, z, M, a, b, L, gam)
    np.testing.assert_allclose(phi, g[name + "_phi"], rtol=1e-11, atol=0)
    np.testing.assert_allclose(rho, g[name + "_rho"], rtol=1e-9, atol=1e-12 * np.abs(g[name + "_rho"]).max())
    X, Y, Z = Dd.seed(x, y, z)
    p = op.DEHNEN_PHI[code](X, Y, Z, M, a, b, L, gam)
    acc = -np.stack([p.d[0], p.d[1], p.d[2]], -1)
    np.testing.assert_allclose(acc, g[name + "_acc"], rtol=1e-9, atol=1e-10 * np.abs(g[name + "_acc"]).max())


def test_cylspline_matches_reference():
    """The cylindrical-spline potential (CylindricalSpline.py:354-519, CubicSpline.py:5-305):
    Phi and -grad Phi of a table in get_phi_m's format, and the table's spline second
    derivatives, against the reference's own evaluate_phi / get_acc / jax_precompute_splines."""
    from oracle import cylspline as oc
    g = dict(golden("cylspline"))
    phi, acc = oc.phi_and_acc(g["x"], g["y"], g["z"], g)
    np.testing.assert_allclose(phi, g["phi"], rtol=0, atol=1e-13 * np.abs(g["phi"]).max())
    np.testing.assert_allclose(acc, g["acc"], rtol=0, atol=1e-13 * np.abs(g["acc"]).max())
    for m in g["m"]:
        for part in ("real", "img"):
            Mx, My = oc.precompute_splines(g["Rgrid"], g["Zgrid"], g[f"Phi_m_{part}"][m])
            np.testing.assert_allclose(Mx, g[f"Mx_{part}"][m], rtol=1e-12, atol=1e-12 * np.abs(Mx).max())
            np.testing.assert_allclose(My, g[f"My_{part}"][m], rtol=1e-12, atol=1e-12 * np.abs(My).max())
