"""End-to-end GPU evaluations through the reference-named entry points,
against golden vectors produced by the reference's own code."""
import numpy as np
import pytest

from conftest import golden, tiny_dict_data

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def smx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import schwarmax_gb300
    return schwarmax_gb300


def _grid_kw(dd):
    return dict(Rzphi_n_grid=dd["Rzphi_n_grid"], Rzphi_lim_grid=np.array([dd["R_minmax"], dd["z_minmax"],
                                                                          dd["phi_minmax"]]),
                xy_lim_grid=np.array([dd["X_minmax"], dd["Y_minmax"]]), xy_n_grid=dd["nX_nY"])


def test_model_likelihood_fp64_matches_reference(smx):
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    logl = smx.model_likelihood(g["theta"], dd, 4, 48, sigma_amplify=float(g["sigma_amplify"]),
                                settings=dict(precision="fp64"))
    ref = float(g["logL"])
    assert abs(logl - ref) <= 1e-6 * abs(ref), (logl, ref)


def test_build_model_fp64_matches_reference(smx):
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    halo, bary = smx.unpack_params(g["theta"])
    out = smx.build_model(smx.density_func, smx.potential_func, halo, bary, dd, 4, 48, nnls_maxiter=60,
                          settings=dict(precision="fp64"), **_grid_kw(dd))
    for k in ("density_3d", "density_3d_model", "surface_density", "h1", "h2", "h3", "h4", "V", "sigma", "weights"):
        ref = g["bm_" + k]
        np.testing.assert_allclose(out[k].cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max(), err_msg=k)


def test_model_likelihood_mixed_precision_error(smx):
    """The mixed evaluation of the tiny case, quantity by quantity.  Its FP32 orbits
    diverge from their FP64 twins along the 5,000 attempts (a chaotic potential), so
    the end-to-end logL is not bounded here; what precision controls is:
      * the Jacobi-integral drift of the FP32 orbits, set by rtol as in FP64;
      * the mixed NNLS against the FP64 NNLS on the same FP32 library (the solver's
        contract): every bootstrap chi^2 within 0.1, weights within 1e-6 of the largest."""
    from schwarmax_gb300 import _lib, engine, kernels
    from schwarmax_gb300.likelihood import grid_of, log_likelihoods
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    logl32, r32 = log_likelihoods(g["theta"], dd, 4, 48, sigma_amplify=float(g["sigma_amplify"]))
    logl64, r64 = log_likelihoods(g["theta"], dd, 4, 48, sigma_amplify=float(g["sigma_amplify"]),
                                  settings=dict(precision="fp64"))
    assert torch.isfinite(logl32).all()

    def drift(r):
        info = r["lib"]["bufs"].info.double()
        return (info[_lib.INFO_EJ] / info[_lib.INFO_EJ0] - 1).abs().max().item()
    assert drift(r32) <= 10 * drift(r64) + 1e-5, (drift(r32), drift(r64))
    # same FP32 library, FP64 NNLS + maps
    lib = r32["lib"]["library"]
    d = r32["data"]
    ddv = engine.device_data(dd)
    row_scale, Y = engine.nnls_inputs(d, ddv, 48, (np.sqrt(5.0), np.sqrt(5.0), 1.0))
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    W64 = kernels.nnls_admm(lib.double(), engine.row_map(48, 4), row_scale, Y, 200, 1.0, w_init, mixed=False)
    y_xy_b, y_h_b, sh = engine.likelihood_data(ddv)
    lum = float(d["mmpo"].item()) * d["l2m"]
    _, l64 = kernels.model_maps(lib.double(), 48, 4, W64, d["gamma"].contiguous(), ddv.v0, ddv.s,
                                d["y_rz"].contiguous(), ddv.xy, y_xy_b, y_h_b, sh, lum, float(g["sigma_amplify"]))
    assert float((2 * (logl32 - l64)).abs().max()) <= 0.1
    assert float((r32["W"] - W64).abs().max()) <= 1e-6 * float(W64.abs().max())


def test_mixed_nnls_on_the_fp64_library(smx):
    """Mixed NNLS (split bf16 tensor-core products, FP64 factor) vs FP64 NNLS on
    the same library: weights within 1e-6 of the largest and chi^2 within 0.1."""
    from schwarmax_gb300 import engine, kernels
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    halo, bary = smx.unpack_params(g["theta"])
    out = smx.build_model(smx.density_func, smx.potential_func, halo, bary, dd, 4, 48, nnls_maxiter=200,
                          settings=dict(precision="fp64"), return_library=True, **_grid_kw(dd))
    r = out["_eval"]
    lib = r["lib"]["library"]
    d = r["data"]
    row_scale, Y = engine.nnls_inputs(d, engine.device_data(dd), 48, (np.sqrt(5.0), np.sqrt(5.0), 1.0))
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    W64 = kernels.nnls_admm(lib, engine.row_map(48, 4), row_scale, Y, 200, 1.0, w_init, mixed=False)
    W32 = kernels.nnls_admm(lib.float().contiguous(), engine.row_map(48, 4), row_scale, Y, 200, 1.0, w_init,
                            mixed=True)
    np.testing.assert_allclose(W64.cpu().numpy(), out["weights"].cpu().numpy(), rtol=1e-12, atol=1e-14)
    scale = float(W64.abs().max())
    assert float((W32 - W64).abs().max()) <= 1e-6 * scale
    ddv = engine.device_data(dd)
    y_xy_b, y_h_b, sh = engine.likelihood_data(ddv)
    lum = float(d["mmpo"].item()) * d["l2m"]

    def chi2(W):
        _, ll = kernels.model_maps(lib, 48, 4, W, d["gamma"].contiguous(), ddv.v0, ddv.s, d["y_rz"].contiguous(),
                                   ddv.xy, y_xy_b, y_h_b, sh, lum, float(g["sigma_amplify"]), want_maps=False)
        return -2.0 * ll.cpu().numpy()

    assert np.abs(chi2(W32) - chi2(W64)).max() <= 0.1


def test_calculate_delta_chi2_fp64_matches_reference(smx):
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    d = smx.calculate_delta_chi2(g["theta"], dd, 4, 48, settings=dict(precision="fp64"))
    ref = float(g["delta_chi2"])
    assert abs(d - ref) <= 1e-5 * abs(ref), (d, ref)


def test_get_model_with_orbit_fp64_matches_reference(smx):
    g = golden("end_to_end")
    w = golden("with_orbit")
    dd = tiny_dict_data(g)
    dd["jitter_uniforms_traj"] = w["jitter_uniforms"]
    halo, bary = smx.unpack_params(g["theta"])
    out = smx.get_model_with_orbit(smx.density_func, smx.potential_func, halo, bary, dd, 4, 48, nnls_maxiter=60,
                                   settings=dict(precision="fp64"), **_grid_kw(dd))
    for k in ("t_traj", "y_traj", "weights_all_boot", "density_3d_model", "surface_density", "h1", "V", "sigma"):
        ref = w["mo_" + k]
        np.testing.assert_allclose(out[k].cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max(), err_msg=k)


def test_noncanonical_model_rejected(smx):
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    halo, bary = smx.unpack_params(g["theta"])
    with pytest.raises(NotImplementedError):
        smx.build_model(lambda *a: 0, smx.potential_func, halo, bary, dd, 4, 48, **_grid_kw(dd))
    bad = dict(bary, x_origin=1.0)
    with pytest.raises(NotImplementedError):
        smx.build_model(smx.density_func, smx.potential_func, halo, bad, dd, 4, 48, **_grid_kw(dd))


def test_poisson_bootstrap_matches_oracle(smx):
    """The Poisson-weighted bootstrap (config 1's resampling: aperture g of resample b
    weighted by k_bg ~ Poisson(1)), FP64: every resample's weights against the oracle's
    Cholesky ADMM on the row-scaled design, and its weighted chi^2 (likelihood.py:214-226
    with the weights) against NumPy on the oracle's model maps."""
    from oracle import model as omodel, nnls as onnls
    from schwarmax_gb300 import engine
    from schwarmax_gb300.likelihood import log_likelihoods
    g = golden("end_to_end")
    dd = tiny_dict_data(g)
    amp = float(g["sigma_amplify"])
    logl, r = log_likelihoods(g["theta"], dd, 4, 48, sigma_amplify=amp,
                              settings=dict(precision="fp64", bootstrap="poisson"))
    ddv = engine.device_data(dd)
    lib = r["lib"]["library"].cpu().numpy()
    d = r["data"]
    nc, nb, B = 48, 4, ddv.n_boot
    row_scale, Y0 = engine.nnls_inputs(d, ddv, nc, (np.sqrt(5.0), np.sqrt(5.0), 1.0), boot=False)
    rm = engine.row_map(nc, nb).cpu().numpy()
    U = (lib[:, rm] * row_scale.cpu().numpy()[None]).T
    K = engine.poisson_weights(B, nb, 0).cpu().numpy()
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    Z = []
    for b in range(B):
        sq = np.sqrt(np.concatenate([np.ones(nc)] + [K[b]] * 5))
        Z.append(onnls.admm(U * sq[:, None], (Y0.cpu().numpy()[0] * sq)[None], w_init, 1.0, 200)[0])
    Z = np.array(Z)
    W = r["W"].cpu().numpy()
    np.testing.assert_allclose(W, Z, rtol=0, atol=1e-9 * np.abs(Z).max())
    cols = lambda a, b_: lib[:, a:b_].T          # noqa: E731
    lum = float(d["mmpo"].item()) * float(d["l2m"])
    d3, d2, h1, h2, h3, h4, _, _ = omodel.compute_model_batch(
        Z, cols(0, nc), cols(nc, nc + nb), *[cols(nc + (1 + k) * nb, nc + (2 + k) * nb) for k in range(1, 5)],
        d["gamma"].cpu().numpy(), ddv.v0.cpu().numpy(), ddv.s.cpu().numpy())
    y_rz, xy = d["y_rz"].cpu().numpy(), ddv.xy.cpu().numpy()
    sh = (ddv.h_err + 1e-12).cpu().numpy()
    hd = ddv.h.cpu().numpy()
    res = np.nansum(((d3 - y_rz) / (0.1 * y_rz * amp)) ** 2) + np.nansum(K * ((d2 * lum - xy) / (0.1 * xy * amp)) ** 2, 1)
    for k, hk in enumerate((h1, h2, h3, h4)):
        res = res + np.nansum(K * ((hk - hd[k]) / (sh[k] * amp)) ** 2, 1)
    np.testing.assert_allclose(logl.cpu().numpy(), -0.5 * res, rtol=1e-9)
