"""Batched evaluation over parameter points (jax.vmap(model_likelihood) of the
reference's notebooks) against per-point evaluations, library determinism, and the
mixed solver's chi^2 error at the width of the benchmark library."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def small():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import synthetic
    cfg = synthetic.Config("batch-test", n_part=96, n_samples=60, n_pix=16, n_bins=12, n_grid=(6, 4, 4), n_boot=4,
                           n_periods=3.0, rtol=1e-5)
    dd, theta = synthetic.make_dataset(cfg, seed=5, precision="fp64")
    thetas = np.stack([theta, theta + np.array([0, 0, 0.05, 0, 0, 0, 0, 0.1, -0.1, 0.05, 0.02, 0.03]),
                       theta + np.array([0, 0.02, -0.05, 0, 0, 0, 0.02, -0.05, 0.05, 0.0, -0.03, -0.04])])
    return cfg, dd, thetas


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_points(small, precision):
    """One integrator launch over all points' orbits (one work queue) and one
    projection launch with per-point rotations give each point's single-evaluation
    log-likelihoods."""
    from schwarmax_gb300.likelihood import log_likelihoods, log_likelihoods_batch
    cfg, dd, thetas = small
    st = cfg.settings(precision)
    nc = int(np.prod(cfg.n_grid))
    lb, rb = log_likelihoods_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=80, keep=True)
    assert lb.shape == (len(thetas), cfg.n_boot)
    for q, th in enumerate(thetas):
        ls, rs = log_likelihoods(th, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=80)
        lib_b = rb["libraries"][0][q]
        lib_s = rs["lib"]["library"]
        scale = float(lib_s.abs().max())
        # the batched kernel reads each point's constants from shared memory, the single
        # one from kernel parameters; the compiler may contract a multiply-add differently,
        # and FP32 orbits amplify a rounding difference over the three periods
        tol = 1e-10 if precision == "fp64" else 2e-3
        assert float((lib_b - lib_s).abs().max()) <= tol * scale
        np.testing.assert_allclose(lb[q].cpu().numpy(), ls.cpu().numpy(), rtol=1e-8 if precision == "fp64" else 2e-3)


def test_batch_chunks_agree(small):
    """Splitting the batch into chunks (device memory) changes nothing."""
    from schwarmax_gb300.likelihood import log_likelihoods_batch
    cfg, dd, thetas = small
    st = cfg.settings("fp64")
    nc = int(np.prod(cfg.n_grid))
    a, _ = log_likelihoods_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40)
    b, _ = log_likelihoods_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40, max_points=2)
    np.testing.assert_allclose(a.cpu().numpy(), b.cpu().numpy(), rtol=1e-12)


def test_model_likelihood_batch_api(small):
    import schwarmax_gb300 as smx
    cfg, dd, thetas = small
    nc = int(np.prod(cfg.n_grid))
    st = cfg.settings("fp64")
    v = smx.model_likelihood_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40)
    for q, th in enumerate(thetas):
        s = smx.model_likelihood(th, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40)
        assert abs(v[q] - s) <= 1e-9 * abs(s)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_library_is_deterministic(small, precision):
    """Exact fixed-point binning: the same samples give the same library bit for bit."""
    from schwarmax_gb300 import engine
    from schwarmax_gb300.likelihood import grid_of, unpack_params
    from schwarmax_gb300.potentials import potential_struct
    cfg, dd, thetas = small
    st = cfg.settings(precision)
    halo, bary = unpack_params(thetas[0])
    pot = potential_struct(bary, halo, st.bulge_mass)
    ddv = engine.DeviceData(dd, n_real=st.n_real)
    a = engine.build_library(pot, bary, ddv, grid_of(dd), st)["library"].clone()
    b = engine.build_library(pot, bary, ddv, grid_of(dd), st)["library"]
    assert torch.equal(a, b)


def test_mixed_solver_chi2_at_benchmark_width():
    """Mixed NNLS + maps against FP64 NNLS + maps on one config-1 library
    (16,384 columns, 4,608 + 5 x 400 = 6,608 design rows, 100 bootstraps, 200
    iterations): every bootstrap's chi^2 within 0.05 (the metric allows 0.1)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import engine, kernels, synthetic
    from schwarmax_gb300.likelihood import log_likelihoods
    cfg = synthetic.CONFIGS[1]
    dd, theta = synthetic.make_dataset(cfg, seed=0)
    st = cfg.settings("mixed")
    ddv = engine.DeviceData(dd, n_real=st.n_real)
    nc = int(np.prod(cfg.n_grid))
    logl_m, r = log_likelihoods(theta, ddv, cfg.n_bins, nc, settings=st, nnls_maxiter=200)
    lib = r["lib"]["library"]
    assert lib.shape == (16384, nc + 6 * cfg.n_bins)
    d = r["data"]
    row_scale, Y = engine.nnls_inputs(d, ddv, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    assert Y.shape == (100, 6608)
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    W64 = kernels.nnls_admm(lib.double(), engine.row_map(nc, cfg.n_bins), row_scale, Y, 200, 1.0, w_init,
                            mixed=False)
    y_xy_b, y_h_b, sh = engine.likelihood_data(ddv)
    lum = float(d["mmpo"].item()) * d["l2m"]
    _, logl_64 = kernels.model_maps(lib.double(), nc, cfg.n_bins, W64, d["gamma"].contiguous(), ddv.v0, ddv.s,
                                    d["y_rz"].contiguous(), ddv.xy, y_xy_b, y_h_b, sh, lum, 1.0, want_maps=False)
    dchi2 = (2 * (logl_m - logl_64)).abs()
    assert float(dchi2.max()) <= 0.05, float(dchi2.max())
    assert float((r["W"] - W64).abs().max() / W64.abs().max()) <= 1e-6


@pytest.mark.parametrize("n_groups", [12, 5])
def test_batched_jackknife_matches_per_replicate_solves(small, n_groups):
    """smx_nnls_jackknife (every replicate from the one G^-1 of the full problem:
    Schur complement of the dropped rows, Neumann series for the shift of rho) against
    one FP64 smx_nnls_admm per replicate with the reference's 1e20 sigma masks, on
    the same library."""
    from schwarmax_gb300 import engine, kernels
    from schwarmax_gb300.likelihood import grid_of, unpack_params
    from schwarmax_gb300.potentials import potential_struct
    cfg, dd, thetas = small
    st = cfg.settings("fp64")
    halo, bary = unpack_params(thetas[0])
    pot = potential_struct(bary, halo, st.bulge_mass)
    ddv = engine.DeviceData(dd, n_real=st.n_real)
    grid = grid_of(dd)
    lib = engine.build_library(pot, bary, ddv, grid, st)["library"]
    nc, nb = grid.n_cells, cfg.n_bins
    y_rz = kernels.density_target(pot, torch.float64, ddv.R_grid, ddv.z_grid, ddv.phi_grid, ddv.dR, ddv.dz, ddv.dphi,
                                  ddv.sample)
    d = engine.data_terms(ddv, bary, y_rz, lib.shape[0])
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    rm = engine.row_map(nc, nb)
    w = (math.sqrt(5.0), math.sqrt(5.0), 1.0)
    per = -(-nb // n_groups)
    drop = -np.ones((n_groups, 5 * per), dtype=np.int32)
    for g in range(n_groups):
        bins = np.arange(g, nb, n_groups)
        rows = [nc + k * nb + b for b in bins for k in range(5)]
        drop[g, :len(rows)] = rows
    rs, Y = engine.nnls_inputs(d, ddv, nc, w, boot=False)
    Wb = kernels.nnls_jackknife(lib, rm, rs, Y[0].contiguous(), torch.as_tensor(drop, device="cuda"), 150, 1.0, w_init)
    grp = torch.arange(nb, device="cuda") % n_groups
    for g in range(n_groups):
        m = grp == g
        sxy = torch.where(m, torch.full_like(d["sig_xy"], 1e20), d["sig_xy"])
        sh = torch.where(m[None], torch.full_like(d["sh"], 1e20), d["sh"])
        rsg, Yg = engine.nnls_inputs(d, ddv, nc, w, boot=False, sig_xy=sxy, sig_h=sh)
        Wg = kernels.nnls_admm(lib, rm, rsg, Yg, 150, 1.0, w_init, mixed=False)[0]
        scale = float(Wg.abs().max())
        assert float((Wb[g] - Wg).abs().max()) <= 1e-6 * scale, g


def test_calculate_delta_chi2_batched_matches_loop(small):
    """calculate_delta_chi2 in mixed precision (batched replicates) against the FP64
    per-replicate loop on the same FP64 library."""
    from schwarmax_gb300 import model
    from schwarmax_gb300.likelihood import chi2_func, grid_of, unpack_params
    from schwarmax_gb300.potentials import density_func, potential_func
    cfg, dd, thetas = small
    halo, bary = unpack_params(thetas[1])
    grid = grid_of(dd)
    nc = grid.n_cells
    kw = dict(Rzphi_n_grid=grid.n_rzphi, Rzphi_lim_grid=grid.rzphi_lim, xy_lim_grid=grid.xy_lim, xy_n_grid=grid.n_xy,
              nnls_maxiter=120, n_groups=cfg.n_bins)
    st64 = cfg.settings("fp64")
    ref = model.model_deltaChi2_jackknife(density_func, potential_func, chi2_func, halo, bary, dd, cfg.n_bins, nc,
                                          settings=st64, **kw)
    # the batched path on the same FP64 library: FP64 orbits, mixed NNLS
    st_b = cfg.settings("fp64")
    st_b.nnls = "mixed"
    got = model.model_deltaChi2_jackknife(density_func, potential_func, chi2_func, halo, bary, dd, cfg.n_bins, nc,
                                          settings=st_b, **kw)
    assert abs(float(got) - float(ref)) <= 1e-6 * abs(float(ref)) + 1e-9, (float(got), float(ref))


def test_mixed_solver_at_config4_geometry():
    """The large-library geometry of config 4 (120 x 120 pixels, 1,500 apertures, a
    32 x 32 x 16 grid: 16,384 + 5 x 1,500 = 23,884 design rows, 25,384 library rows)
    with a reduced orbit count: the NNLS workspace, the shared-memory histogram row
    (25,384 int64 = 203 KB) and the Newton-Schulz inverse of a 23,884^2 G at that size,
    against the FP64 solver on the same library."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import engine, kernels, synthetic
    from schwarmax_gb300.likelihood import log_likelihoods
    cfg = synthetic.Config("config4-geometry", n_part=8192, n_samples=100, n_pix=120, n_bins=1500,
                           n_grid=(32, 32, 16), n_boot=10, n_periods=5.0, n_real=1, bar_mass=2e10,
                           omega_kms_kpc=40.0)
    dd, theta = synthetic.make_dataset(cfg, seed=2)
    st = cfg.settings("mixed")
    ddv = engine.DeviceData(dd, n_real=st.n_real)
    nc = 32 * 32 * 16
    logl_m, r = log_likelihoods(theta, ddv, cfg.n_bins, nc, settings=st, nnls_maxiter=50)
    lib = r["lib"]["library"]
    assert lib.shape == (8192, nc + 6 * 1500)
    d = r["data"]
    row_scale, Y = engine.nnls_inputs(d, ddv, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    assert Y.shape == (10, nc + 5 * 1500)
    w_init = float((d["y_rz"].sum() / lib.shape[0]).item())
    W64 = kernels.nnls_admm(lib.double(), engine.row_map(nc, cfg.n_bins), row_scale, Y, 50, 1.0, w_init, mixed=False)
    y_xy_b, y_h_b, sh = engine.likelihood_data(ddv)
    lum = float(d["mmpo"].item()) * d["l2m"]
    _, logl_64 = kernels.model_maps(lib.double(), nc, cfg.n_bins, W64, d["gamma"].contiguous(), ddv.v0, ddv.s,
                                    d["y_rz"].contiguous(), ddv.xy, y_xy_b, y_h_b, sh, lum, 1.0, want_maps=False)
    assert float((2 * (logl_m - logl_64)).abs().max()) <= 0.05
    assert float((r["W"] - W64).abs().max() / W64.abs().max()) <= 1e-6


def test_autotuned_batch_gives_the_same_results(small, tmp_path, monkeypatch):
    """The tuner's launch choices (blocks per SM, queue order) change no result; its
    choice is cached."""
    from schwarmax_gb300 import autotune
    from schwarmax_gb300.likelihood import log_likelihoods_batch
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "autotune.json"))
    cfg, dd, thetas = small
    st = cfg.settings("fp64")
    nc = int(np.prod(cfg.n_grid))
    a, _ = log_likelihoods_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40)
    st.autotune = True
    b, _ = log_likelihoods_batch(thetas, dd, cfg.n_bins, nc, settings=st, nnls_maxiter=40)
    np.testing.assert_allclose(a.cpu().numpy(), b.cpu().numpy(), rtol=1e-12)
    assert autotune.load()
