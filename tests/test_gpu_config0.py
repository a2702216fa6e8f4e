"""The plain FP64 evaluation at the size of the reference's CPU-runnable case
(2,048 particles x 4 realisations, 50 circular periods with 500 samples each,
40 x 40 pixels in 120 apertures, a 20 x 16 x 10 (R, z, phi) grid, 100 bootstraps),
checked stage by stage against the oracle on the kernels' own inputs:

* every stored sample's four images: (R, z, phi) cell and aperture bit for bit
  (oracle/grid.py, utils.py:10-42 and integrates.py:115-147);
* the library columns binned by the oracle from the same samples, normalised and
  averaged over realisations (integrates.py:207-238, 287-298);
* the bootstrap ADMM weights against the oracle's Cholesky ADMM (nnls.py:68-166);
* the model maps, h -> (V, sigma) and the bootstrap chi^2 (model.py:14-68,
  likelihood.py:192-238);
* the mixed-precision NNLS on the float-rounded library against the oracle on the same
  library: the bootstrap chi^2 within 0.1.
Integrating 8,192 orbits for 50 periods in NumPy would take hours, so the orbits are
the FP64 kernel's (their parity with the oracle integrator is checked on shorter
horizons in test_gpu_kernels.py)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def run():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import engine, synthetic
    from schwarmax_gb300.likelihood import grid_of, unpack_params
    from schwarmax_gb300.potentials import potential_struct
    cfg = synthetic.CONFIGS[0]
    dict_data, theta = synthetic.make_dataset(cfg, seed=0)
    st = cfg.settings("fp64")
    dd = engine.DeviceData(dict_data, n_real=st.n_real)
    halo, bary = unpack_params(theta)
    pot = potential_struct(bary, halo, st.bulge_mass)
    grid = grid_of(dict_data)
    r = engine.evaluate(pot, bary, dd, grid, st, cfg.admm_iters, 1.0, want_maps=True)
    torch.cuda.synchronize()
    return dict(cfg=cfg, dd=dd, dict_data=dict_data, bary=bary, r=r, grid=grid, st=st)


def _oracle_geometry(run):
    from oracle import integrate as oi, orbits as oo
    b, g, dd = run["bary"], run["grid"], run["dd"]
    rot = oo.rotation_matrix(b["alpha"], b["beta"], b["gamma"])
    return oi.BinGeometry(rot, g.rzphi_lim, g.n_rzphi, g.xy_lim, g.n_xy, dd.bin_mapping.cpu().numpy(),
                          dd.num_per_bin.cpu().numpy(), dd.v0.cpu().numpy(), dd.s.cpu().numpy())


def _samples(run):
    bufs = run["r"]["lib"]["bufs"]
    smp = bufs.samples.cpu().numpy()                     # (7, n_orb, slots)
    ns = bufs.n_stored.cpu().numpy()
    j = np.arange(bufs.slots)[:, None]
    ys = np.ascontiguousarray(smp[:6].transpose(2, 1, 0))  # (slots, n_orb, 6)
    w = np.where(j < ns[None, :], smp[6].T, 0.0)           # (slots, n_orb)
    return ys, w, ns


def test_config0_bin_indices_bit_exact(run):
    from schwarmax_gb300 import kernels
    ys, w, ns = _samples(run)
    keep = (w > 0).T                                        # (n_orb, slots) stored, weighted samples
    pts = ys.transpose(1, 0, 2)[keep]                       # (N, 6)
    assert pts.shape[0] > 3_000_000
    cells, bins, _ = kernels.sample_cells(run["r"]["lib"]["geo"], torch.as_tensor(pts.T.copy(), device="cuda"),
                                          run["dd"].bin_mapping)
    ref = _oracle_geometry(run).cells(pts)
    for im, (rz_cell, vbin, _) in enumerate(ref):
        np.testing.assert_array_equal(cells[im].cpu().numpy(), rz_cell, err_msg=f"cells of image {im}")
        np.testing.assert_array_equal(bins[im].cpu().numpy(), vbin, err_msg=f"apertures of image {im}")


def test_config0_library_from_the_same_samples(run):
    from oracle import integrate as oi
    from schwarmax_gb300._lib import INFO_EJ, INFO_EJ0, INFO_T
    r, dd = run["r"], run["dd"]
    ys, w, ns = _samples(run)
    n_orb = w.shape[1]
    acc = oi.Accumulator(n_orb, _oracle_geometry(run))
    acc.add(ys, w)
    info = r["lib"]["bufs"].info.cpu().numpy()
    t_total = r["lib"]["ic"]["t_total"].cpu().numpy()
    Rz, surf, h, valid = oi.normalise(acc, info[INFO_EJ0], info[INFO_EJ], info[INFO_T], t_total)
    n_part, n_real = dd.n, run["st"].n_real
    np.testing.assert_array_equal(r["lib"]["valid"].cpu().numpy().astype(bool), valid > 0.5)
    A_rz, A_xy, A_h = oi.realisation_mean(Rz, surf, h, valid, n_part, n_real)
    lib = r["lib"]["library"].cpu().numpy()                 # (n_part, rows): [Rzphi | xy | h0..h4]
    nc, nb = run["grid"].n_cells, dd.n_bins
    ref = np.concatenate([A_rz, A_xy] + [A_h[k] for k in range(5)], axis=0).T
    scale = np.abs(ref).max(0, keepdims=True) + 1e-300      # per row of the design matrix
    assert lib.shape == ref.shape == (n_part, nc + 6 * nb)
    np.testing.assert_allclose(lib / scale, ref / scale, rtol=0, atol=1e-11)


def _maps_and_logl(run, W, lib):
    from oracle import model as omodel
    from schwarmax_gb300 import engine
    r, dd = run["r"], run["dd"]
    d = r["data"]
    nc, nb = run["grid"].n_cells, dd.n_bins
    lum = float(d["mmpo"].item()) * float(d["l2m"])
    cols = lambda a, b: lib[:, a:b].T                       # noqa: E731
    A_h = [cols(nc + (1 + k) * nb, nc + (2 + k) * nb) for k in range(1, 5)]
    gamma = d["gamma"].cpu().numpy()
    d3, d2, h1, h2, h3, h4, V, sig = omodel.compute_model_batch(W, cols(0, nc), cols(nc, nc + nb), *A_h, gamma,
                                                                dd.v0.cpu().numpy(), dd.s.cpu().numpy())
    d2 = d2 * lum
    y_xy_b, y_h_b, sh = (t.cpu().numpy() for t in engine.likelihood_data(dd))
    y_rz = d["y_rz"].cpu().numpy()
    y_xy = dd.xy.cpu().numpy()
    res = np.nansum(((d3 - y_rz) / (0.1 * y_rz)) ** 2) + np.nansum(((d2 - y_xy_b) / (0.1 * y_xy)) ** 2, axis=1)
    for k, hk in enumerate((h1, h2, h3, h4)):
        res = res + np.nansum(((hk - y_h_b[k]) / sh[k]) ** 2, axis=1)
    return np.concatenate([d3, d2, h1, h2, h3, h4, V, sig], axis=1), -0.5 * res


def _oracle_weights(run, lib):
    from oracle import nnls as onnls
    from schwarmax_gb300 import engine
    r, dd = run["r"], run["dd"]
    nc = run["grid"].n_cells
    row_scale, Y = engine.nnls_inputs(r["data"], dd, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    rm = engine.row_map(nc, dd.n_bins).cpu().numpy()
    U = (lib[:, rm] * row_scale.cpu().numpy()[None]).T       # (m, n)
    w_init = float((r["data"]["y_rz"].sum() / lib.shape[0]).item())
    return onnls.admm(U, Y.cpu().numpy(), w_init, 1.0, run["cfg"].admm_iters), w_init


def test_config0_weights_maps_and_chi2(run):
    r = run["r"]
    lib = r["lib"]["library"].cpu().numpy()
    Z, _ = _oracle_weights(run, lib)
    W = r["W"].cpu().numpy()
    np.testing.assert_allclose(W, Z, rtol=0, atol=1e-9 * np.abs(Z).max())
    maps_ref, logl_ref = _maps_and_logl(run, Z, lib)
    sc = np.abs(maps_ref).max(0, keepdims=True) + 1e-300
    np.testing.assert_allclose(r["maps"].cpu().numpy() / sc, maps_ref / sc, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r["logl"].cpu().numpy(), logl_ref, rtol=1e-9)


def test_config0_mixed_nnls_chi2_within_0p1(run):
    from schwarmax_gb300 import engine, kernels
    r, dd = run["r"], run["dd"]
    nc, nb = run["grid"].n_cells, dd.n_bins
    lib32 = r["lib"]["library"].float().contiguous()
    lib = lib32.double().cpu().numpy()
    Z, w_init = _oracle_weights(run, lib)
    row_scale, Y = engine.nnls_inputs(r["data"], dd, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    Wm = kernels.nnls_admm(lib32, engine.row_map(nc, nb), row_scale, Y, run["cfg"].admm_iters, 1.0, w_init,
                           mixed=True).cpu().numpy()
    _, logl_ref = _maps_and_logl(run, Z, lib)
    _, logl_m = _maps_and_logl(run, Wm, lib)
    assert np.abs(2 * (logl_m - logl_ref)).max() <= 0.1
    assert np.abs(Wm - Z).max() <= 1e-6 * np.abs(Z).max()
