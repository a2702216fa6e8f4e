"""Post-analysis kernels (build_Lcirc_of_E, circularity, histogram2d, the PSF
transfer matrix) against the reference's own outputs and the oracle."""
import numpy as np
import pytest

from conftest import golden, params_from_flat

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def an():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import analysis
    return analysis


def test_lcirc_matches_reference(an):
    from schwarmax_gb300.potentials import potential_func
    g = golden("analysis")
    pb, ph = params_from_flat(g["params"])
    interp, E, L = an.build_Lcirc_of_E(potential_func, (pb, ph), n_grid=400)
    np.testing.assert_allclose(E, g["E_circ"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(L, g["L_circ"], rtol=1e-9, atol=1e-12 * np.abs(g["L_circ"]).max())
    Lq = interp(g["E_query"])
    np.testing.assert_allclose(Lq, g["L_query"], rtol=1e-8, atol=1e-9 * np.abs(g["L_query"]).max())
    Ld = interp(torch.as_tensor(g["E_query"], device="cuda"))
    assert Ld.is_cuda


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_circularity_matches_oracle(an, dtype):
    from oracle import analysis as oa, potential as op
    from schwarmax_gb300.potentials import potential_func
    g = golden("analysis")
    pb, ph = params_from_flat(g["params"])
    interp, _, _ = an.build_Lcirc_of_E(potential_func, (pb, ph), n_grid=400)
    oi, _, _ = oa.build_Lcirc_of_E(op.canonical_params(pb, ph), n_grid=400)
    rng = np.random.default_rng(2)
    n = 5000
    R = rng.uniform(0.3, 15, n)
    ph_ = rng.uniform(0, 2 * np.pi, n)
    pts = np.stack([R * np.cos(ph_), R * np.sin(ph_), rng.normal(0, 0.5, n), rng.normal(0, 150, n),
                    rng.normal(0, 150, n), rng.normal(0, 60, n)])
    lam, Rd, Ed = an.circularity(torch.as_tensor(pts, dtype=dtype, device="cuda").contiguous(), pb, ph, interp)
    lo, Ro, Eo = oa.circularity(pts.astype(np.float64) if dtype == torch.float64
                                else pts.astype(np.float32).astype(np.float64), op.canonical_params(pb, ph), oi)
    tol = 1e-8 if dtype == torch.float64 else 2e-4
    np.testing.assert_allclose(Ed.double().cpu().numpy(), Eo, rtol=tol)
    np.testing.assert_allclose(Rd.double().cpu().numpy(), Ro, rtol=tol)
    np.testing.assert_allclose(lam.double().cpu().numpy(), lo, rtol=tol, atol=tol)


def test_histogram2d_matches_numpy(an):
    rng = np.random.default_rng(3)
    n = 200_000
    a = rng.uniform(-1.2, 1.2, n)
    b = rng.normal(0, 0.6, n)
    a[:3] = [-1.0, 1.0, 0.25]          # edges and an interior edge
    b[:3] = [1.0, -1.0, 0.0]
    w = rng.uniform(0, 2, n)
    ref, _, _ = np.histogram2d(a, b, bins=[50, 70], range=[[-1, 1], [-1, 1]], weights=w)
    out = an.histogram2d(torch.as_tensor(a, device="cuda"), torch.as_tensor(b, device="cuda"), (50, 70),
                         [[-1, 1], [-1, 1]], torch.as_tensor(w, device="cuda"))
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-10, atol=1e-9)
    cnt, _, _ = np.histogram2d(a, b, bins=[50, 70], range=[[-1, 1], [-1, 1]])
    out = an.histogram2d(torch.as_tensor(a, device="cuda"), torch.as_tensor(b, device="cuda"), (50, 70),
                         [[-1, 1], [-1, 1]])
    np.testing.assert_array_equal(out.cpu().numpy(), cnt)


def test_transfer_matrix_matches_reference(an):
    g = golden("analysis")
    d = golden("example_data")
    nX, nY = (int(v) for v in d["out_nX_nY"])
    P = an.compute_transfer_matrix(float(g["psf_sigma"]), nX, nY, d["out_X_minmax"], d["out_Y_minmax"],
                                   d["out_bin_mapping"], int(d["out_total_bins"]), grid_res=int(g["psf_grid_res"]))
    np.testing.assert_allclose(P.cpu().numpy(), g["psf_P"], rtol=0, atol=1e-11)
    eye = an.compute_transfer_matrix(0, nX, nY, d["out_X_minmax"], d["out_Y_minmax"], d["out_bin_mapping"], 5)
    assert torch.equal(eye.cpu(), torch.eye(5, dtype=torch.float64))


def test_apply_psf_to_library(an):
    rng = np.random.default_rng(4)
    nc, nb, n = 10, 6, 20
    lib = torch.as_tensor(rng.uniform(0, 1, (n, nc + 6 * nb)), device="cuda")
    P = torch.as_tensor(rng.uniform(0, 1, (nb, nb)), device="cuda")
    P = P / P.sum(0, keepdim=True)
    out = an.apply_psf(lib, P, nc, nb)
    assert torch.equal(out[:, :nc], lib[:, :nc])
    for k in range(6):
        sl = slice(nc + k * nb, nc + (k + 1) * nb)
        np.testing.assert_allclose(out[:, sl].cpu().numpy(), (P.cpu().numpy() @ lib[:, sl].cpu().numpy().T).T,
                                   rtol=1e-12)
