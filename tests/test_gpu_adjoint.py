"""Differentiable projection + NNLS (no reference counterpart; the reference stops
gradients at its NNLS): the soft-aperture kernel and its adjoint against the dense
FP64 PyTorch reference in oracle/soft_projection.py, and the chi^2 gradient with
respect to (alpha, beta, gamma, velocity scale) against central finite differences
(step 1e-4 rad / 1e-4 relative) and against autograd of the dense reference."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from schwarmax_gb300 import adjoint, synthetic
    cfg = synthetic.Config("adjoint-test", n_part=48, n_samples=120, n_pix=16, n_bins=10, n_grid=(6, 4, 4), n_boot=3,
                           n_periods=3.0)
    dd, theta = synthetic.make_dataset(cfg, seed=3, precision="fp64")
    p, theta0 = adjoint.problem_from_evaluation(theta, dd, cfg.n_bins, int(np.prod(cfg.n_grid)),
                                                settings=cfg.settings("fp64"), sigma_pix=0.5)
    p.admm_iters = 3000       # converged, so that the free set is that of the exact solution
    return p, theta0


def _ref_rows(p, theta_t):
    from oracle import soft_projection as sp
    return sp.soft_sky_rows(p.samples, p.n_stored, p.info, p.t_total, p.geometry_dict(), theta_t, p.sigma_pix)


def test_soft_rows_match_dense_reference(prob):
    p, theta0 = prob
    th = theta0 + np.array([0.05, -0.08, 0.11, 0.07])
    lib = p.soft_library(th)
    ref = _ref_rows(p, torch.tensor(th, dtype=torch.float64, device="cuda"))
    sky = lib[:, p.nc:]
    scale = ref.abs().amax(0).clamp_min(1e-300)
    assert ((sky - ref).abs() / scale[None, :]).max().item() <= 1e-10
    # the Rzphi rows are the hard library's
    assert torch.equal(lib[:, :p.nc], p.library[:, :p.nc])


def test_soft_adjoint_matches_autograd(prob):
    p, theta0 = prob
    th = theta0 + np.array([-0.03, 0.04, 0.02, -0.05])
    g = torch.Generator(device="cuda").manual_seed(11)
    cot = torch.randn(p.n, p.rows, dtype=torch.float64, device="cuda", generator=g)
    ours = p.project_adjoint(th, cot).cpu().numpy()
    th_t = torch.tensor(th, dtype=torch.float64, device="cuda", requires_grad=True)
    L = (cot[:, p.nc:] * _ref_rows(p, th_t)).sum()
    (ref,) = torch.autograd.grad(L, th_t)
    ref = ref.cpu().numpy()
    np.testing.assert_allclose(ours, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


def test_chi2_gradient_vs_fd_and_dense_reference(prob):
    from oracle import soft_projection as sp
    p, theta0 = prob
    th = theta0 + np.array([0.06, 0.05, -0.07, 0.1])
    c2, g = p.chi2_and_grad(th)
    g = g.cpu().numpy()
    assert np.isfinite(c2) and np.all(np.isfinite(g))
    # central finite differences of the same forward model
    h = np.array([1e-4, 1e-4, 1e-4, 1e-4 * th[3]])
    fd = np.zeros(4)
    for t in range(4):
        e = np.zeros(4)
        e[t] = h[t]
        fd[t] = (p.chi2(th + e) - p.chi2(th - e)) / (2 * h[t])
    np.testing.assert_allclose(g, fd, rtol=1e-3, atol=1e-3 * np.abs(fd).max())
    # autograd of the dense reference on the same free set
    lib = p.soft_library(th)
    U = p.design(lib)
    _, idx, _ = p.solve(lib, U)
    free = torch.zeros(p.n, dtype=torch.bool, device="cuda")
    free[idx] = True
    th_t = torch.tensor(th, dtype=torch.float64, device="cuda", requires_grad=True)
    A = torch.cat([p.library[:, :p.nc], _ref_rows(p, th_t)], 1)
    Ut = (A[:, p.row_map.long()] * p.row_scale[None, :]).t()
    w = sp.kkt_solution(Ut, p.y, p.lam / p.n, free)
    c2_ref = sp.chi2(A.t() @ w, p.nc, p.nb, p.d["y_rz"], p.dd.xy, p.d["gamma"], p.h_data, p.sig_h, p.lum)
    (g_ref,) = torch.autograd.grad(c2_ref, th_t)
    g_ref = g_ref.cpu().numpy()
    assert abs(float(c2_ref.detach()) - c2) <= 1e-9 * abs(c2)
    np.testing.assert_allclose(g, g_ref, rtol=1e-6, atol=1e-8 * np.abs(g_ref).max())


def test_soft_chi2_autograd_function(prob):
    from schwarmax_gb300.adjoint import SoftChi2
    p, theta0 = prob
    th = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    c2 = SoftChi2.apply(th, p)
    c2.backward()
    _, g = p.chi2_and_grad(theta0)
    np.testing.assert_allclose(th.grad.numpy(), g.cpu().numpy(), rtol=1e-12)
