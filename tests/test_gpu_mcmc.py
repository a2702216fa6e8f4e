"""Device RMH steps against the CPU restatement, a Gaussian target, and a short
run on the batched model likelihood."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import _lib
    return _lib


def test_rmh_step_matches_oracle(lib):
    from oracle.mcmc import rmh_step
    from schwarmax_gb300.kernels import _ptr, _stream
    rng = np.random.default_rng(0)
    C, D = 40, 5
    lo, hi = -np.ones(D) * 2, np.ones(D) * 2
    x = rng.uniform(-1, 1, (C, D))
    L = np.tril(rng.normal(0, 0.3, (D, D)))
    eps = rng.normal(size=(C, D))
    u = rng.uniform(size=C)
    mu = rng.normal(0, 0.5, D)

    def ll(z):
        return -0.5 * np.sum((z - mu) ** 2, axis=1)

    lp = -np.sum(np.log(hi - lo)) + ll(x)
    lp[3] = -np.inf
    xr, lpr, accr = rmh_step(x, lp, L, eps, u, lo, hi, ll)
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    xd, lpd, Ld, ed, ud, lod, hid = d(x), d(lp), d(L), d(eps), d(u), d(lo), d(hi)
    xp = torch.empty_like(xd)
    lpri = torch.empty(C, dtype=torch.float64, device="cuda")
    acc = torch.empty(C, dtype=torch.int32, device="cuda")
    lib.call("smx_rmh_propose", _ptr(xd), _ptr(Ld), _ptr(ed), C, D, _ptr(lod), _ptr(hid),
             float(np.sum(np.log(hi - lo))), _ptr(xp), _ptr(lpri), _stream())
    llp = d(ll(xp.cpu().numpy()))
    lib.call("smx_rmh_accept", _ptr(xd), _ptr(lpd), _ptr(xp), _ptr(lpri), _ptr(llp), _ptr(ud), C, D, _ptr(acc),
             _stream())
    np.testing.assert_array_equal(acc.cpu().numpy().astype(bool), accr)
    np.testing.assert_allclose(xd.cpu().numpy(), xr, rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(lpd.cpu().numpy(), lpr, rtol=1e-15)


def test_rmh_samples_a_gaussian(lib):
    from schwarmax_gb300.mcmc import run_rmh
    mu = torch.tensor([0.3, -0.2, 0.5], dtype=torch.float64, device="cuda")
    s = torch.tensor([0.1, 0.2, 0.05], dtype=torch.float64, device="cuda")

    def loglike(th):
        return -0.5 * (((th - mu[None]) / s[None]) ** 2).sum(dim=1)

    r = run_rmh(None, [0.0, 0.0, 0.0], [-2, -2, -2], [2, 2, 2], n_chains=64, n_steps=1500,
                sigma_init=[0.05, 0.1, 0.03], adapt_every=50, adapt_after=150, loglike=loglike, seed=7)
    flat = r.chain[500:].reshape(-1, 3)
    np.testing.assert_allclose(flat.mean(0), mu.cpu().numpy(), atol=0.03)
    np.testing.assert_allclose(flat.std(0), s.cpu().numpy(), rtol=0.15)
    assert 0.1 < r.acceptance[500:].mean() < 0.7
    assert r.adapt_count > 0


def test_rmh_on_the_model_likelihood(lib):
    """Three steps of four chains on a small synthetic galaxy: every proposal batch is
    one batched model evaluation, and the chains' log densities are the model's."""
    from schwarmax_gb300 import synthetic
    from schwarmax_gb300.mcmc import log_likelihood_device, run_rmh
    cfg = synthetic.Config("mcmc-test", n_part=64, n_samples=40, n_pix=16, n_bins=8, n_grid=(6, 4, 4), n_boot=3,
                           n_periods=2.0, rtol=1e-5)
    dd, theta = synthetic.make_dataset(cfg, seed=11, precision="fp64")
    st = cfg.settings("fp64")
    lo, hi = theta - 0.5, theta + 0.5
    r = run_rmh(dd, theta, lo, hi, n_chains=4, n_steps=3, sigma_init=np.full(12, 0.01), init_sigma=np.full(12, 0.005),
                settings=st, nnls_maxiter=40, seed=3)
    assert r.chain.shape == (3, 4, 12)
    last = torch.as_tensor(r.chain[-1], device="cuda")
    ll = log_likelihood_device(last, dd, cfg.n_bins, int(np.prod(cfg.n_grid)), settings=st, nnls_maxiter=40)
    np.testing.assert_allclose(r.logprob[-1], ll.cpu().numpy() - np.sum(np.log(hi - lo)), rtol=1e-9)
