"""Device-resident batched MCMC: adaptive random-walk Metropolis-Hastings over the
batched likelihood (the sampler loop of example/example_schwarmax.ipynb cell 12,
BlackJAX's additive normal random walk with a uniform box prior).

Every step runs on the GPU: the proposals of all chains (``smx_rmh_propose``), one
batched evaluation of all proposals (``log_likelihoods_batch``: one integrator
launch over every chain's orbits), and the acceptance (``smx_rmh_accept``); chain
positions and log densities stay in device memory.  The host only adapts the
proposal covariance every ``adapt_every`` steps after ``adapt_after`` (as the
reference: covariance of the recent samples, 0.8 cov + 0.2 diag, scaled by
2.38^2 / ndim, Cholesky) and keeps the chain history.  Random draws come from a
seeded torch generator on the device (the reference uses jax.random keys).
"""
import math
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import call
from .kernels import _ptr, _stream
from .likelihood import log_likelihoods_batch


@dataclass
class RMHResult:
    chain: np.ndarray          # (n_steps, n_chains, ndim)
    logprob: np.ndarray        # (n_steps, n_chains)
    acceptance: np.ndarray     # (n_steps,) mean acceptance of each step
    adapt_count: int
    proposal_L: np.ndarray


def _lme(logl):
    m = torch.max(logl, dim=1, keepdim=True).values
    return m[:, 0] + torch.log(torch.mean(torch.exp(logl - m), dim=1))


def log_likelihood_device(thetas, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify=1.0, settings=None,
                          nnls_maxiter=200):
    """model_likelihood of every row of thetas (a (P, 12) device or host array), as a
    device tensor (P,)."""
    th = thetas.detach().cpu().numpy() if isinstance(thetas, torch.Tensor) else np.asarray(thetas)
    logl, _ = log_likelihoods_batch(th, dict_data, num_Vbin, Rzphi_n_tot, sigma_amplify, settings, nnls_maxiter)
    return _lme(logl)


def run_rmh(dict_data, theta0, bounds_lo, bounds_hi, n_chains=32, n_steps=1000, sigma_init=None, init_sigma=None,
            sigma_amplify=1.0, adapt_every=50, adapt_after=150, settings=None, nnls_maxiter=200, seed=42,
            loglike=None, callback=None):
    """Adaptive RMH with n_chains chains started at theta0 + N(0, init_sigma^2),
    clipped to the bounds.  loglike (optional) replaces the model likelihood: a
    function (P, ndim) device tensor -> (P,) device tensor (used by the tests).
    Returns RMHResult."""
    dev = torch.device("cuda")
    lo = torch.as_tensor(np.asarray(bounds_lo, dtype=np.float64), device=dev)
    hi = torch.as_tensor(np.asarray(bounds_hi, dtype=np.float64), device=dev)
    D = lo.numel()
    log_vol = float(torch.log(hi - lo).sum().item())
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    sigma_init = np.full(D, 0.02) if sigma_init is None else np.asarray(sigma_init, dtype=np.float64)
    init_sigma = sigma_init if init_sigma is None else np.asarray(init_sigma, dtype=np.float64)
    if loglike is None:
        nb = int(dict_data["total_bins"]) if "total_bins" in dict_data else len(dict_data["v0"])
        nc = int(dict_data["Rzphi_n_tot"])

        def loglike(th):
            return log_likelihood_device(th, dict_data, nb, nc, sigma_amplify, settings, nnls_maxiter)

    x = torch.as_tensor(np.asarray(theta0, dtype=np.float64), device=dev)[None].repeat(n_chains, 1)
    x = x + torch.randn(n_chains, D, generator=gen, device=dev, dtype=torch.float64) * \
        torch.as_tensor(init_sigma, device=dev)[None]
    x = torch.minimum(torch.maximum(x, lo[None]), hi[None]).contiguous()
    inb = ((x >= lo[None]) & (x <= hi[None])).all(dim=1)
    ll0 = loglike(x)
    lp = torch.where(inb, torch.full_like(ll0, -log_vol), torch.full_like(ll0, -math.inf)) + \
        torch.where(torch.isfinite(ll0), ll0, torch.full_like(ll0, -1e30))
    lp = lp.contiguous()
    L = torch.diag(torch.as_tensor(sigma_init, device=dev)).contiguous()
    opt_scale = 2.38 / math.sqrt(D)
    xp = torch.empty_like(x)
    logprior = torch.empty(n_chains, dtype=torch.float64, device=dev)
    accepted = torch.empty(n_chains, dtype=torch.int32, device=dev)
    chain, logprob, acc_hist = [], [], []
    adapt_count = 0
    for step in range(1, n_steps + 1):
        eps = torch.randn(n_chains, D, generator=gen, device=dev, dtype=torch.float64)
        u = torch.rand(n_chains, generator=gen, device=dev, dtype=torch.float64)
        call("smx_rmh_propose", _ptr(x), _ptr(L), _ptr(eps), n_chains, D, _ptr(lo), _ptr(hi), log_vol, _ptr(xp),
             _ptr(logprior), _stream())
        llp = loglike(xp).to(torch.float64).contiguous()
        call("smx_rmh_accept", _ptr(x), _ptr(lp), _ptr(xp), _ptr(logprior), _ptr(llp), _ptr(u), n_chains, D,
             _ptr(accepted), _stream())
        chain.append(x.clone())
        logprob.append(lp.clone())
        acc_hist.append(accepted.double().mean())
        if step >= adapt_after and step % adapt_every == 0:
            recent = torch.stack(chain[int(max(adapt_after - 50, step - 200)):]).reshape(-1, D)
            if recent.shape[0] > 2 * D:
                cov = torch.cov(recent.t())
                cov_reg = 0.8 * cov + 0.2 * torch.diag(torch.diagonal(cov))
                try:
                    L = torch.linalg.cholesky(opt_scale ** 2 * cov_reg).contiguous()
                    adapt_count += 1
                except RuntimeError:
                    pass
        if callback is not None:
            callback(step, x, lp)
    return RMHResult(chain=torch.stack(chain).cpu().numpy(), logprob=torch.stack(logprob).cpu().numpy(),
                     acceptance=torch.stack(acc_hist).cpu().numpy(), adapt_count=adapt_count, proposal_L=L.cpu().numpy())
