"""One random-walk Metropolis-Hastings step restated on the CPU (test
infrastructure): BlackJAX's additive random walk with a normal proposal
(x' = x + L eps) and the acceptance u < min(1, exp(lp' - lp)), with the uniform
box prior and the -1e30 replacement of non-finite log-likelihoods of the
reference's logdensity_fn (example/example_schwarmax.ipynb cell 12)."""
import numpy as np


def rmh_step(x, lp, L, eps, u, lo, hi, loglike):
    log_vol = np.sum(np.log(hi - lo))
    xp = x + eps @ L.T
    inb = np.all((xp >= lo) & (xp <= hi), axis=1)
    ll = loglike(xp)
    lpn = np.where(inb, -log_vol, -np.inf) + np.where(np.isfinite(ll), ll, -1e30)
    p = np.where(lpn - lp >= 0, 1.0, np.exp(np.minimum(lpn - lp, 0.0)))
    acc = u < p
    return np.where(acc[:, None], xp, x), np.where(acc, lpn, lp), acc
