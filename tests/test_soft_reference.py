"""The dense reference of the differentiable projection (oracle/soft_projection.py)
on the CPU: its autograd gradient against central finite differences, the soft
weights against the hard binning in the limit of a narrow kernel, and conservation
of the sample weight when the whole window lies on the grid."""
import math

import numpy as np
import torch

from oracle import soft_projection as sp


def _case(seed=0, n_part=6, n_real=2, slots=40, nX=12, nY=10, nb=7):
    rng = np.random.default_rng(seed)
    n_orb = n_part * n_real
    samples = np.zeros((7, n_orb, slots))
    samples[:3] = rng.normal(0, 0.6, (3, n_orb, slots))
    samples[3:6] = rng.normal(0, 120.0, (3, n_orb, slots))
    samples[6] = rng.uniform(0.5, 1.5, (n_orb, slots))
    n_stored = rng.integers(slots // 2, slots + 1, n_orb)
    info = np.zeros((6, n_orb))
    info[0] = 10.0
    info[1] = -1.0
    info[2] = -1.0 + rng.uniform(-0.05, 0.05, n_orb)
    info[3] = samples[6].sum(1)
    t_total = np.full(n_orb, 10.0)
    bm = rng.integers(-1, nb, nX * nY + 1).astype(np.int32)
    bm[-1] = -1
    geo = dict(xlo=-1.5, ylo=-1.2, dx=3.0 / nX, dy=2.4 / nY, nX=nX, nY=nY, n_bins=nb, n_part=n_part, n_real=n_real,
               bin_mapping=torch.tensor(bm), num_per_bin=torch.tensor(np.bincount(bm[bm >= 0], minlength=nb) + 1.0),
               v0=torch.tensor(rng.normal(0, 20, nb)), s=torch.tensor(rng.uniform(80, 140, nb)), area=1.0)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    return t(samples), torch.tensor(n_stored), t(info), t(t_total), geo


def test_reference_gradient_matches_finite_differences():
    samples, n_stored, info, t_total, geo = _case()
    rng = np.random.default_rng(1)
    C = torch.tensor(rng.normal(size=(geo["n_part"], 6 * geo["n_bins"])))
    theta = torch.tensor([0.4, 1.0, 0.7, 1.05], dtype=torch.float64, requires_grad=True)
    L = (C * sp.soft_sky_rows(samples, n_stored, info, t_total, geo, theta, 0.5)).sum()
    (g,) = torch.autograd.grad(L, theta)
    fd = []
    for t in range(4):
        e = torch.zeros(4, dtype=torch.float64)
        e[t] = 1e-6
        f = lambda th: float((C * sp.soft_sky_rows(samples, n_stored, info, t_total, geo, th, 0.5)).sum())
        fd.append((f(theta.detach() + e) - f(theta.detach() - e)) / 2e-6)
    np.testing.assert_allclose(g.numpy(), np.array(fd), rtol=1e-6, atol=1e-8 * np.abs(fd).max())


def test_narrow_kernel_weight_is_conserved_inside_the_grid():
    samples, n_stored, info, t_total, geo = _case(seed=2)
    geo = dict(geo, bin_mapping=torch.zeros(geo["nX"] * geo["nY"] + 1, dtype=torch.int32))   # one bin everywhere
    geo["bin_mapping"][-1] = -1
    samples[:3] *= 0.05                      # every image well inside the grid
    theta = torch.tensor([0.3, 0.9, 0.2, 1.0], dtype=torch.float64)
    rows = sp.soft_sky_rows(samples, n_stored, info, t_total, geo, theta, 0.3)
    # the xy row of bin 0 holds the per-orbit weight sum: every image deposits all of its weight
    sc = sp.realisation_scales(info, t_total, geo["n_part"], geo["n_real"])
    j = torch.arange(samples.shape[2])
    keep = j[None, :] < n_stored[:, None]
    per_orb = (samples[6] * keep).sum(1) * sc * 4.0
    expect = per_orb.reshape(geo["n_part"], geo["n_real"]).sum(1) / (geo["num_per_bin"][0] * geo["area"] + 1e-12)
    np.testing.assert_allclose(rows[:, 0].numpy(), expect.numpy(), rtol=1e-9)


def test_rotation_matches_the_engine_convention():
    from schwarmax_gb300.engine import rotation_matrix
    th = torch.tensor([0.4, 1.1, -0.3], dtype=torch.float64)
    R = sp.rotation(th).numpy()
    np.testing.assert_allclose(R, rotation_matrix(*(math.degrees(float(v)) for v in th)), rtol=1e-14, atol=1e-15)
