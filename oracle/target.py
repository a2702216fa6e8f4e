"""3-D density target (model.py:192-213) and the Rzphi grid of the loader
(utils.py:627-659).

y[c] = dR dz dphi * mean_j rho(R_j cos phi_j, R_j sin phi_j, z_j) R_j with
R_j = R_c + (s_j0 - 1/2) dR (likewise z, phi) over the 1024 unscrambled Sobol
points s_j; cells are ordered by their flattened index (R fastest).
"""
import numpy as np

from . import grid
from . import potential as pot


def rzphi_grid(n_R, n_z, n_phi, R_lim=(0.0, 10.0), z_lim=(-3.0, 3.0), phi_lim=(-np.pi, np.pi)):
    """Returns dict(R_grid, z_grid, phi_grid, dR, dz, dphi, lim, n) with cells
    sorted by the assign_regular_grid flat index."""
    Re = np.linspace(R_lim[0], R_lim[1], n_R + 1)
    ze = np.linspace(z_lim[0], z_lim[1], n_z + 1)
    pe = np.linspace(phi_lim[0], phi_lim[1], n_phi + 1)
    Rm, zm, pm = 0.5 * (Re[:-1] + Re[1:]), 0.5 * (ze[:-1] + ze[1:]), 0.5 * (pe[:-1] + pe[1:])
    RR, ZZ, PP = np.meshgrid(Rm, zm, pm, indexing="ij")
    mids = np.stack([RR.ravel(), ZZ.ravel(), PP.ravel()], -1)
    lim = np.array([R_lim, z_lim, phi_lim], dtype=np.float64)
    idx = grid.assign_regular_grid(mids, lim[:, 0], lim[:, 1], (n_R, n_z, n_phi))
    order = np.argsort(idx, kind="stable")
    mids = mids[order]
    return dict(R_grid=mids[:, 0], z_grid=mids[:, 1], phi_grid=mids[:, 2],
                dR=Re[1] - Re[0], dz=ze[1] - ze[0], dphi=pe[1] - pe[0], lim=lim,
                n=np.array([n_R, n_z, n_phi]))


def sobol_1024():
    from scipy.stats import qmc
    return qmc.Sobol(d=3, scramble=False).random_base2(m=10)


def density_target(R_grid, z_grid, phi_grid, dR, dz, dphi, sample, P):
    R = R_grid[:, None] + (sample[None, :, 0] - 0.5) * dR
    z = z_grid[:, None] + (sample[None, :, 1] - 0.5) * dz
    ph = phi_grid[:, None] + (sample[None, :, 2] - 0.5) * dphi
    rho = pot.rho(R * np.cos(ph), R * np.sin(ph), z, P)
    return (rho * R).sum(1) / sample.shape[0] * dR * dz * dphi
