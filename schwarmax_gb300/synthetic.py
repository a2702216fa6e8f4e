"""Seeded synthetic inputs for the benchmark configurations.

No public data set is involved.  A configuration is a potential, a synthetic
IFU (a square pixel map grouped into Voronoi apertures by the nearest of K
seeded generator pixels, sentinel -1 for the unused last entry), an (R, z, phi)
grid, initial positions from a double-exponential disc, and observables made
from a "truth" library with seeded Dirichlet orbit weights plus noise.  The
truth library is built by this package's own kernels from an independent set
of initial conditions, with GH moments taken about per-aperture (v0, s) that
are the truth model's own mean and dispersion.  Output follows the dict_data
schema of the reference loader (utils.py:688-741).
"""
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import engine, kernels
from .potentials import potential_struct
from .utils import logM_logRs_to_logMenc_logc

KMS_TO_KPCGYR = 1.0 / 0.9777922216807892
ARCSEC_KPC_AT_50MPC = 50e3 * math.pi / (180 * 3600)      # 0.2424 kpc per arcsec


@dataclass
class Config:
    name: str
    n_part: int
    n_samples: int
    n_pix: int
    n_bins: int
    n_grid: tuple
    n_boot: int
    mode: str = "sampled"
    rtol: float = 1e-6
    atol: float = 1e-7
    n_periods: float = 50.0
    n_real: int = 4
    bar_mass: float = 1e10
    omega_kms_kpc: float = 35.0
    bulge_mass: float = 5e9
    pixel_arcsec: float = 0.5
    admm_iters: int = 200

    def settings(self, precision="mixed"):
        return engine.Settings(n_real=self.n_real, mode=self.mode, n_samples=self.n_samples, rtol=self.rtol,
                               atol=self.atol, n_periods=self.n_periods, bulge_mass=self.bulge_mass,
                               precision=precision)


CONFIGS = {
    0: Config("config0", 2048, 500, 40, 120, (20, 16, 10), 100),
    1: Config("config1", 16384, 1000, 80, 400, (24, 16, 12), 100),
    # config 1's library per point, 64 parameter points per batch (points_for)
    2: Config("config2", 16384, 1000, 80, 400, (24, 16, 12), 100),
    4: Config("config4", 65536, 1000, 120, 1500, (32, 32, 16), 200, bar_mass=2e10, omega_kms_kpc=40.0),
    # config 1 over one circular period with 20 samples: the same orbit count and
    # per-attempt work on a short horizon, for profiler captures
    "small": Config("small", 16384, 20, 80, 400, (24, 16, 12), 100, n_periods=1.0),
}


def theta_for(cfg: Config):
    """12-D parameter vector (likelihood.py:105-165 convention)."""
    M200, c = 1e12, 10.0
    R_vir = (3 * M200 / (4 * math.pi * 200 * 277.54)) ** (1 / 3)
    logMenc, logc = logM_logRs_to_logMenc_logc(math.log10(M200), math.log10(R_vir / c))
    return np.array([logMenc, math.log10(5e10), math.log10(cfg.bar_mass), logc, math.log10(3.0), math.log10(0.3),
                     math.log10(4.0), math.radians(30.0), math.radians(60.0), math.radians(45.0), 0.0,
                     math.log10(cfg.omega_kms_kpc * KMS_TO_KPCGYR)])


def points_for(cfg: Config, n_points, seed=0):
    """Parameter points of the batched workload: the halo mass and concentration, the
    disc mass, scale length and height, the bar mass and half-length drawn uniformly
    within +-20% of the configuration's values, and Omega_p uniform in [25, 45]
    km/s/kpc; viewing angles and M/L as in theta_for.  Returns (n_points, 12)."""
    rng = np.random.default_rng(seed)
    base = theta_for(cfg)
    out = np.repeat(base[None], n_points, axis=0)
    for k in (0, 1, 2, 3, 4, 5, 6):          # log10 quantities: +-20% of the value
        out[:, k] = base[k] + np.log10(rng.uniform(0.8, 1.2, n_points))
    out[:, 11] = np.log10(rng.uniform(25.0, 45.0, n_points) * KMS_TO_KPCGYR)
    return out


def disc_positions(rng, n, Rd=2.5, zd=0.3):
    R = rng.gamma(2.0, Rd, n)          # surface density R exp(-R/Rd)
    ph = rng.uniform(0, 2 * math.pi, n)
    z = rng.exponential(zd, n) * rng.choice([-1.0, 1.0], n)
    return np.stack([R * np.cos(ph), R * np.sin(ph), z], -1)


def apertures(rng, n_pix, n_bins):
    pix = np.stack(np.meshgrid(np.arange(n_pix), np.arange(n_pix), indexing="xy"), -1).reshape(-1, 2)
    gen = pix[rng.choice(len(pix), n_bins, replace=False)]
    d2 = ((pix[:, None, :].astype(np.float64) - gen[None]) ** 2).sum(-1)
    bm = np.argmin(d2, 1)
    return np.concatenate([bm, [-1]]).astype(np.int32), np.bincount(bm, minlength=n_bins)


def rzphi_grid(n_grid, R_lim=(0.0, 10.0), z_lim=(-3.0, 3.0)):
    n_R, n_z, n_phi = n_grid
    edges = [np.linspace(R_lim[0], R_lim[1], n_R + 1), np.linspace(z_lim[0], z_lim[1], n_z + 1),
             np.linspace(-math.pi, math.pi, n_phi + 1)]
    mids = [0.5 * (e[:-1] + e[1:]) for e in edges]
    M = np.stack([m.ravel() for m in np.meshgrid(*mids, indexing="ij")], -1)
    # sort by the flat cell index (R fastest), as the loader does
    iR = np.clip(((M[:, 0] - R_lim[0]) / (R_lim[1] - R_lim[0]) * n_R).astype(int), 0, n_R - 1)
    iz = np.clip(((M[:, 1] - z_lim[0]) / (z_lim[1] - z_lim[0]) * n_z).astype(int), 0, n_z - 1)
    ip = np.clip(((M[:, 2] + math.pi) / (2 * math.pi) * n_phi).astype(int), 0, n_phi - 1)
    M = M[np.argsort(iR + n_R * (iz + n_z * ip), kind="stable")]
    return M, [e[1] - e[0] for e in edges]


def skeleton(cfg: Config, seed=0, n_part=None, geometry_seed=None):
    """dict_data without observables: geometry, grids, draws and positions.  The
    Voronoi apertures come from geometry_seed (default: seed), the particles and
    draws from seed, so that a truth library can share the data's apertures."""
    from scipy.stats import qmc
    rng = np.random.default_rng(seed)
    n = cfg.n_part if n_part is None else n_part
    half = cfg.n_pix * cfg.pixel_arcsec * ARCSEC_KPC_AT_50MPC / 2
    bm, npb = apertures(rng if geometry_seed is None else np.random.default_rng(geometry_seed), cfg.n_pix, cfg.n_bins)
    M, (dR, dz, dphi) = rzphi_grid(cfg.n_grid)
    d = dict(num_per_bin=npb, bin_mapping=bm, total_bins=cfg.n_bins,
             R_grid=M[:, 0], z_grid=M[:, 1], phi_grid=M[:, 2], R_minmax=[0.0, 10.0], z_minmax=[-3.0, 3.0],
             phi_minmax=[-math.pi, math.pi], Rzphi_n_tot=int(np.prod(cfg.n_grid)), Rzphi_n_grid=np.array(cfg.n_grid),
             dR=dR, dz=dz, dphi=dphi, sample_for_integration=qmc.Sobol(d=3, scramble=False).random_base2(m=10),
             X_minmax=np.array([-half, half]), Y_minmax=np.array([-half, half]),
             nX_nY=np.array([cfg.n_pix, cfg.n_pix]))
    d["w0"] = disc_positions(rng, n)
    d["jeans_normals"] = rng.standard_normal((3, n))
    d["jitter_uniforms"] = rng.random((6, n, cfg.n_real))
    nrm = np.random.default_rng(42)
    for k in ("XY", "h1", "h2", "h3", "h4"):
        a = nrm.normal(size=(cfg.n_boot, cfg.n_bins))
        a[0] = 0.0
        d[f"{k}_standard_normal"] = a
    return d


def _library(cfg, d, theta, v0, s, precision):
    from .likelihood import grid_of, unpack_params
    halo, bary = unpack_params(theta)
    st = cfg.settings(precision)
    d = dict(d, v0=v0, s=s)
    # placeholders so DeviceData can be formed before observables exist
    nb = cfg.n_bins
    for k in ("XY_density_data", "XY_density_data_err"):
        d.setdefault(k, np.ones(nb))
    for k in range(1, 5):
        d.setdefault(f"h{k}_data", np.zeros(nb))
        d.setdefault(f"h{k}_data_err", np.ones(nb))
    dd = engine.DeviceData(d, n_real=st.n_real)
    pot = potential_struct(bary, halo, st.bulge_mass)
    grid = grid_of(d)
    libd = engine.build_library(pot, bary, dd, grid, st)
    y_rz = kernels.density_target(pot, torch.float64, dd.R_grid, dd.z_grid, dd.phi_grid, dd.dR, dd.dz, dd.dphi,
                                  dd.sample)
    return libd["library"].double(), y_rz, bary


def make_dataset(cfg: Config, seed=0, precision="mixed", noise=True):
    """Returns (dict_data, theta) on the host (NumPy arrays)."""
    theta = theta_for(cfg)
    # independent initial conditions and draws on the data's own apertures
    truth = skeleton(cfg, seed + 1000, geometry_seed=seed)
    nb = cfg.n_bins
    nc = int(np.prod(cfg.n_grid))
    rng = np.random.default_rng(seed + 7)
    # pass 1: broad GH reference (v0 = 0, s = 2000 km/s) -> per-aperture mean and dispersion
    S = 2000.0
    lib, y_rz, bary = _library(cfg, truth, theta, np.zeros(nb), np.full(nb, S), precision)
    n = lib.shape[0]
    w = torch.as_tensor(rng.dirichlet(np.ones(n)) * n, device="cuda")
    mom = (w[None, :] @ lib[:, nc + nb:]).reshape(6 - 1, nb).cpu().numpy()   # h0..h4 rows
    h0, h1, h2 = mom[0], mom[1], mom[2]
    ok = h0 > 0
    my = np.where(ok, h1 / np.sqrt(2) / np.where(ok, h0, 1), 0.0)
    my2 = np.where(ok, (np.sqrt(2) * h2 + h0) / 2 / np.where(ok, h0, 1), 0.01)
    v0 = S * my
    s = S * np.sqrt(np.clip(my2 - my ** 2, 1e-4, None))
    s = np.clip(s, 20.0, 400.0)
    # pass 2: moments about (v0, s)
    lib, y_rz, bary = _library(cfg, truth, theta, v0, s, precision)
    cols = (w[None, :] @ lib).cpu().numpy()[0]
    l2m = 1.0 / float(bary["mass_to_light_ratio"])
    mmpo = float(y_rz.sum().item()) / n
    A_xy_w = cols[nc:nc + nb]
    hk = cols[nc + 2 * nb: nc + 6 * nb].reshape(4, nb)
    d = skeleton(cfg, seed)
    half = d["X_minmax"][1]
    area = (2 * half / cfg.n_pix) ** 2 * 1e6
    sd = A_xy_w * mmpo * l2m                                   # surface density in light units
    M_b = A_xy_w * d["num_per_bin"] * area
    h4 = np.zeros(nb)
    for _ in range(8):                                          # gamma_kin depends on h4
        gamma = M_b / ((1.0 + h4 * math.sqrt(6.0) / 4.0) * 2.0 * math.sqrt(math.pi) * s + 1e-12)
        h = hk / np.where(np.abs(gamma) > 1e-8, gamma, 1e-8)[None]
        h4 = h[3]
    h_err = np.stack([np.full(nb, 0.02), np.full(nb, 0.02), np.full(nb, 0.03), np.full(nb, 0.03)])
    if noise:
        sd = sd * (1.0 + 0.05 * rng.standard_normal(nb))
        h = h + h_err * rng.standard_normal(h.shape)
    sd = np.abs(sd) + 1e-6
    dv = math.sqrt(2.0) * h[0] + math.sqrt(3.0) * h[2]
    V = v0 + s * dv
    sig = s * np.sqrt(np.clip(1 + 2 * math.sqrt(2) * h[1] + 2 * math.sqrt(6) * h[3] - dv ** 2, 1e-10, None))
    d.update(v0=v0, s=s, XY_density_data=sd, XY_density_data_err=0.01 * sd + 1e-12, V_data=V,
             V_data_err=np.full(nb, 5.0), sigma_data=sig, sigma_data_err=np.full(nb, 5.0))
    for k in range(4):
        d[f"h{k + 1}_data"] = h[k]
        d[f"h{k + 1}_data_err"] = h_err[k]
    return d, theta
