"""Host-side helpers of utils.py: halo parameter transforms (514-569), the
rotation matrix (164-179) and the data loader (572-743)."""
import math
import pickle

import numpy as np

from .engine import rotation_matrix as makeRotationMatrix_deg

EPSILON = 1e-12


def makeRotationMatrix(alpha, beta, gamma):
    """utils.py:176-179, angles in degrees; X = R @ x."""
    return makeRotationMatrix_deg(alpha, beta, gamma)


def logM_logRs_to_logMenc_logc(logM_halo, logRs_halo, r_enc=10.0, Delta=200.0, rho_crit=277.54):
    M, Rs = 10.0 ** logM_halo, 10.0 ** logRs_halo
    x = r_enc / Rs
    M_enc = M * (math.log(1.0 + x) - x / (1.0 + x))
    R_vir = (3.0 * M / (4.0 * math.pi * Delta * rho_crit)) ** (1.0 / 3.0)
    return math.log10(M_enc), math.log10(R_vir / Rs)


def logMenc_logc_to_logM_logRs(logM_enc, log_c, r_enc=10.0, Delta=200.0, rho_crit=277.54):
    """Six Newton steps from logM_enc + 0.5 (utils.py:526-569)."""
    M_enc = 10.0 ** logM_enc
    c = 10.0 ** log_c
    coeff = 4.0 * math.pi * Delta * rho_crit / 3.0
    ln10 = math.log(10.0)
    logM = logM_enc + 0.5
    for _ in range(6):
        M = 10.0 ** logM
        Rs = (M / coeff) ** (1.0 / 3.0) / c
        x = r_enc / Rs
        f_nfw = math.log(1.0 + x) - x / (1.0 + x)
        df = (f_nfw - x * x / (3.0 * (1.0 + x) ** 2)) * M * ln10
        logM = logM - (M * f_nfw - M_enc) / df
    Rs = (10.0 ** logM / coeff) ** (1.0 / 3.0) / c
    return logM, math.log10(Rs)


def assign_regular_grid(positions, grid_min, grid_max, n_bins):
    """utils.py:10-42 in the dtype of `positions` (NumPy)."""
    pos = np.asarray(positions)
    dt = pos.dtype
    n = np.asarray(n_bins, dtype=np.int64)
    lo = np.asarray(grid_min, dtype=dt)
    span = (np.asarray(grid_max, dtype=dt) - lo).astype(dt)
    norm = ((pos - lo).astype(dt) / span).astype(dt)
    k = np.clip(np.floor((norm * n.astype(dt)).astype(dt)).astype(np.int64), 0, n - 1)
    flat = (k * np.concatenate([[1], np.cumprod(n[:-1])])).sum(-1)
    oob = np.any((norm >= 1.0) | (norm < 0.0), axis=-1)
    return np.where(oob, int(np.prod(n)), flat)


def _xexpx_logpdf(x, scale):
    return np.log(np.maximum(x, 1e-300)) - x / scale


def _expx_logpdf(x, scale):
    return -x / scale


def _sample_from_logP(x_grid, logP, N, u):
    """utils.py:488-509 with the uniforms given."""
    P = np.exp(logP - np.max(logP))
    P /= P.sum()
    return np.interp(u, np.cumsum(P), x_grid)


class _JaxArrayUnpickler(pickle.Unpickler):
    """Loads pickles holding jax arrays without JAX (they carry NumPy state)."""

    def find_class(self, module, name):
        if name == "_reconstruct_array":
            def rebuild(fun, args, state, aval=None):
                a = fun(*args)
                a.__setstate__(state)
                return a
            return rebuild
        return super().find_class(module, name)


def load_data_bootstrap(path, filename, N_BOOTSTRAP=100, n_samples=5_000, n_real=4):
    """utils.py:572-743 with NumPy generators in place of the threefry draws of
    keys 10086 and 10010 (R and z samples); the Gaussian bootstrap draws use
    default_rng(42) as the reference does.  Adds 'jeans_normals' and
    'jitter_uniforms' (seeded 42/109/2026 and 911) for the device path."""
    with open(path + filename, "rb") as f:
        b = _JaxArrayUnpickler(f).load()
    A = lambda k: np.asarray(b[k])  # noqa: E731
    sd = A("surface_density").astype(np.float64)
    rng = np.random.default_rng(42)
    nb = len(sd)
    N = {k: rng.normal(size=(N_BOOTSTRAP, nb)) for k in ("XY", "h1", "h2", "h3", "h4", "V", "sigma")}
    for v in N.values():
        v[0, :] = 0.0
    n_R, n_z, n_phi = 10, 6, 10
    edges = [np.linspace(0.0, 10.0, n_R + 1), np.linspace(-3.0, 3.0, n_z + 1), np.linspace(-np.pi, np.pi, n_phi + 1)]
    mids = [0.5 * (e[:-1] + e[1:]) for e in edges]
    M = np.stack([m.ravel() for m in np.meshgrid(*mids, indexing="ij")], -1)
    lim = np.array([[0.0, 10.0], [-3.0, 3.0], [-np.pi, np.pi]])
    order = np.argsort(assign_regular_grid(M, lim[:, 0], lim[:, 1], (n_R, n_z, n_phi)), kind="stable")
    M = M[order]
    from scipy.stats import qmc
    smp = qmc.Sobol(d=3, scramble=False).random_base2(m=10)
    xg = np.linspace(0.0, 12.0, 1000)
    R = _sample_from_logP(xg, _xexpx_logpdf(xg, 3), n_samples, np.random.default_rng(10086).random(n_samples))
    ph = np.random.default_rng(42).uniform(0, 2 * np.pi, size=n_samples)
    zg = np.linspace(0, 5, 1000)
    z = _sample_from_logP(zg, _expx_logpdf(zg, 1.2), n_samples, np.random.default_rng(10010).random(n_samples))
    w0 = np.stack([R * np.cos(ph), R * np.sin(ph), z], -1)
    Xg, Yg = A("X_regular_grid"), A("Y_regular_grid")
    d = dict(v0=A("v0"), s=A("s"), XY_density_data=sd, XY_density_data_err=0.01 * sd + EPSILON,
             V_data=A("V_mean"), V_data_err=A("V_mean_err"), sigma_data=A("V_sigma"), sigma_data_err=A("V_sigma_err"),
             num_per_bin=A("num_per_bin"), bin_mapping=A("bin_mapping"), total_bins=int(A("total_bins")),
             XY_standard_normal=N["XY"], V_standard_normal=N["V"], sigma_standard_normal=N["sigma"],
             R_grid=M[:, 0], z_grid=M[:, 1], phi_grid=M[:, 2], R_minmax=[0.0, 10.0], z_minmax=[-3.0, 3.0],
             phi_minmax=[-np.pi, np.pi], Rzphi_n_tot=n_R * n_z * n_phi, Rzphi_n_grid=np.array([n_R, n_z, n_phi]),
             dR=edges[0][1] - edges[0][0], dz=edges[1][1] - edges[1][0], dphi=edges[2][1] - edges[2][0],
             sample_for_integration=smp, X_regular_grid=Xg, Y_regular_grid=Yg,
             dX=np.unique(Xg)[1] - np.unique(Xg)[0], dY=np.unique(Yg)[1] - np.unique(Yg)[0],
             sample_for_integration_XY=smp, X_minmax=A("X_minmax"), Y_minmax=A("Y_minmax"), nX_nY=A("nX_nY"), w0=w0)
    for k in range(1, 5):
        d[f"h{k}_data"] = A(f"h{k}")
        d[f"h{k}_data_err"] = A(f"h{k}_err")
        d[f"h{k}_standard_normal"] = N[f"h{k}"]
    d["jeans_normals"] = np.stack([np.random.default_rng(s).standard_normal(n_samples) for s in (42, 109, 2026)])
    d["jitter_uniforms"] = np.random.default_rng(911).random((6, n_samples, n_real))
    return d
