"""Device-side pipeline of one model evaluation.

ICs (Jeans + V_c + T_orb + jitter) -> orbits -> projection/binning -> 3-D
target -> data scaling and gamma_kin -> bootstrap ADMM NNLS -> model maps and
chi^2.  Mirrors build_model (model.py:70-286) and the chi^2 of
model_likelihood (likelihood.py:192-244).  All arrays live on the GPU; the host
only forms small parameter structs and launches.

Random draws are inputs: dict_data may carry 'jeans_normals' (3, n) and
'jitter_uniforms' (6, n, n_real) in place of the reference's threefry keys
42/109/2026 and 911 (model.py:112-138).  When they are absent they are drawn
once from NumPy generators seeded with the same numbers.
"""
import math
from dataclasses import dataclass, replace

import numpy as np
import torch

from . import kernels
from ._lib import INFO_NATT, SMX_MODE_REFERENCE, SMX_MODE_SAMPLED, SmxBinning, SmxIntegrator

EPSILON = 1e-12
KPCGYR_TO_KMS = 0.9777922216807892


@dataclass
class Settings:
    """Integrator and precision settings.  Defaults are the reference's
    hard-coded values (model.py:127, 163-169)."""
    n_real: int = 4
    mode: str = "reference"          # "reference" (N_max attempts) or "sampled"
    n_attempts: int = 5000
    n_periods: float = 50.0
    steps_per_period: float = 100.0
    atol: float = 1e-7
    rtol: float = 1e-4
    dt_min: float = 1e-5
    dt_max: float = 0.3
    n_samples: int = 1000
    max_attempts: int = 1_000_000
    bulge_mass: float = None
    precision: str = "mixed"         # "mixed" (FP32 orbits, split tensor-core NNLS) or "fp64"
    order_probe: bool = False        # sampled mode: order the orbits by the cost of a one-period probe
    nnls: str = None                 # "mixed" / "fp64" NNLS independently of the orbits (None: follow precision)
    autotune: bool = False           # batched evaluations: tuned integrator launch (autotune.py, cached)
    bootstrap: str = "gaussian"      # "gaussian": the reference's perturbed data rows (likelihood.py:199-211);
                                     # "poisson": Poisson(1) weights of the apertures per resample (one solve each)
    bootstrap_seed: int = 0          # seed of the Poisson weights

    @property
    def dtype(self):
        return torch.float32 if self.precision == "mixed" else torch.float64

    @property
    def nnls_mixed(self):
        return (self.nnls or self.precision) == "mixed"

    @property
    def slots(self):
        return self.n_attempts if self.mode == "reference" else self.n_samples


def settings_from(settings=None, **kw):
    s = Settings() if settings is None else (replace(settings) if isinstance(settings, Settings) else Settings(**settings))
    return replace(s, **{k: v for k, v in kw.items() if v is not None})


def _np(x, dtype=np.float64):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy().astype(dtype)
    return np.asarray(x, dtype=dtype)


def default_draws(n, n_real):
    """Seeded stand-ins for the threefry draws of model.py:112-138."""
    normals = np.stack([np.random.default_rng(k).standard_normal(n) for k in (42, 109, 2026)])
    uniforms = np.random.default_rng(911).random((6, n, n_real))
    return normals, uniforms


class DeviceData:
    """dict_data (utils.py:688-741 schema) on the device."""

    def __init__(self, dict_data, device="cuda", n_real=4, pin=False):
        d = dict_data
        self.source = d

        def dev(x, dtype=torch.float64):
            if isinstance(x, torch.Tensor):    # host tensors (pinned when the caller pinned them)
                return x.to(device, non_blocking=True).to(dtype).contiguous()
            a = torch.as_tensor(_np(x, np.float64 if dtype == torch.float64 else np.int32))
            if pin:
                a = a.pin_memory()
            return a.to(device, dtype=dtype, non_blocking=pin).contiguous()

        w0 = d["w0"]
        self.n = int(w0.shape[0])
        if "jeans_normals" in d and "jitter_uniforms" in d:
            normals, uniforms = d["jeans_normals"], d["jitter_uniforms"]
        else:
            normals, uniforms = default_draws(self.n, max(n_real, 1))
        self.uniforms_traj = _np(d["jitter_uniforms_traj"]) if "jitter_uniforms_traj" in d else None
        self.pos64 = dev(w0).t().contiguous()
        self.normals64 = dev(normals)
        self.uniforms64 = dev(uniforms)
        self.bin_mapping = dev(d["bin_mapping"], torch.int32)
        self.num_per_bin = dev(d["num_per_bin"])
        self.v0 = dev(d["v0"])
        self.s = dev(d["s"])
        self.n_bins = int(self.v0.numel())
        self.R_grid, self.z_grid, self.phi_grid = dev(d["R_grid"]), dev(d["z_grid"]), dev(d["phi_grid"])
        self.dR, self.dz, self.dphi = float(_np(d["dR"])), float(_np(d["dz"])), float(_np(d["dphi"]))
        self.sample = dev(d["sample_for_integration"])
        self.xy = dev(d["XY_density_data"])
        self.xy_err = dev(d["XY_density_data_err"])
        self.h = torch.stack([dev(d[f"h{k}_data"]) for k in range(1, 5)])
        self.h_err = torch.stack([dev(d[f"h{k}_data_err"]) for k in range(1, 5)])
        self.N_xy = dev(d["XY_standard_normal"])
        self.N_h = torch.stack([dev(d[f"h{k}_standard_normal"]) for k in range(1, 5)])
        self.n_boot = int(self.N_xy.shape[0])
        X, Y, nXY = _np(d["X_minmax"]), _np(d["Y_minmax"]), _np(d["nX_nY"])
        self.area_pixel = ((X[1] - X[0]) / nXY[0]) * ((Y[1] - Y[0]) / nXY[1]) * 1e6
        self._cast = {}

    def cast(self, dtype, n_real):
        key = (dtype, n_real)
        if key not in self._cast:
            uni = self.uniforms64[:, :, :n_real]
            self._cast[key] = (self.pos64.to(dtype).contiguous(), self.normals64.to(dtype).contiguous(),
                               uni.to(dtype).contiguous())
        return self._cast[key]

    def traj_uniforms(self, dtype):
        if self.uniforms_traj is not None:
            return torch.as_tensor(self.uniforms_traj, dtype=dtype, device=self.pos64.device).contiguous()
        return self.uniforms64[:, :, :1].to(dtype).contiguous()


_device_cache = []


def device_data(dict_data, n_real=4, cache=True):
    if isinstance(dict_data, DeviceData):
        return dict_data
    if cache:
        for src, dd in _device_cache:
            if src is dict_data:
                return dd
    dd = DeviceData(dict_data, n_real=n_real)
    if cache:
        _device_cache.append((dict_data, dd))
        if len(_device_cache) > 4:
            _device_cache.pop(0)
    return dd


@dataclass
class Grid:
    n_rzphi: tuple
    rzphi_lim: np.ndarray
    xy_lim: np.ndarray
    n_xy: tuple

    @property
    def n_cells(self):
        return int(np.prod(self.n_rzphi))


_buffers = {}


def _integrator_buffers(n_orb, slots, dtype, role="main"):
    key = (role, n_orb, slots, dtype)
    b = _buffers.get(key)
    if b is None:
        for k in [k for k in _buffers if k[0] == role]:
            del _buffers[k]
        b = kernels.IntegratorBuffers(n_orb, slots, dtype, torch.device("cuda"))
        _buffers[key] = b
    return b


def probe_order(pot, cfg, ic, st: Settings):
    """Orbit order for the sampled integration, longest first: attempts of each
    orbit over one circular period (1/n_periods of its horizon).  The order
    changes which lanes share a warp, not any result."""
    frac = 1.0 / max(st.n_periods, 1.0)
    ns = max(1, int(round(st.n_samples * frac)))
    pcfg = SmxIntegrator(mode=SMX_MODE_SAMPLED, store_all=0, n_attempts=0, n_samples=ns,
                         max_attempts=max(1, int(st.max_attempts * frac)), atol=cfg.atol, rtol=cfg.rtol,
                         dt_min=cfg.dt_min, dt_max=cfg.dt_max, omega=cfg.omega)
    n_orb = ic["w0"].shape[1]
    pb = _integrator_buffers(n_orb, ns, st.dtype, role="probe")
    kernels.integrate(pot, pcfg, ic["w0"], ic["dt_init"], (ic["t_total"] * frac).contiguous(), pb)
    cost = pb.info[INFO_NATT]
    return torch.argsort(cost, descending=True).to(torch.int32).contiguous()


def build_library(pot, params_disk_rho, dd: DeviceData, grid: Grid, st: Settings, trajectory=False):
    """Returns dict(library (n, rows), ic, bufs, valid)."""
    dtype = st.dtype
    n_real = 1 if trajectory else st.n_real
    pos, normals, uni = dd.cast(dtype, st.n_real)
    if trajectory:
        uni = dd.traj_uniforms(dtype)
    ic = kernels.initial_conditions(pot, pos, normals, uni, n_real, st.n_periods, st.steps_per_period)
    mode = "reference" if trajectory else st.mode
    cfg = SmxIntegrator(mode=SMX_MODE_REFERENCE if mode == "reference" else SMX_MODE_SAMPLED,
                        store_all=1 if trajectory else 0, n_attempts=st.n_attempts, n_samples=st.n_samples,
                        max_attempts=st.max_attempts, atol=st.atol, rtol=st.rtol, dt_min=st.dt_min,
                        dt_max=st.dt_max, omega=-float(params_disk_rho["Omega_bar"]))
    slots = st.n_attempts if mode == "reference" else st.n_samples
    order = None
    if mode == "sampled" and st.order_probe:
        order = probe_order(pot, cfg, ic, st)
        cfg.order = order.data_ptr()
    bufs = _integrator_buffers(dd.n * n_real, slots, dtype)
    kernels.integrate(pot, cfg, ic["w0"], ic["dt_init"], ic["t_total"], bufs)
    geo = binning_geometry(params_disk_rho, grid, dd, n_real, symmetry=0 if trajectory else 1)
    valid = torch.empty(dd.n * n_real, dtype=torch.int8, device="cuda")
    lib = kernels.project_bin(geo, bufs, ic["t_total"], dd.bin_mapping, dd.num_per_bin, dd.v0, dd.s, valid=valid)
    return dict(library=lib, ic=ic, bufs=bufs, valid=valid, geo=geo)


def rotation_matrix(alpha_deg, beta_deg, gamma_deg):
    """makeRotationMatrix (utils.py:164-179): (Rz(g) Rx(b) Rz(a))^T, X = R @ x."""
    a, b, g = (math.radians(float(v)) for v in (alpha_deg, beta_deg, gamma_deg))

    def Rz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    def Rx(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])

    return (Rz(g) @ Rx(b) @ Rz(a)).T


def binning_geometry(params_disk_rho, grid: Grid, dd: DeviceData, n_real, symmetry=1):
    rot = rotation_matrix(params_disk_rho["alpha"], params_disk_rho["beta"], params_disk_rho["gamma"])
    lim = np.asarray(grid.rzphi_lim, dtype=np.float64)
    xl = np.asarray(grid.xy_lim, dtype=np.float64)
    nR, nz, nphi = (int(v) for v in grid.n_rzphi)
    nX, nY = (int(v) for v in grid.n_xy)
    g = SmxBinning(n_part=dd.n, n_real=n_real, nR=nR, nz=nz, nphi=nphi, R_lo=lim[0, 0], R_hi=lim[0, 1],
                   z_lo=lim[1, 0], z_hi=lim[1, 1], phi_lo=lim[2, 0], phi_hi=lim[2, 1], nX=nX, nY=nY,
                   X_lo=xl[0, 0], X_hi=xl[0, 1], Y_lo=xl[1, 0], Y_hi=xl[1, 1], n_bins=dd.n_bins, symmetry=symmetry)
    for i in range(9):
        g.rot[i] = float(rot.reshape(-1)[i])
    return g


_rowmaps = {}


def row_map(n_cells, nb):
    key = (n_cells, nb)
    if key not in _rowmaps:
        idx = [np.arange(n_cells), n_cells + np.arange(nb)]
        for k in range(1, 5):
            idx.append(n_cells + (1 + k) * nb + np.arange(nb))
        _rowmaps[key] = torch.as_tensor(np.concatenate(idx).astype(np.int32), device="cuda")
    return _rowmaps[key]


def data_terms(dd: DeviceData, params_disk_rho, y_rz_raw, n_orb):
    """Target normalisation, data scaling and gamma_kin (model.py:213-258)."""
    l2m = 1.0 / float(params_disk_rho["mass_to_light_ratio"])
    y_rz = y_rz_raw.to(torch.float64)
    sig_rz = 0.02 * y_rz + 1e-10
    y_xy = dd.xy / l2m
    sig_xy = (dd.xy_err + EPSILON) / l2m
    sh = dd.h_err + EPSILON
    mmpo = y_rz.sum() / n_orb
    y_xy, sig_xy, y_rz, sig_rz = y_xy / mmpo, sig_xy / mmpo, y_rz / mmpo, sig_rz / mmpo
    M_b = y_xy * dd.num_per_bin * dd.area_pixel
    normGH = 1.0 + dd.h[3] * math.sqrt(6.0) / 4.0
    gamma = M_b / (normGH * 2.0 * math.sqrt(math.pi) * dd.s + EPSILON)
    return dict(y_rz=y_rz, sig_rz=sig_rz, y_xy=y_xy, sig_xy=sig_xy, sh=sh, mmpo=mmpo, gamma=gamma, l2m=l2m)


def nnls_inputs(d, dd: DeviceData, n_cells, weights, boot=True, sig_xy=None, sig_h=None):
    """row_scale (m,) and scaled data Y (B, m) of nnls.py:19-33 / 107-140."""
    w_rz, w_xy, w_h = weights
    sig_xy = d["sig_xy"] if sig_xy is None else sig_xy
    sig_h = d["sh"] if sig_h is None else sig_h
    g = torch.where(d["gamma"].abs() > 1e-8, d["gamma"], torch.full_like(d["gamma"], 1e-8))
    rs = [w_rz / (d["sig_rz"] + 1e-8), w_xy / (sig_xy + 1e-8)]
    rs += [w_h / (g * (sig_h[k] + 1e-8)) for k in range(4)]
    row_scale = torch.cat(rs).contiguous()
    if boot:
        y_xy_b = d["y_xy"][None] + dd.N_xy * d["sig_xy"][None]
        y_h_b = dd.h[:, None, :] + dd.N_h * d["sh"][:, None, :]
    else:
        y_xy_b = d["y_xy"][None]
        y_h_b = dd.h[:, None, :]
    B = y_xy_b.shape[0]
    parts = [(w_rz * d["y_rz"] / (d["sig_rz"] + 1e-8))[None].expand(B, -1),
             w_xy * y_xy_b / (sig_xy + 1e-8)[None]]
    parts += [w_h * y_h_b[k] / (sig_h[k] + 1e-8)[None] for k in range(4)]
    Y = torch.cat(parts, dim=1).contiguous()
    return row_scale, Y


def likelihood_data(dd: DeviceData):
    """Raw bootstrap data of likelihood.py:199-211."""
    sxy = dd.xy_err + EPSILON
    sh = dd.h_err + EPSILON
    y_xy_b = (dd.xy[None] + dd.N_xy * sxy[None]).contiguous()
    y_h_b = (dd.h[:, None, :] + dd.N_h * sh[:, None, :]).contiguous()
    return y_xy_b, y_h_b, sh.contiguous()


def evaluate(pot, params_disk_rho, dd: DeviceData, grid: Grid, st: Settings, nnls_maxiter=200,
             regularization=1.0, weights=(math.sqrt(5.0), math.sqrt(5.0), 1.0), sigma_amplify=1.0,
             trajectory=False, want_maps=True):
    """One model evaluation on the device.  Returns a dict of device tensors."""
    libd = build_library(pot, params_disk_rho, dd, grid, st, trajectory=trajectory)
    r = solve_library(pot, params_disk_rho, dd, grid, st, libd["library"], nnls_maxiter, regularization, weights,
                      sigma_amplify, want_maps)
    r["lib"] = libd
    return r


def poisson_weights(n_boot, n_bins, seed=0):
    """Poisson(1) weight of every aperture in every resample, (n_boot, n_bins) double."""
    rng = np.random.default_rng(seed)
    return torch.as_tensor(rng.poisson(1.0, (n_boot, n_bins)).astype(np.float64), device="cuda")


def solve_library_poisson(d, dd: DeviceData, nc, lib, st: Settings, nnls_maxiter, regularization, weights,
                          sigma_amplify, w_init, lum):
    """The Poisson bootstrap: resample b weighs aperture g by k_bg ~ Poisson(1), so its
    design and data rows (xy, h1..h4 of g) are scaled by sqrt(k_bg) and it is solved on
    its own (the design differs per resample), against the unperturbed data; its chi^2
    weighs the aperture terms by k_bg (likelihood.py:214-226 with weights).  Returns
    (W (B, n), maps, logl (B,))."""
    nb = dd.n_bins
    B = dd.n_boot
    row_scale, Y0 = nnls_inputs(d, dd, nc, weights, boot=False)
    K = poisson_weights(B, nb, st.bootstrap_seed)
    rows_k = torch.cat([torch.ones(B, nc, dtype=torch.float64, device="cuda")] + [K] * 5, dim=1).sqrt()
    rm = row_map(nc, nb)
    W = torch.stack([kernels.nnls_admm(lib, rm, (row_scale * rows_k[b]).contiguous(),
                                       (Y0[0] * rows_k[b])[None].contiguous(), nnls_maxiter, regularization, w_init,
                                       mixed=st.nnls_mixed)[0] for b in range(B)])
    y_xy_b, y_h_b, sh_raw = likelihood_data(dd)
    maps, _ = kernels.model_maps(lib, nc, nb, W, d["gamma"].contiguous(), dd.v0, dd.s, d["y_rz"].contiguous(), dd.xy,
                                 y_xy_b, y_h_b, sh_raw, lum, sigma_amplify, want_maps=True)
    m = split_maps(maps, nc, nb)
    amp = sigma_amplify
    res = torch.nansum(((m["density_3d_model"] - d["y_rz"]) / (0.1 * d["y_rz"] * amp)) ** 2)
    res = res + (K * ((m["surface_density"] - dd.xy) / (0.1 * dd.xy * amp)) ** 2).nansum(dim=1)
    for k in range(4):
        res = res + (K * ((m[f"h{k + 1}"] - dd.h[k]) / (sh_raw[k] * amp)) ** 2).nansum(dim=1)
    return W, maps, -0.5 * res


def solve_library(pot, params_disk_rho, dd: DeviceData, grid: Grid, st: Settings, lib, nnls_maxiter=200,
                  regularization=1.0, weights=(math.sqrt(5.0), math.sqrt(5.0), 1.0), sigma_amplify=1.0,
                  want_maps=True):
    """3-D target, data scaling, bootstrap NNLS, maps and chi^2 of one library
    (model.py:192-272, likelihood.py:192-244)."""
    n = lib.shape[0]
    nc = grid.n_cells
    nb = dd.n_bins
    y_rz_raw = kernels.density_target(pot, st.dtype, dd.R_grid, dd.z_grid, dd.phi_grid, dd.dR, dd.dz, dd.dphi,
                                      dd.sample)
    d = data_terms(dd, params_disk_rho, y_rz_raw, n)
    if st.bootstrap == "poisson":
        host = torch.stack([d["y_rz"].sum() / n, d["mmpo"]]).cpu()
        W, maps, logl = solve_library_poisson(d, dd, nc, lib, st, nnls_maxiter, regularization, weights,
                                              sigma_amplify, float(host[0]), float(host[1]) * d["l2m"])
        return dict(data=d, W=W, maps=maps if want_maps else None, logl=logl, n_cells=nc, n_bins=nb)
    if st.bootstrap != "gaussian":
        raise ValueError(f"unknown bootstrap {st.bootstrap!r} (gaussian or poisson)")
    row_scale, Y = nnls_inputs(d, dd, nc, weights)
    # w = z = sum(y_Rzphi)/n at the start (nnls.py:122); read back with mmpo in one copy
    host = torch.stack([d["y_rz"].sum() / n, d["mmpo"]]).cpu()
    w_init, mmpo = float(host[0]), float(host[1])
    W = kernels.nnls_admm(lib, row_map(nc, nb), row_scale, Y, nnls_maxiter, regularization, w_init,
                          mixed=st.nnls_mixed)
    y_xy_b, y_h_b, sh_raw = likelihood_data(dd)
    maps, logl = kernels.model_maps(lib, nc, nb, W, d["gamma"].contiguous(), dd.v0, dd.s, d["y_rz"].contiguous(),
                                    dd.xy, y_xy_b, y_h_b, sh_raw, mmpo * d["l2m"], sigma_amplify,
                                    want_maps=want_maps)
    return dict(data=d, W=W, maps=maps, logl=logl, n_cells=nc, n_bins=nb)


MAX_POINTS_PER_LAUNCH = 32


def _batch_bytes_per_point(dd: DeviceData, st: Settings, grid: Grid):
    el = 4 if st.dtype == torch.float32 else 8
    pp = dd.n * st.n_real
    rows = grid.n_cells + 6 * dd.n_bins
    return pp * (7 * st.slots + 16) * el + dd.n * rows * el


def evaluate_batch(pots, barys, dd: DeviceData, grid: Grid, st: Settings, nnls_maxiter=200, regularization=1.0,
                   weights=(math.sqrt(5.0), math.sqrt(5.0), 1.0), sigma_amplify=1.0, max_points=None,
                   blocks_per_sm=0, want_maps=False, keep=False):
    """Model evaluations at P parameter points (jax.vmap(model_likelihood) of the
    reference's notebooks, example/example_schwarmax.ipynb cells 8 and 12).

    The initial conditions are set up per point; then ONE integrator launch runs
    the orbits of all points from one work queue (smx_integrate_batch), so the
    uneven step counts of every point's orbits even out across the SMs, and ONE
    projection launch bins them with each point's rotation (smx_project_bin_batch).
    The target, NNLS, maps and chi^2 follow per point.  Points are processed in
    chunks whose sample store fits the free device memory (max_points caps a chunk).
    Returns dict(logl (P, B) device tensor, W list, ...)."""
    P = len(pots)
    if P != len(barys) or P < 1:
        raise ValueError("evaluate_batch: one params_disk_rho per potential")
    if st.mode != "sampled" and st.mode != "reference":
        raise ValueError(f"unknown mode {st.mode}")
    dtype = st.dtype
    n_real = st.n_real
    pos, normals, uni = dd.cast(dtype, n_real)
    pp = dd.n * n_real
    free = torch.cuda.mem_get_info()[0]
    fit = max(1, int(0.6 * free // _batch_bytes_per_point(dd, st, grid)))
    # at most 32 points per integrator launch: at 16,384 particles x 4 realisations per
    # point a 64-point launch (4.2M orbits, 117 GB of samples) ran 35% slower per orbit
    # than 32-point launches, and 8- and 16-point launches 7% and 2% slower
    chunk = min(P, fit, max_points or MAX_POINTS_PER_LAUNCH, 1024)
    mode = SMX_MODE_REFERENCE if st.mode == "reference" else SMX_MODE_SAMPLED
    cfg = SmxIntegrator(mode=mode, store_all=0, n_attempts=st.n_attempts, n_samples=st.n_samples,
                        max_attempts=st.max_attempts, atol=st.atol, rtol=st.rtol, dt_min=st.dt_min,
                        dt_max=st.dt_max, omega=0.0)
    out = dict(logl=[], W=[], data=[], maps=[], chunk=chunk)
    for c0 in range(0, P, chunk):
        c1 = min(P, c0 + chunk)
        Pc = c1 - c0
        w0 = torch.empty(6, Pc * pp, dtype=dtype, device="cuda")
        tt = torch.empty(Pc * pp, dtype=dtype, device="cuda")
        dt0 = torch.empty(Pc * pp, dtype=dtype, device="cuda")
        for q in range(Pc):
            ic = kernels.initial_conditions(pots[c0 + q], pos, normals, uni, n_real, st.n_periods, st.steps_per_period,
                                            extras=False)
            sl = slice(q * pp, (q + 1) * pp)
            w0[:, sl] = ic["w0"]
            tt[sl] = ic["t_total"]
            dt0[sl] = ic["dt_init"]
        pts = kernels.points_tensor(pots[c0:c1], [-float(b["Omega_bar"]) for b in barys[c0:c1]], w0.device)
        bps, order = blocks_per_sm, None
        if st.autotune and mode == SMX_MODE_SAMPLED:
            from . import autotune
            tuned = autotune.lookup(Pc * pp, st.n_samples, st.rtol) or \
                autotune.tune_integrator(pts, Pc, pp, w0, dt0, tt, st)
            bps = tuned["blocks_per_sm"]
            if tuned["order"] == "cost":
                order = autotune.cost_order(pts, Pc, pp, w0, dt0, tt, st)
        cfg.order = 0 if order is None else order.data_ptr()
        bufs = _integrator_buffers(Pc * pp, st.slots, dtype, role="batch")
        kernels.integrate_batch(pts, Pc, pp, cfg, w0, dt0, tt, bufs, bps)
        geo = binning_geometry(barys[c0], grid, dd, n_real)
        rots = torch.as_tensor(np.stack([rotation_matrix(b["alpha"], b["beta"], b["gamma"]).reshape(-1)
                                         for b in barys[c0:c1]]), dtype=torch.float64, device="cuda").contiguous()
        lib = kernels.project_bin_batch(geo, Pc, rots, bufs, tt, dd.bin_mapping, dd.num_per_bin, dd.v0, dd.s)
        for q in range(Pc):
            r = solve_library(pots[c0 + q], barys[c0 + q], dd, grid, st, lib[q], nnls_maxiter, regularization, weights,
                              sigma_amplify, want_maps)
            out["logl"].append(r["logl"])
            if keep:
                out["W"].append(r["W"])
                out["data"].append(r["data"])
                out["maps"].append(r["maps"])
        if keep:
            out.setdefault("libraries", []).append(lib)
            out.setdefault("bufs", bufs)
    out["logl"] = torch.stack(out["logl"])
    return out


def split_maps(maps, nc, nb):
    o = dict(density_3d_model=maps[:, :nc], surface_density=maps[:, nc:nc + nb])
    for k in range(4):
        o[f"h{k + 1}"] = maps[:, nc + (1 + k) * nb: nc + (2 + k) * nb]
    o["V"] = maps[:, nc + 5 * nb: nc + 6 * nb]
    o["sigma"] = maps[:, nc + 6 * nb: nc + 7 * nb]
    return o
