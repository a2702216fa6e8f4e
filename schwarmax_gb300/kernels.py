"""Typed wrappers over the C ABI for device tensors.

Each function takes CUDA torch tensors, checks device, dtype, shape and
contiguity, and launches the matching ``smx_*`` entry point on the current
torch stream.  Nothing here computes on the host: a missing library or a CPU
tensor is an error.
"""
import ctypes

import torch

from . import _lib
from ._lib import (SmxBinning, SmxIntegrator, SmxMapsProblem, SmxNnlsProblem, SmxPoint, SmxPotential, call)

DTYPES = {torch.float32: _lib.SMX_FP32, torch.float64: _lib.SMX_FP64}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _check(t, name, dtype=None, shape=None):
    if t is None:
        return
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the library has no CPU path)")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")


def _prec(dtype):
    if dtype not in DTYPES:
        raise TypeError(f"unsupported dtype {dtype}")
    return DTYPES[dtype]


def potential_eval(pot: SmxPotential, x, y, z, want_phi=True, want_acc=True, want_rho=False):
    dt = x.dtype
    n = x.numel()
    for t, nm in ((x, "x"), (y, "y"), (z, "z")):
        _check(t, nm, dt, (n,))
    out = {}
    phi = torch.empty(n, dtype=dt, device=x.device) if want_phi else None
    acc = torch.empty(3, n, dtype=dt, device=x.device) if want_acc else None
    rho = torch.empty(n, dtype=dt, device=x.device) if want_rho else None
    call("smx_potential_eval", ctypes.byref(pot), _prec(dt), _ptr(x), _ptr(y), _ptr(z), n, _ptr(phi),
         _ptr(acc[0] if want_acc else None), _ptr(acc[1] if want_acc else None), _ptr(acc[2] if want_acc else None),
         _ptr(rho), _stream())
    if want_phi:
        out["phi"] = phi
    if want_acc:
        out["acc"] = acc
    if want_rho:
        out["rho"] = rho
    return out


def initial_conditions(pot, pos, normals, uniforms, n_real, n_periods, steps_per_period, extras=True):
    """pos (3, n), normals (3, n), uniforms (6, n, n_real) -> dict of device tensors."""
    dt = pos.dtype
    n = pos.shape[1]
    _check(pos, "pos", dt, (3, n))
    _check(normals, "normals", dt, (3, n))
    _check(uniforms, "uniforms", dt, (6, n, n_real))
    dev = pos.device
    w = torch.empty(6, n * n_real, dtype=dt, device=dev)
    tt = torch.empty(n * n_real, dtype=dt, device=dev)
    dt0 = torch.empty(n * n_real, dtype=dt, device=dev)
    w0n = torch.empty(6, n, dtype=dt, device=dev) if extras else None
    torb = torch.empty(n, dtype=dt, device=dev) if extras else None
    vc = torch.empty(n, dtype=dt, device=dev) if extras else None
    call("smx_initial_conditions", ctypes.byref(pot), _prec(dt), _ptr(pos), _ptr(normals), _ptr(uniforms), n,
         n_real, float(n_periods), float(steps_per_period), _ptr(w), _ptr(tt), _ptr(dt0), _ptr(w0n), _ptr(torb),
         _ptr(vc), _stream())
    return dict(w0=w, t_total=tt, dt_init=dt0, w0_new=w0n, t_orb=torb, vc=vc)


def density_target(pot, dtype, R_grid, z_grid, phi_grid, dR, dz, dphi, sample):
    n = R_grid.numel()
    for t, nm in ((R_grid, "R_grid"), (z_grid, "z_grid"), (phi_grid, "phi_grid")):
        _check(t, nm, torch.float64, (n,))
    _check(sample, "sample", torch.float64)
    out = torch.empty(n, dtype=dtype, device=R_grid.device)
    call("smx_density_target", ctypes.byref(pot), _prec(dtype), _ptr(R_grid), _ptr(z_grid), _ptr(phi_grid), n,
         float(dR), float(dz), float(dphi), _ptr(sample), int(sample.shape[0]), _ptr(out), _stream())
    return out


class IntegratorBuffers:
    """Sample store and per-orbit records for smx_integrate, reusable across calls."""

    def __init__(self, n_orb, slots, dtype, device):
        self.n_orb, self.slots, self.dtype = n_orb, slots, dtype
        self.samples = torch.empty(7, n_orb, slots, dtype=dtype, device=device)
        self.n_stored = torch.empty(n_orb, dtype=torch.int32, device=device)
        self.info = torch.empty(_lib.INFO_FIELDS, n_orb, dtype=dtype, device=device)
        self.status = torch.empty(n_orb, dtype=torch.int32, device=device)
        self.queue = torch.zeros(1, dtype=torch.int32, device=device)


def integrate(pot, cfg: SmxIntegrator, w0, dt_init, t_total, bufs: IntegratorBuffers):
    dt = w0.dtype
    n_orb = w0.shape[1]
    _check(w0, "w0", dt, (6, n_orb))
    _check(dt_init, "dt_init", dt, (n_orb,))
    _check(t_total, "t_total", dt, (n_orb,))
    if bufs.n_orb != n_orb or bufs.dtype != dt:
        raise ValueError("integrator buffers do not match the orbits")
    call("smx_integrate", ctypes.byref(pot), ctypes.byref(cfg), _prec(dt), _ptr(w0), _ptr(dt_init), _ptr(t_total),
         n_orb, bufs.slots, _ptr(bufs.samples), _ptr(bufs.n_stored), _ptr(bufs.info), _ptr(bufs.status),
         _ptr(bufs.queue), _stream())
    return bufs


def points_tensor(pots, omegas, device):
    """Device array of smx_point (potential + frame rate) for a batched call."""
    arr = (SmxPoint * len(pots))()
    for i, (p, om) in enumerate(zip(pots, omegas)):
        arr[i].pot = p
        arr[i].omega = float(om)
    raw = bytes(arr)
    t = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)
    return t


def integrate_batch(points, n_points, per_point, cfg: SmxIntegrator, w0, dt_init, t_total, bufs: IntegratorBuffers,
                    blocks_per_sm=0):
    """Orbits of n_points parameter points in one launch (smx_integrate_batch); points is
    the device array of points_tensor()."""
    dt = w0.dtype
    n_orb = w0.shape[1]
    if n_orb != n_points * per_point:
        raise ValueError("w0 must hold n_points * per_point orbits")
    _check(w0, "w0", dt, (6, n_orb))
    _check(dt_init, "dt_init", dt, (n_orb,))
    _check(t_total, "t_total", dt, (n_orb,))
    _check(points, "points", torch.uint8, (n_points * ctypes.sizeof(SmxPoint),))
    if bufs.n_orb != n_orb or bufs.dtype != dt:
        raise ValueError("integrator buffers do not match the orbits")
    call("smx_integrate_batch", _ptr(points), int(n_points), int(per_point), ctypes.byref(cfg), _prec(dt), _ptr(w0),
         _ptr(dt_init), _ptr(t_total), bufs.slots, _ptr(bufs.samples), _ptr(bufs.n_stored), _ptr(bufs.info),
         _ptr(bufs.status), _ptr(bufs.queue), int(blocks_per_sm), _stream())
    return bufs


def project_bin_batch(geo: SmxBinning, n_points, rots, bufs: IntegratorBuffers, t_total, bin_mapping, num_per_bin, v0,
                      s, library=None, valid=None):
    """smx_project_bin_batch: rots (n_points, 9) double; returns library (n_points, n_part, rows)."""
    dt = bufs.dtype
    rows = geo.nR * geo.nz * geo.nphi + 6 * geo.n_bins
    n_orb = n_points * geo.n_part * geo.n_real
    if n_orb != bufs.n_orb:
        raise ValueError("binning geometry does not match the integrated orbits")
    _check(rots, "rots", torch.float64, (n_points, 9))
    _check(t_total, "t_total", dt, (n_orb,))
    _check(bin_mapping, "bin_mapping", torch.int32, (geo.nX * geo.nY + 1,))
    for t, nm in ((num_per_bin, "num_per_bin"), (v0, "v0"), (s, "s")):
        _check(t, nm, torch.float64, (geo.n_bins,))
    dev = bufs.samples.device
    if library is None:
        library = torch.empty(n_points, geo.n_part, rows, dtype=dt, device=dev)
    _check(library, "library", dt, (n_points, geo.n_part, rows))
    if valid is not None:
        _check(valid, "valid", torch.int8, (n_orb,))
    call("smx_project_bin_batch", ctypes.byref(geo), int(n_points), _ptr(rots), _prec(dt), _ptr(bufs.samples),
         _ptr(bufs.n_stored), bufs.slots, _ptr(bufs.info), _ptr(t_total), _ptr(bin_mapping), _ptr(num_per_bin), _ptr(v0),
         _ptr(s), _ptr(library), _ptr(valid), _stream())
    return library


def project_bin(geo: SmxBinning, bufs: IntegratorBuffers, t_total, bin_mapping, num_per_bin, v0, s, library=None,
                valid=None):
    dt = bufs.dtype
    rows = geo.nR * geo.nz * geo.nphi + 6 * geo.n_bins
    n_orb = geo.n_part * geo.n_real
    if n_orb != bufs.n_orb:
        raise ValueError("binning geometry does not match the integrated orbits")
    _check(t_total, "t_total", dt, (n_orb,))
    _check(bin_mapping, "bin_mapping", torch.int32, (geo.nX * geo.nY + 1,))
    for t, nm in ((num_per_bin, "num_per_bin"), (v0, "v0"), (s, "s")):
        _check(t, nm, torch.float64, (geo.n_bins,))
    dev = bufs.samples.device
    if library is None:
        library = torch.empty(geo.n_part, rows, dtype=dt, device=dev)
    _check(library, "library", dt, (geo.n_part, rows))
    if valid is not None:
        _check(valid, "valid", torch.int8, (n_orb,))
    call("smx_project_bin", ctypes.byref(geo), _prec(dt), _ptr(bufs.samples), _ptr(bufs.n_stored), bufs.slots,
         _ptr(bufs.info), _ptr(t_total), _ptr(bin_mapping), _ptr(num_per_bin), _ptr(v0), _ptr(s), _ptr(library),
         _ptr(valid), _stream())
    return library


class Workspace:
    """Grow-only device scratch shared by calls on one stream."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes, device):
        if self.buf is None or self.buf.numel() < nbytes or self.buf.device != device:
            self.buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        return self.buf


_ws = Workspace()
_ws_maps = Workspace()


def nnls_admm(library, row_map, row_scale, Y, maxiter, lambda_reg, w_init, mixed):
    """library (n, ld) float/double; row_map (m,) int32; row_scale (m,) double;
    Y (B, m) double -> Z (B, n) double."""
    n, ld = library.shape
    m = row_map.numel()
    B = Y.shape[0]
    _check(library, "library", library.dtype, (n, ld))
    _check(row_map, "row_map", torch.int32, (m,))
    _check(row_scale, "row_scale", torch.float64, (m,))
    _check(Y, "Y", torch.float64, (B, m))
    prob = SmxNnlsProblem(n=n, m=m, n_rhs=B, ld_lib=ld, lib_precision=_prec(library.dtype),
                          mode=_lib.SMX_NNLS_MIXED if mixed else _lib.SMX_NNLS_FP64, maxiter=int(maxiter),
                          lambda_reg=float(lambda_reg), w_init=float(w_init))
    nbytes = ctypes.c_size_t(0)
    call("smx_nnls_workspace_size", ctypes.byref(prob), ctypes.byref(nbytes))
    ws = _ws.get(nbytes.value, library.device)
    Z = torch.empty(B, n, dtype=torch.float64, device=library.device)
    call("smx_nnls_admm", ctypes.byref(prob), _ptr(library), _ptr(row_map), _ptr(row_scale), _ptr(Y), _ptr(Z),
         _ptr(ws), ws.numel(), _stream())
    return Z


def nnls_jackknife(library, row_map, row_scale, y, drop_rows, maxiter, lambda_reg, w_init):
    """All leave-group-out replicates of the single right-hand-side NNLS in one batched
    mixed-precision solve (smx_nnls_jackknife).  y (m,) double scaled data row;
    drop_rows (G, max_drop) int32 design rows dropped by each replicate (-1 padding).
    Returns Z (G, n) double."""
    n, ld = library.shape
    m = row_map.numel()
    G, max_drop = drop_rows.shape
    _check(library, "library", library.dtype, (n, ld))
    _check(row_map, "row_map", torch.int32, (m,))
    _check(row_scale, "row_scale", torch.float64, (m,))
    _check(y, "y", torch.float64, (m,))
    _check(drop_rows, "drop_rows", torch.int32, (G, max_drop))
    prob = SmxNnlsProblem(n=n, m=m, n_rhs=G, ld_lib=ld, lib_precision=_prec(library.dtype), mode=_lib.SMX_NNLS_MIXED,
                          maxiter=int(maxiter), lambda_reg=float(lambda_reg), w_init=float(w_init))
    nbytes = ctypes.c_size_t(0)
    call("smx_nnls_jackknife_workspace_size", ctypes.byref(prob), int(max_drop), ctypes.byref(nbytes))
    ws = _ws.get(nbytes.value, library.device)
    Z = torch.empty(G, n, dtype=torch.float64, device=library.device)
    call("smx_nnls_jackknife", ctypes.byref(prob), _ptr(library), _ptr(row_map), _ptr(row_scale), _ptr(y),
         _ptr(drop_rows), int(max_drop), _ptr(Z), _ptr(ws), ws.numel(), _stream())
    return Z


def spd_inverse_f32(G):
    """FP32 inverse of a symmetric positive definite double CUDA matrix (smx_spd_inverse_f32)."""
    m = G.shape[0]
    _check(G, "G", torch.float64, (m, m))
    nbytes = ctypes.c_size_t(0)
    call("smx_spd_inverse_f32_workspace_size", m, ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=G.device)
    X = torch.empty(m, m, dtype=torch.float32, device=G.device)
    call("smx_spd_inverse_f32", _ptr(G), m, _ptr(X), _ptr(ws), ws.numel(), _stream())
    return X


def spd_inverse_seed(G):
    """Seed inverse of a symmetric positive definite double CUDA matrix by Schur-complement
    recursion on split products (smx_spd_inverse_seed); double, exactly symmetric."""
    m = G.shape[0]
    _check(G, "G", torch.float64, (m, m))
    nbytes = ctypes.c_size_t(0)
    call("smx_spd_inverse_seed_workspace_size", m, ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=G.device)
    X = torch.empty(m, m, dtype=torch.float64, device=G.device)
    call("smx_spd_inverse_seed", _ptr(G), m, _ptr(X), _ptr(ws), ws.numel(), _stream())
    return X


def split_gemm(A, B, a_slices=4, b_slices=4, lower=False):
    """C = A @ B for double CUDA tensors A (M, K), B (K, N) through the split
    (Ozaki) tensor-core product smx_split_gemm; returns C (M, N) double.
    lower: only the 128 x 128 tiles on and below the diagonal (M == N)."""
    M, K = A.shape
    K2, N = B.shape
    if K2 != K:
        raise ValueError("split_gemm: inner dimensions differ")
    At = A.t().contiguous()          # column-major A
    Bt = B.t().contiguous()          # column-major B
    _check(At, "A", torch.float64, (K, M))
    _check(Bt, "B", torch.float64, (N, K))
    nbytes = ctypes.c_size_t(0)
    call("smx_split_gemm_workspace_size", M, N, K, a_slices, b_slices, ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=A.device)
    Ct = torch.empty(N, M, dtype=torch.float64, device=A.device)
    call("smx_split_gemm", M, N, K, a_slices, b_slices, int(lower), _ptr(At), _ptr(Bt), _ptr(Ct), _ptr(ws), ws.numel(),
         _stream())
    return Ct.t()


def model_maps(library, n_cells, n_bins, W, gamma_kin, v0, s, y_rz, y_xy, y_xy_boot, y_h_boot, sig_h_raw,
               lum_factor, sigma_amplify=1.0, want_maps=True):
    n, ld = library.shape
    B = W.shape[0]
    _check(W, "W", torch.float64, (B, n))
    for t, nm, sh in ((gamma_kin, "gamma_kin", (n_bins,)), (v0, "v0", (n_bins,)), (s, "s", (n_bins,)),
                      (y_rz, "y_rz", (n_cells,)), (y_xy, "y_xy", (n_bins,)), (y_xy_boot, "y_xy_boot", (B, n_bins)),
                      (y_h_boot, "y_h_boot", (4, B, n_bins)), (sig_h_raw, "sig_h_raw", (4, n_bins))):
        _check(t, nm, torch.float64, sh)
    prob = SmxMapsProblem(n=n, n_rhs=B, ld_lib=ld, lib_precision=_prec(library.dtype), n_cells=n_cells,
                          n_bins=n_bins, lum_factor=float(lum_factor), sigma_amplify=float(sigma_amplify))
    nbytes = ctypes.c_size_t(0)
    call("smx_model_maps_workspace_size", ctypes.byref(prob), ctypes.byref(nbytes))
    ws = _ws_maps.get(nbytes.value, library.device)
    maps = torch.empty(B, n_cells + 7 * n_bins, dtype=torch.float64, device=library.device) if want_maps else None
    logl = torch.empty(B, dtype=torch.float64, device=library.device)
    call("smx_model_maps", ctypes.byref(prob), _ptr(library), _ptr(W), _ptr(gamma_kin), _ptr(v0), _ptr(s),
         _ptr(y_rz), _ptr(y_xy), _ptr(y_xy_boot), _ptr(y_h_boot), _ptr(sig_h_raw), _ptr(maps), _ptr(logl), _ptr(ws),
         ws.numel(), _stream())
    return maps, logl


def sample_cells(geo: SmxBinning, points, bin_mapping):
    """points (6, N) -> (cells (n_img, N), bins (n_img, N), vlos (n_img, N) km/s)."""
    dt = points.dtype
    N = points.shape[1]
    _check(points, "points", dt, (6, N))
    _check(bin_mapping, "bin_mapping", torch.int32, (geo.nX * geo.nY + 1,))
    n_img = 4 if geo.symmetry else 1
    cells = torch.empty(n_img, N, dtype=torch.int32, device=points.device)
    bins = torch.empty(n_img, N, dtype=torch.int32, device=points.device)
    vlos = torch.empty(n_img, N, dtype=dt, device=points.device)
    call("smx_sample_cells", ctypes.byref(geo), _prec(dt), _ptr(points), N, _ptr(bin_mapping), _ptr(cells),
         _ptr(bins), _ptr(vlos), _stream())
    return cells, bins, vlos
