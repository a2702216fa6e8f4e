"""Kernel-vs-oracle parity on the GPU, through the C ABI (schwarmax_gb300.kernels)."""
import math

import numpy as np
import pytest

from conftest import golden, params_from_flat
from oracle import grid as ogrid
from oracle import integrate as ointeg
from oracle import jeans as ojeans
from oracle import nnls as onnls
from oracle import model as omodel
from oracle import orbits as oorbits
from oracle import potential as opot
from oracle import target as otarget

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def K():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import kernels
    return kernels


def _params(scale=1.0):
    pb = dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3 * scale, logM_bar=10.0, L_bar=4.0 * scale,
              a_bar=0.8 * scale, b_bar=0.3 * scale, x_origin=0.0, y_origin=0.0, z_origin=0.0,
              dirx=0.0, diry=0.0, dirz=1.0)
    ph = dict(logM=12.0, Rs=20.6, a=1.0, b=1.0, c=1.0)
    return pb, ph


def _structs(pb, ph, bulge_mass=None):
    from schwarmax_gb300.potentials import potential_struct
    return potential_struct(pb, ph, bulge_mass), opot.canonical_params(pb, ph, bulge_mass)


def _cuda(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("scale,bulge", [(1.0, None), (1.3, 5e9)])
def test_potential_force_density_fp64(K, scale, bulge):
    rng = np.random.default_rng(10)
    pb, ph = _params(scale)
    S, P = _structs(pb, ph, bulge)
    x, y, z = rng.uniform(-14, 14, 4096), rng.uniform(-14, 14, 4096), rng.uniform(-4, 4, 4096)
    x[:3], y[:3], z[:3] = [-9.0, 0.01, 30.0], [0.0, -0.02, 1.0], [0.0, 0.0, -5.0]
    out = K.potential_eval(S, _cuda(x, torch.float64), _cuda(y, torch.float64), _cuda(z, torch.float64),
                           want_rho=True)
    phi, ax, ay, az = opot.phi_acc(x, y, z, P)
    np.testing.assert_allclose(out["phi"].cpu().numpy(), phi, rtol=1e-12)
    a = np.stack([ax, ay, az])
    amax = np.abs(a).max(0)
    np.testing.assert_allclose(out["acc"].cpu().numpy() / amax, a / amax, rtol=0, atol=2e-10)
    np.testing.assert_allclose(out["rho"].cpu().numpy(), opot.rho(x, y, z, P), rtol=1e-10)


def test_potential_matches_reference_golden_fp64(K):
    g = golden("potential")
    for tag in ("a", "b"):
        pb, ph = params_from_flat(g[f"{tag}_params"])
        S, _ = _structs(pb, ph)
        x, y, z = (_cuda(g[f"{tag}_{c}"], torch.float64) for c in "xyz")
        out = K.potential_eval(S, x, y, z, want_rho=True)
        np.testing.assert_allclose(out["phi"].cpu().numpy(), g[f"{tag}_phi"], rtol=1e-12)
        np.testing.assert_allclose(out["rho"].cpu().numpy(), g[f"{tag}_rho"], rtol=1e-10)
        ref = g[f"{tag}_acc"].T
        amax = np.abs(ref).max(0)
        np.testing.assert_allclose(out["acc"].cpu().numpy() / amax, ref / amax, rtol=0, atol=1e-10)


def test_potential_force_density_fp32(K):
    """FP32 error against the FP64 oracle: Phi 2e-6, forces 5e-5 of |a| (median 2e-6),
    rho 1e-3 at most (median 1e-6)."""
    rng = np.random.default_rng(11)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    x, y, z = rng.uniform(-14, 14, 8192), rng.uniform(-14, 14, 8192), rng.uniform(-4, 4, 8192)
    out = K.potential_eval(S, _cuda(x, torch.float32), _cuda(y, torch.float32), _cuda(z, torch.float32),
                           want_rho=True)
    xf, yf, zf = (np.float32(v).astype(np.float64) for v in (x, y, z))
    phi, ax, ay, az = opot.phi_acc(xf, yf, zf, P)
    np.testing.assert_allclose(out["phi"].cpu().double().numpy(), phi, rtol=2e-6)
    a = np.stack([ax, ay, az])
    amag = np.sqrt((a ** 2).sum(0))
    err = np.abs(out["acc"].cpu().double().numpy() - a).max(0) / amag
    assert err.max() < 5e-5 and np.median(err) < 2e-6, (err.max(), np.median(err))
    # rho: the T3 needle's second difference C(x+L) + C(x-L) - 2C(x) cancels in FP32 away
    # from the bar (the reference's FP32 path evaluates the same expression)
    rr = opot.rho(xf, yf, zf, P)
    rel = np.abs(out["rho"].cpu().double().numpy() - rr) / rr
    assert rel.max() < 1e-3 and np.median(rel) < 1e-6 and np.mean(rel > 2e-5) < 0.02, (rel.max(), np.median(rel))


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 3e-3)])
def test_initial_conditions(K, dtype, tol):
    rng = np.random.default_rng(12)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    n, n_real = 64, 4
    R = 6 * np.sqrt(rng.uniform(0.01, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([R * np.cos(th), R * np.sin(th), rng.exponential(0.3, n)])
    normals = rng.standard_normal((3, n))
    unif = rng.random((6, n, n_real))
    out = K.initial_conditions(S, _cuda(pos, dtype), _cuda(normals, dtype), _cuda(unif, dtype), n_real, 50, 100)
    w0n = ojeans.w0_new(pos.T, normals, P)
    Rn = np.sqrt(w0n[:, 0] ** 2 + w0n[:, 1] ** 2)
    Vc = oorbits.rotation_curve(Rn, w0n[:, 2], P)
    To = oorbits.orbital_timescale(Rn, w0n[:, 2], P)
    wb = oorbits.jitter(w0n, Vc, unif).reshape(-1, 6)
    got = out["w0_new"].cpu().double().numpy().T
    scale = np.abs(w0n).max(0)
    assert np.abs(got - w0n).max(0).max() / scale.min() < tol * 10 or np.all(np.abs(got - w0n) <= tol * scale)
    np.testing.assert_allclose(out["vc"].cpu().double().numpy(), Vc, rtol=tol)
    np.testing.assert_allclose(out["t_orb"].cpu().double().numpy(), To, rtol=tol)
    np.testing.assert_allclose(out["t_total"].cpu().double().numpy(), np.repeat(To, n_real) * 50, rtol=tol)
    np.testing.assert_allclose(out["dt_init"].cpu().double().numpy(), np.repeat(To, n_real) / 100, rtol=tol)
    np.testing.assert_allclose(out["w0"].cpu().double().numpy().T, wb, rtol=0, atol=tol * scale.max())


def test_initial_conditions_golden_fp64(K):
    g = golden("jeans")
    pb, ph = params_from_flat(g["params"])
    S, _ = _structs(pb, ph)
    n = g["w0"].shape[0]
    out = K.initial_conditions(S, _cuda(g["w0"].T, torch.float64), _cuda(g["normals"], torch.float64),
                               _cuda(np.full((6, n, 1), 0.5), torch.float64), 1, 50, 100)
    np.testing.assert_allclose(out["w0_new"].cpu().numpy().T, g["w0_new"], rtol=1e-8, atol=1e-9)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 1e-5)])
def test_density_target(K, dtype, tol):
    pb, ph = _params()
    S, P = _structs(pb, ph)
    gr = otarget.rzphi_grid(6, 4, 8)
    smp = otarget.sobol_1024()
    ref = otarget.density_target(gr["R_grid"], gr["z_grid"], gr["phi_grid"], gr["dR"], gr["dz"], gr["dphi"], smp, P)
    got = K.density_target(S, dtype, _cuda(gr["R_grid"], torch.float64), _cuda(gr["z_grid"], torch.float64),
                           _cuda(gr["phi_grid"], torch.float64), gr["dR"], gr["dz"], gr["dphi"],
                           _cuda(smp, torch.float64))
    np.testing.assert_allclose(got.cpu().double().numpy(), ref, rtol=tol)


def _orbit_states(rng, n, P):
    R = rng.uniform(0.8, 8.0, n)
    th = rng.uniform(0, 2 * np.pi, n)
    z = rng.normal(0, 0.3, n)
    vc = oorbits.rotation_curve(R, z, P)
    ecc = rng.uniform(0.6, 1.0, n)
    w = np.stack([R * np.cos(th), R * np.sin(th), z, vc * ecc * np.sin(th), -vc * ecc * np.cos(th),
                  rng.normal(0, 20, n)], -1)
    To = oorbits.orbital_timescale(R, z, P)
    return w, To


def _integ_cfg(mode, n_attempts=300, n_samples=0, omega=-35.79, store_all=0, rtol=1e-4):
    from schwarmax_gb300._lib import SmxIntegrator
    return SmxIntegrator(mode=mode, store_all=store_all, n_attempts=n_attempts, n_samples=n_samples,
                         max_attempts=200000, atol=1e-7, rtol=rtol, dt_min=1e-5, dt_max=0.3, omega=omega)


def test_integrate_reference_fp64_matches_oracle(K):
    rng = np.random.default_rng(13)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    n, N = 48, 300
    w, To = _orbit_states(rng, n, P)
    dt0 = To / 100
    om = -35.79
    bufs = K.IntegratorBuffers(n, N, torch.float64, torch.device("cuda"))
    K.integrate(S, _integ_cfg(0, N, omega=om), _cuda(w.T, torch.float64), _cuda(dt0, torch.float64),
                _cuda(To * 50, torch.float64), bufs)
    ref = ointeg.integrate_reference(w, P, om, N, dt0, 1e-7, 1e-4, 1e-5, 0.3, store=True)
    nst = bufs.n_stored.cpu().numpy()
    np.testing.assert_array_equal(nst, ref["n_acc"])
    info = bufs.info.cpu().numpy()
    np.testing.assert_allclose(info[0], ref["t_final"], rtol=1e-10)
    np.testing.assert_allclose(info[1], ref["EJ0"], rtol=1e-12)
    np.testing.assert_allclose(info[2], ref["EJ_final"], rtol=1e-9)
    samples = bufs.samples.cpu().numpy()
    for o in range(n):
        acc = ref["dts"][:, o] > 0
        ys = ref["ys"][acc, o]
        np.testing.assert_allclose(samples[:6, o, :nst[o]].T, ys, rtol=1e-8, atol=1e-9)
        np.testing.assert_allclose(samples[6, o, :nst[o]], ref["dts"][acc, o], rtol=1e-9)
    assert (bufs.status.cpu().numpy() == 0).all()


def test_integrate_reference_fp32_error(K):
    """FP32 orbits against FP64: short-horizon end states, E_J drift, step counts."""
    rng = np.random.default_rng(14)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    n, N = 256, 200
    w, To = _orbit_states(rng, n, P)
    w = w.astype(np.float32).astype(np.float64)
    dt0 = (To / 100).astype(np.float32).astype(np.float64)
    om = -35.79
    bufs = K.IntegratorBuffers(n, N, torch.float32, torch.device("cuda"))
    K.integrate(S, _integ_cfg(0, N, omega=om), _cuda(w.T, torch.float32), _cuda(dt0, torch.float32),
                _cuda(To * 50, torch.float32), bufs)
    ref = ointeg.integrate_reference(w, P, om, N, dt0, 1e-7, 1e-4, 1e-5, 0.3)
    info = bufs.info.cpu().double().numpy()
    nacc = bufs.n_stored.cpu().numpy()
    same = nacc == ref["n_acc"]
    assert same.mean() > 0.8
    yk = bufs.samples[:6, :, :].cpu().double().numpy()
    end = np.stack([yk[:, o, nacc[o] - 1] for o in range(n)])
    scale = np.abs(ref["y_final"]).max(1, keepdims=True)
    err = (np.abs(end - ref["y_final"]) / scale).max(1)[same]
    assert np.median(err) < 1e-4 and err.max() < 1e-2, (np.median(err), err.max())
    drift = np.abs(info[2] / info[1] - 1)
    assert np.median(drift) < 1e-4


def test_integrate_trajectory_store_all_fp64(K):
    g = golden("withtraj")
    pb, ph = params_from_flat(g["params"])
    S, P = _structs(pb, ph)
    w0 = g["w0"].reshape(-1, 6)
    n, N = w0.shape[0], int(g["N_max"])
    bufs = K.IntegratorBuffers(n, N, torch.float64, torch.device("cuda"))
    om = -float(g["Omega_bar"])
    K.integrate(S, _integ_cfg(0, N, omega=om, store_all=1), _cuda(w0.T, torch.float64),
                _cuda(g["dt_init"].reshape(-1), torch.float64), _cuda(g["T_total"].reshape(-1), torch.float64), bufs)
    smp = bufs.samples.cpu().numpy()
    traj = smp[:6].transpose(1, 2, 0).copy()
    traj[..., 3:] *= 0.9777922216807892
    np.testing.assert_allclose(traj, g["y_traj"].reshape(n, N, 6), rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(np.cumsum(smp[6], axis=1), g["t_traj"].reshape(n, N), rtol=1e-10)


def test_integrate_sampled_fp64_matches_oracle(K):
    """Uniform-time samples of the dense output; includes orbits that plunge to the
    centre and stall at dt_min (status bit 3) and keep the samples emitted so far."""
    rng = np.random.default_rng(15)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    n, Sn = 24, 64
    w, To = _orbit_states(rng, n, P)
    T_end = To * 3
    om = -35.79
    bufs = K.IntegratorBuffers(n, Sn, torch.float64, torch.device("cuda"))
    K.integrate(S, _integ_cfg(1, n_samples=Sn, omega=om, rtol=1e-6), _cuda(w.T, torch.float64),
                _cuda(To / 100, torch.float64), _cuda(T_end, torch.float64), bufs)
    ref = ointeg.integrate_sampled(w, P, om, T_end, Sn, To / 100, 1e-7, 1e-6, 1e-5, 0.3, max_attempts=200000)
    smp = bufs.samples.cpu().numpy()
    nst = bufs.n_stored.cpu().numpy()
    np.testing.assert_array_equal(nst, ref["n_emitted"])
    st = bufs.status.cpu().numpy()
    np.testing.assert_array_equal((st & 8) != 0, ref["stalled"])
    assert ref["stalled"].any() and not ref["stalled"].all()
    for o in range(n):
        np.testing.assert_allclose(smp[:6, o, :nst[o]].T, ref["ys"][:nst[o], o], rtol=1e-7, atol=1e-8)
        np.testing.assert_allclose(smp[6, o, :nst[o]], T_end[o] / Sn, rtol=1e-14)
    info = bufs.info.cpu().numpy()
    np.testing.assert_array_equal(info[4].astype(int), ref["n_acc"])
    np.testing.assert_array_equal(info[5].astype(int), ref["n_att"])


def _geometry(rot, n_part, n_real, symmetry=1):
    from schwarmax_gb300._lib import SmxBinning
    g = SmxBinning(n_part=n_part, n_real=n_real, nR=10, nz=6, nphi=8, R_lo=0.0, R_hi=10.0, z_lo=-3.0, z_hi=3.0,
                   phi_lo=-math.pi, phi_hi=math.pi, nX=16, nY=12, X_lo=-6.0, X_hi=6.0, Y_lo=-4.0, Y_hi=4.0,
                   n_bins=9, symmetry=symmetry)
    for i in range(9):
        g.rot[i] = float(rot.reshape(-1)[i])
    return g


def _aperture_map(rng, nX=16, nY=12, nb=9):
    pix = np.stack(np.meshgrid(np.arange(nX), np.arange(nY), indexing="xy"), -1).reshape(-1, 2)
    gen = pix[rng.choice(len(pix), nb, replace=False)]
    bm = np.argmin(((pix[:, None] - gen[None]) ** 2).sum(-1), 1)
    bm[rng.random(len(bm)) < 0.1] = -1     # holes outside every aperture
    return np.concatenate([bm, [-1]]).astype(np.int32)


@pytest.mark.parametrize("dtype,npdt", [(torch.float32, np.float32), (torch.float64, np.float64)])
def test_sample_cells_bit_exact(K, dtype, npdt):
    """Integer cell and aperture indices of the kernel equal the oracle's on the
    same points, evaluated in the same precision and operation order."""
    rng = np.random.default_rng(16)
    N = 200000
    pts = np.stack([rng.uniform(-11, 11, N), rng.uniform(-11, 11, N), rng.uniform(-3.5, 3.5, N),
                    rng.normal(0, 200, N), rng.normal(0, 200, N), rng.normal(0, 60, N)]).astype(npdt)
    # exact edge values: the upper edge is outside, the lower edge inside
    pts[0, :4] = [10.0, 0.0, 5.0, -2.0]
    pts[1, :4] = [0.0, 0.0, 0.0, 0.0]
    pts[2, :4] = [0.0, -3.0, 3.0, 1.0]
    rot = oorbits.rotation_matrix(30.0, 60.0, 45.0)
    geo = _geometry(rot, 1, 1)
    bm = _aperture_map(rng)
    cells, bins, vlos = K.sample_cells(geo, _cuda(pts, dtype), _cuda(bm, torch.int32))
    cells, bins = cells.cpu().numpy(), bins.cpu().numpy()
    lim = np.array([[0, 10.0], [-3, 3], [-math.pi, math.pi]])
    mism = 0
    for im, sg in enumerate(ogrid.SIGN_SYM):
        w = (pts.T * sg).astype(npdt)
        rz, vb, vl = ogrid.sample_cells(w[:, 0], w[:, 1], w[:, 2], w[:, 3], w[:, 4], w[:, 5], rot.astype(npdt),
                                        lim[:, 0], lim[:, 1], (10, 6, 8), np.array([-6.0, -4.0]),
                                        np.array([6.0, 4.0]), (16, 12), bm)
        np.testing.assert_array_equal(bins[im], vb)
        bad = cells[im] != rz
        if bad.any():
            # only the azimuth can differ, and only within 2 ulp of a cell edge
            # (atan2 is not correctly rounded on either side)
            ph = np.arctan2(w[bad, 1].astype(np.float64), w[bad, 0].astype(np.float64))
            edge = (ph + math.pi) / (2 * math.pi) * 8
            ulp = np.spacing(npdt(math.pi)) * 8 / (2 * math.pi)
            assert np.all(np.abs(edge - np.round(edge)) < 4 * ulp), "cell mismatch away from an edge"
            mism += bad.sum()
        np.testing.assert_allclose(vlos[im].cpu().double().numpy(), vl * 0.9777922216807892,
                                   rtol=1e-5 if npdt == np.float32 else 1e-13, atol=1e-3 if npdt == np.float32 else 1e-10)
    assert mism <= 2
    assert cells[0, 0] == 480 and cells[0, 1] < 480 and cells[0, 2] == 480


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_project_bin_matches_oracle(K, dtype):
    """Library columns from stored samples: oracle accumulation over the same samples."""
    rng = np.random.default_rng(17)
    pb, ph = _params()
    S, P = _structs(pb, ph)
    n_part, n_real, N = 12, 3, 250
    w, To = _orbit_states(rng, n_part * n_real, P)
    dt0 = To / 100
    Tt = To * 0.5
    Tt[5] = 1e6    # fails the time rule
    om = -35.79
    bufs = K.IntegratorBuffers(n_part * n_real, N, dtype, torch.device("cuda"))
    K.integrate(S, _integ_cfg(0, N, omega=om), _cuda(w.T, dtype), _cuda(dt0, dtype), _cuda(Tt, dtype), bufs)
    rot = oorbits.rotation_matrix(30.0, 60.0, 45.0)
    geo = _geometry(rot, n_part, n_real)
    bm = _aperture_map(rng)
    nb = 9
    npb = np.bincount(bm[bm >= 0], minlength=nb).astype(np.float64)
    v0 = rng.normal(0, 30, nb)
    s = rng.uniform(80, 200, nb)
    valid = torch.empty(n_part * n_real, dtype=torch.int8, device="cuda")
    lib = K.project_bin(geo, bufs, _cuda(Tt, dtype), _cuda(bm, torch.int32), _cuda(npb, torch.float64),
                        _cuda(v0, torch.float64), _cuda(s, torch.float64), valid=valid).cpu().double().numpy()
    # oracle: bin the kernel's own samples
    smp = bufs.samples.cpu().double().numpy()
    nst = bufs.n_stored.cpu().numpy()
    info = bufs.info.cpu().double().numpy()
    geoo = ointeg.BinGeometry(rot, [[0, 10.0], [-3, 3], [-math.pi, math.pi]], (10, 6, 8), [[-6, 6], [-4, 4]],
                              (16, 12), bm, npb, v0, s)
    acc = ointeg.Accumulator(n_part * n_real, geoo)
    ys = np.zeros((N, n_part * n_real, 6))
    ws = np.zeros((N, n_part * n_real))
    for o in range(n_part * n_real):
        ys[:nst[o], o] = smp[:6, o, :nst[o]].T
        ws[:nst[o], o] = smp[6, o, :nst[o]]
    acc.add(ys, ws)
    Rz, surf, h, vld = ointeg.normalise(acc, info[1], info[2], info[0], Tt)
    A_rz, A_xy, A_h = ointeg.realisation_mean(Rz, surf, h, vld, n_part, n_real)
    np.testing.assert_array_equal(valid.cpu().numpy(), vld.astype(np.int8))
    assert vld[5] == 0
    ref = np.concatenate([A_rz.T, A_xy.T] + [A_h[k].T for k in range(5)], axis=1)
    tol = 1e-12 if dtype == torch.float64 else 3e-6
    scale = np.abs(ref).max(1, keepdims=True) + 1e-300
    np.testing.assert_allclose(lib / scale, ref / scale, rtol=0, atol=tol)


def _nnls_case(rng, nrz=40, nb=12, n=96, B=5):
    A_rz = rng.uniform(0, 1, (nrz, n)) * (rng.uniform(0, 1, (nrz, n)) > 0.4)
    A_xy = rng.uniform(0, 1e-4, (nb, n))
    A_h = rng.normal(0, 1e-4, (5, nb, n))
    y_rz = A_rz @ rng.uniform(0.5, 1.5, n)
    y_xy = A_xy @ rng.uniform(0.5, 1.5, n) * 1.05
    gamma = rng.uniform(1e-3, 2e-3, nb)
    y_h = rng.normal(0, 0.05, (4, nb))
    sig_rz = 0.02 * y_rz + 1e-10
    sig_xy = 0.05 * y_xy
    sig_h = rng.uniform(0.02, 0.04, (4, nb))
    y_xy_b = y_xy[None] + rng.normal(0, 1, (B, nb)) * sig_xy[None]
    y_h_b = y_h[:, None] + rng.normal(0, 1, (4, B, nb)) * sig_h[:, None]
    return locals()


def _library_from(c):
    """(n, rows) library with rows [Rzphi | xy | h0 | h1..h4] from the A blocks."""
    return np.concatenate([c["A_rz"].T, c["A_xy"].T] + [c["A_h"][k].T for k in range(5)], axis=1)


def _nnls_inputs(c, w=(math.sqrt(5.0), math.sqrt(5.0), 1.0)):
    nrz, nb = c["nrz"], c["nb"]
    g = np.where(np.abs(c["gamma"]) > 1e-8, c["gamma"], 1e-8)
    row_map = np.concatenate([np.arange(nrz), nrz + np.arange(nb)] +
                             [nrz + (1 + k) * nb + np.arange(nb) for k in range(1, 5)]).astype(np.int32)
    rs = np.concatenate([w[0] / (c["sig_rz"] + 1e-8), w[1] / (c["sig_xy"] + 1e-8)] +
                        [w[2] / (g * (c["sig_h"][k] + 1e-8)) for k in range(4)])
    Y = np.stack([onnls.rhs_vector(c["y_rz"], c["y_xy_b"][b], *[c["y_h_b"][k][b] for k in range(4)], c["sig_rz"],
                                   c["sig_xy"], *c["sig_h"], w[0], w[1], w[2]) for b in range(c["B"])])
    return row_map, rs, Y


@pytest.mark.parametrize("mixed,tol", [(False, 1e-9), (True, 2e-7)])
def test_nnls_admm_matches_oracle(K, mixed, tol):
    """FP64 and mixed (split tensor-core products) ADMM against the oracle.  The
    mixed path takes a float library, so the oracle gets the same float-rounded
    design matrices; what remains is the solver's own error."""
    rng = np.random.default_rng(18)
    c = _nnls_case(rng)
    if mixed:
        c = dict(c, A_rz=c["A_rz"].astype(np.float32).astype(np.float64),
                 A_xy=c["A_xy"].astype(np.float32).astype(np.float64),
                 A_h=c["A_h"].astype(np.float32).astype(np.float64))
    w = (math.sqrt(5.0), math.sqrt(5.0), 1.0)
    ref = onnls.solve_nnls_admm_bootstrap(c["A_rz"], c["A_xy"], *c["A_h"][1:], c["y_rz"], c["y_xy"], c["gamma"],
                                          c["y_xy_b"], *c["y_h_b"], c["sig_rz"], c["sig_xy"], *c["sig_h"],
                                          lambda_reg=1.0, maxiter=150, w_rzphi=w[0], w_xy=w[1], w_h=w[2])
    row_map, rs, Y = _nnls_inputs(c, w)
    lib = _library_from(c)
    dtype = torch.float32 if mixed else torch.float64
    Z = K.nnls_admm(_cuda(lib, dtype), _cuda(row_map, torch.int32), _cuda(rs, torch.float64),
                    _cuda(Y, torch.float64), 150, 1.0, np.sum(c["y_rz"]) / c["n"], mixed).cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(Z / scale, ref / scale, rtol=0, atol=tol)


def test_nnls_admm_golden_fp64(K):
    g = golden("nnls")
    c = dict(A_rz=g["A_rz"], A_xy=g["A_xy"], A_h=np.concatenate([np.zeros_like(g["A_h"][:1]), g["A_h"]]),
             y_rz=g["y_rz"], gamma=g["gamma"], sig_rz=g["sig_rz"], sig_xy=g["sig_xy"], sig_h=g["sig_h"],
             y_xy_b=g["y_xy_b"], y_h_b=g["y_h_b"], nrz=g["A_rz"].shape[0], nb=g["A_xy"].shape[0],
             n=g["A_rz"].shape[1], B=g["y_xy_b"].shape[0])
    row_map, rs, Y = _nnls_inputs(c)
    Z = K.nnls_admm(_cuda(_library_from(c), torch.float64), _cuda(row_map, torch.int32), _cuda(rs, torch.float64),
                    _cuda(Y, torch.float64), int(g["maxiter"]), 1.0, np.sum(c["y_rz"]) / c["n"], False).cpu().numpy()
    np.testing.assert_allclose(Z, g["W_boot"], rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_model_maps_and_chi2(K, dtype):
    rng = np.random.default_rng(19)
    c = _nnls_case(rng)
    nrz, nb, n, B = c["nrz"], c["nb"], c["n"], c["B"]
    W = rng.uniform(0, 2, (B, n))
    v0, s = rng.normal(0, 20, nb), rng.uniform(80, 150, nb)
    y_xy_raw = rng.uniform(100, 200, nb)
    y_xy_b = y_xy_raw[None] * (1 + 0.01 * rng.normal(size=(B, nb)))
    sh = rng.uniform(0.02, 0.04, (4, nb))
    lum, amp = 3.7, 1.3
    maps, logl = K.model_maps(_cuda(_library_from(c), dtype), nrz, nb, _cuda(W, torch.float64),
                              _cuda(c["gamma"], torch.float64), _cuda(v0, torch.float64), _cuda(s, torch.float64),
                              _cuda(c["y_rz"], torch.float64), _cuda(y_xy_raw, torch.float64),
                              _cuda(y_xy_b, torch.float64), _cuda(c["y_h_b"], torch.float64),
                              _cuda(sh, torch.float64), lum, amp)
    d3, d2, h1, h2, h3, h4, V, sig = omodel.compute_model_batch(W, c["A_rz"], c["A_xy"], *c["A_h"][1:], c["gamma"], v0, s)
    d2 = d2 * lum
    ref = np.concatenate([d3, d2, h1, h2, h3, h4, V, sig], axis=1)
    tol = 1e-11 if dtype == torch.float64 else 1e-5
    sc = np.abs(ref).max(0, keepdims=True) + 1e-300
    np.testing.assert_allclose(maps.cpu().numpy() / sc, ref / sc, rtol=0, atol=tol)
    res_rz = np.nansum(((d3 - c["y_rz"]) / (0.1 * c["y_rz"] * amp)) ** 2)
    res = np.nansum(((d2 - y_xy_b) / (0.1 * y_xy_raw * amp)) ** 2, axis=1)
    for k, hk in enumerate((h1, h2, h3, h4)):
        res += np.nansum(((hk - c["y_h_b"][k]) / (sh[k] * amp)) ** 2, axis=1)
    np.testing.assert_allclose(logl.cpu().numpy(), -0.5 * (res + res_rz), rtol=1e-9 if dtype == torch.float64 else 1e-4)
