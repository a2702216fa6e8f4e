"""Orbit integration and library binning (oracle restatement).

Bogacki-Shampine 3(2) in the bar's rotating frame, integrates.py:8-112:
  rhs: dx = v + Om*y, dy = vy - Om*x, dz = vz, dvx = ax + Om*vy,
       dvy = ay - Om*vx, dvz = az            (Om = -Omega_bar)
  k2 = f(y + dt/2 k1), k3 = f(y + 3dt/4 k2), y3 = y + dt(2/9 k1 + 1/3 k2 + 4/9 k3)
  k4 = f(y3), err = dt(-5/72 k1 + 1/12 k2 + 1/9 k3 - 1/8 k4)
  err_norm = rms(err / (atol + rtol max(|y|,|y3|))), accept iff err_norm <= 1
  dt <- clip(dt clip(0.9 max(err_norm,1e-10)^(-1/3), 0.2, 5), dt_min, dt_max)

Two sampling modes share the stepper:
  "reference": a fixed number of attempts N_max; every attempt emits the
      post-attempt state with weight dt (0 when rejected), as
      integrate_adaptive_barred_chunked does (integrates.py:90-205).
  "sampled":   integrate until t >= T_end and emit S samples at the midpoints
      t_j = (j + 1/2) T_end / S of S equal intervals, interpolated with the
      cubic Hermite dense output of each accepted step (y, y3, k1, k4), each
      with weight T_end / S.  Attempts are capped at max_attempts.  An orbit whose
      attempt at dt = dt_min is rejected stalls (every later attempt would repeat
      it) and keeps only the samples emitted so far.

Binning of samples with the fourfold bar symmetry, GH accumulation,
normalisation by T_integrated = 4 sum(weights) + EPSILON, the E_J / time
validity rule and the realisation mean follow integrates.py:115-238, 290-298.
"""
import numpy as np

from . import grid, ghmoments, orbits
from . import potential as pot
from .constants import EPSILON, KPCGYR_TO_KMS

E1, E2, E3, E4 = -5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -1.0 / 8.0
SAFETY = 0.9


def deriv(w, P, Om):
    ax, ay, az = pot.acc(w[:, 0], w[:, 1], w[:, 2], P)
    return np.stack([w[:, 3] + Om * w[:, 1], w[:, 4] - Om * w[:, 0], w[:, 5],
                     ax + Om * w[:, 4], ay - Om * w[:, 3], az], -1)


def bs23_attempt(y, dt, k1, P, Om, atol, rtol, dt_min, dt_max):
    d = dt[:, None]
    k2 = deriv(y + 0.5 * d * k1, P, Om)
    k3 = deriv(y + 0.75 * d * k2, P, Om)
    y_new = y + d * (2.0 / 9.0 * k1 + 1.0 / 3.0 * k2 + 4.0 / 9.0 * k3)
    k4 = deriv(y_new, P, Om)
    err = d * (E1 * k1 + E2 * k2 + E3 * k3 + E4 * k4)
    scale = atol + rtol * np.maximum(np.abs(y), np.abs(y_new))
    en = np.sqrt(np.mean((err / scale) ** 2, axis=1))
    accept = en <= 1.0
    sf = np.clip(SAFETY * np.power(np.maximum(en, 1e-10), -1.0 / 3.0), 0.2, 5.0)
    dt_new = np.clip(dt * sf, dt_min, dt_max)
    return y_new, k4, accept, dt_new


def integrate_reference(w0, P, Om, n_attempts, dt_init, atol, rtol, dt_min, dt_max,
                        on_chunk=None, chunk=100, store=False):
    """w0: (N, 6).  Returns dict with t_final, y_final, EJ0, EJ_final, n_acc and,
    when store=True, ys (n_attempts, N, 6) and dts (n_attempts, N).
    on_chunk(ys_chunk, dts_chunk) is called for every `chunk` attempts."""
    y = np.array(w0, dtype=np.float64)
    N = y.shape[0]
    t = np.zeros(N)
    dt = np.array(dt_init, dtype=np.float64) * np.ones(N)
    k1 = deriv(y, P, Om)
    EJ0 = orbits.jacobi_energy(y, P, Om)
    n_acc = np.zeros(N, dtype=np.int64)
    buf_y, buf_dt = [], []
    all_y, all_dt = [], []
    for i in range(n_attempts):
        y_new, k4, acc, dt_new = bs23_attempt(y, dt, k1, P, Om, atol, rtol, dt_min, dt_max)
        y = np.where(acc[:, None], y_new, y)
        t = np.where(acc, t + dt, t)
        k1 = np.where(acc[:, None], k4, k1)
        dt_out = np.where(acc, dt, 0.0)
        n_acc += acc
        dt = dt_new
        if store:
            all_y.append(y.copy())
            all_dt.append(dt_out)
        if on_chunk is not None:
            buf_y.append(y.copy())
            buf_dt.append(dt_out)
            if len(buf_y) == chunk or i == n_attempts - 1:
                on_chunk(np.stack(buf_y), np.stack(buf_dt))
                buf_y, buf_dt = [], []
    out = dict(t_final=t, y_final=y, EJ0=EJ0, EJ_final=orbits.jacobi_energy(y, P, Om), n_acc=n_acc)
    if store:
        out["ys"] = np.stack(all_y)
        out["dts"] = np.stack(all_dt)
    return out


def integrate_sampled(w0, P, Om, T_end, n_samples, dt_init, atol, rtol, dt_min, dt_max,
                      max_attempts=1_000_000):
    """Returns dict with ys (n_samples, N, 6), weight (N,), t_final, y_final,
    EJ0, EJ_final, n_acc, n_att, capped."""
    y = np.array(w0, dtype=np.float64)
    N = y.shape[0]
    T_end = np.asarray(T_end, dtype=np.float64) * np.ones(N)
    t = np.zeros(N)
    dt = np.array(dt_init, dtype=np.float64) * np.ones(N)
    k1 = deriv(y, P, Om)
    EJ0 = orbits.jacobi_energy(y, P, Om)
    ys = np.zeros((n_samples, N, 6))
    nxt = np.zeros(N, dtype=np.int64)
    n_acc = np.zeros(N, dtype=np.int64)
    n_att = np.zeros(N, dtype=np.int64)
    active = np.ones(N, dtype=bool)
    stalled = np.zeros(N, dtype=bool)
    h = T_end / n_samples
    while active.any():
        idx = np.nonzero(active)[0]
        y_new, k4, acc, dt_new = bs23_attempt(y[idx], dt[idx], k1[idx], P, Om, atol, rtol, dt_min, dt_max)
        n_att[idx] += 1
        a = idx[acc]
        if a.size:
            t0 = t[a]
            dta = dt[a]
            t1 = t0 + dta
            y0, y1, f0, f1 = y[a], y_new[acc], k1[a], k4[acc]
            while True:
                tj = (nxt[a] + 0.5) * h[a]
                m = (nxt[a] < n_samples) & (tj <= t1)
                if not m.any():
                    break
                th = ((tj - t0) / dta)[m][:, None]
                th2, th3 = th * th, th * th * th
                yy = ((2 * th3 - 3 * th2 + 1) * y0[m] + (th3 - 2 * th2 + th) * dta[m][:, None] * f0[m]
                      + (-2 * th3 + 3 * th2) * y1[m] + (th3 - th2) * dta[m][:, None] * f1[m])
                ys[nxt[a][m], a[m]] = yy
                nxt[a[m]] += 1
            y[a] = y1
            k1[a] = f1
            t[a] = t1
            n_acc[a] += 1
        # a rejection at dt_min repeats forever (same state and step): the orbit stalls
        stalled[idx[~acc & (dt[idx] <= dt_min)]] = True
        dt[idx] = dt_new
        active = (nxt < n_samples) & (n_att < max_attempts) & ~stalled
    capped = nxt < n_samples
    return dict(ys=ys, weight=T_end / n_samples, t_final=t, y_final=y, EJ0=EJ0,
                EJ_final=orbits.jacobi_energy(y, P, Om), n_acc=n_acc, n_att=n_att, capped=capped,
                stalled=stalled, n_emitted=nxt)


class BinGeometry:
    """Grids, apertures and GH reference values shared by all samples."""

    def __init__(self, rot, rzphi_lim, n_rzphi, xy_lim, n_xy, bin_mapping, num_per_bin, v0, s):
        self.rot = np.asarray(rot, dtype=np.float64)
        self.rzphi_lim = np.asarray(rzphi_lim, dtype=np.float64)
        self.n_rzphi = np.asarray(n_rzphi, dtype=np.int64)
        self.xy_lim = np.asarray(xy_lim, dtype=np.float64)
        self.n_xy = np.asarray(n_xy, dtype=np.int64)
        self.bin_mapping = np.asarray(bin_mapping, dtype=np.int64)
        self.num_per_bin = np.asarray(num_per_bin, dtype=np.float64)
        self.v0 = np.asarray(v0, dtype=np.float64)
        self.s = np.asarray(s, dtype=np.float64)
        self.n_seg = int(np.prod(self.n_rzphi))
        self.n_bins = self.num_per_bin.shape[0]
        self.area_pixel = ((self.xy_lim[0, 1] - self.xy_lim[0, 0]) / self.n_xy[0]) * \
                          ((self.xy_lim[1, 1] - self.xy_lim[1, 0]) / self.n_xy[1]) * 1e6

    def cells(self, ys, dtype=np.float64, sym=True):
        """ys: (..., 6) -> list over symmetry images of (rz_cell, vbin, vlos)."""
        out = []
        pats = grid.SIGN_SYM if sym else grid.SIGN_SYM[:1]
        for sg in pats:
            w = (ys * sg).astype(dtype)
            c = grid.sample_cells(w[..., 0], w[..., 1], w[..., 2], w[..., 3], w[..., 4], w[..., 5],
                                  self.rot.astype(dtype), self.rzphi_lim[:, 0], self.rzphi_lim[:, 1],
                                  self.n_rzphi, self.xy_lim[:, 0], self.xy_lim[:, 1], self.n_xy,
                                  self.bin_mapping)
            out.append(c)
        return out


class Accumulator:
    """Per-orbit sums Rzphi (N, n_seg), counts and sw0..sw4 (N, n_bins), T."""

    def __init__(self, N, geo):
        self.geo = geo
        self.N = N
        self.rz = np.zeros(N * (geo.n_seg + 1))
        self.cnt = np.zeros(N * (geo.n_bins + 1))
        self.sw = np.zeros((5, N * (geo.n_bins + 1)))
        self.T = np.zeros(N)

    def add(self, ys, w, sym=True):
        """ys: (K, N, 6) samples, w: (K, N) weights."""
        g = self.geo
        K, N = w.shape
        orb = np.broadcast_to(np.arange(N)[None, :], (K, N))
        for rz_cell, vbin, vl in g.cells(ys, sym=sym):
            np.add.at(self.rz, (orb * (g.n_seg + 1) + rz_cell).ravel(), w.ravel())
            ok = vbin >= 0
            b = np.where(ok, vbin, g.n_bins)
            vkm = vl * KPCGYR_TO_KMS
            yv, gau = ghmoments.gauss(vkm, g.v0[b % g.n_bins], g.s[b % g.n_bins])
            Hs = ghmoments.hermite(yv)
            flat = (orb * (g.n_bins + 1) + b).ravel()
            np.add.at(self.cnt, flat, w.ravel())
            for k in range(5):
                np.add.at(self.sw[k], flat, (gau * w * Hs[k]).ravel())
            self.T += w.sum(axis=0)

    def rows(self):
        g = self.geo
        rz = self.rz.reshape(self.N, g.n_seg + 1)[:, :g.n_seg]
        cnt = self.cnt.reshape(self.N, g.n_bins + 1)[:, :g.n_bins]
        sw = self.sw.reshape(5, self.N, g.n_bins + 1)[:, :, :g.n_bins]
        return rz, cnt, sw, self.T


def normalise(acc, EJ0, EJ_final, t_final, T_total):
    """integrates.py:207-238.  Returns (Rzphi, surface, h (5, N, nb), valid)."""
    g = acc.geo
    rz, cnt, sw, T = acc.rows()
    Ti = T + EPSILON
    valid = ((np.abs(EJ_final / EJ0 - 1.0) < 0.1) & (t_final > T_total / 10)).astype(np.float64)
    v = valid[:, None]
    Rz = np.where(v > 0.5, rz / Ti[:, None], 0.0)
    surf = np.where(v > 0.5, (cnt / Ti[:, None]) / (g.num_per_bin * g.area_pixel + EPSILON), 0.0)
    h = np.where(v[None] > 0.5, sw / Ti[None, :, None], 0.0)
    return Rz, surf, h, valid


def realisation_mean(Rz, surf, h, valid, n_part, n_real):
    """integrates.py:287-298: column = sum_r row_r / (sum_r valid_r + 0.1).
    Inputs are ordered (particle, realisation).  Returns A matrices of shape
    (n_rows, n_part): A_Rzphi, A_xy, A_h (5, nb, n_part)."""
    wsum = valid.reshape(n_part, n_real).sum(1) + 0.1
    A_rz = (Rz.reshape(n_part, n_real, -1).sum(1) / wsum[:, None]).T
    A_xy = (surf.reshape(n_part, n_real, -1).sum(1) / wsum[:, None]).T
    A_h = np.stack([(h[k].reshape(n_part, n_real, -1).sum(1) / wsum[:, None]).T for k in range(5)])
    return A_rz, A_xy, A_h


def build_library(w0_batch, T_orb, P, Omega_bar, geo, mode="reference", n_attempts=5000,
                  chunk=100, n_samples=1000, n_periods=50, steps_per_period=100,
                  atol=1e-7, rtol=1e-4, dt_min=1e-5, dt_max=0.3, max_attempts=1_000_000):
    """Library of n_part columns from w0_batch (n_part, n_real, 6) and T_orb (n_part,).
    Settings default to model.py:163-169.  Returns dict with A_Rzphi, A_xy,
    A_h (h0..h4), valid (n_part, n_real), n_valid, plus the raw integration out."""
    n_real = w0_batch.shape[1]
    Tb = np.repeat(T_orb, n_real)
    return library_from_states(w0_batch, Tb * n_periods, Tb / steps_per_period, P, Omega_bar, geo,
                               mode, n_attempts, chunk, n_samples, atol, rtol, dt_min, dt_max, max_attempts)


def library_from_states(w0_batch, T_total, dt_init, P, Omega_bar, geo, mode="reference", n_attempts=5000,
                        chunk=100, n_samples=1000, atol=1e-7, rtol=1e-4, dt_min=1e-5, dt_max=0.3,
                        max_attempts=1_000_000):
    """As build_library with explicit per-orbit T_total and dt_init, ordered
    (particle, realisation) and flattened."""
    n_part, n_real, _ = w0_batch.shape
    w0 = w0_batch.reshape(-1, 6)
    T_total = np.asarray(T_total, dtype=np.float64).reshape(-1)
    dt_init = np.asarray(dt_init, dtype=np.float64).reshape(-1)
    Om = -Omega_bar
    acc = Accumulator(w0.shape[0], geo)
    if mode == "reference":
        res = integrate_reference(w0, P, Om, n_attempts, dt_init, atol, rtol, dt_min, dt_max,
                                  on_chunk=lambda ys, dts: acc.add(ys, dts), chunk=chunk)
    elif mode == "sampled":
        res = integrate_sampled(w0, P, Om, T_total, n_samples, dt_init, atol, rtol, dt_min, dt_max,
                                max_attempts=max_attempts)
        j = np.arange(n_samples)[:, None]
        wts = np.where(j < res["n_emitted"][None, :], res["weight"][None, :], 0.0)
        acc.add(res["ys"], wts)
    else:
        raise ValueError(mode)
    Rz, surf, h, valid = normalise(acc, res["EJ0"], res["EJ_final"], res["t_final"], T_total)
    A_rz, A_xy, A_h = realisation_mean(Rz, surf, h, valid, n_part, n_real)
    return dict(A_Rzphi=A_rz, A_xy=A_xy, A_h=A_h, valid=valid.reshape(n_part, n_real),
                n_valid=valid.reshape(n_part, n_real).sum(1), integ=res)


def trajectory_library(w0_batch, T_orb, P, Omega_bar, geo, n_attempts=5000, n_periods=50,
                       steps_per_period=100, atol=1e-7, rtol=1e-4, dt_min=1e-5, dt_max=0.3,
                       T_total=None, dt_init=None):
    """integrate_adaptive_withtraj_batch (integrates.py:319-570): every attempt
    stored, no symmetry images, dt normalised by T = sum(dt) + EPSILON.
    Returns the A matrices plus y_traj (n_part, n_real, N_max, 6) with
    velocities in km/s and t_traj = cumsum(dt)."""
    n_part, n_real, _ = w0_batch.shape
    w0 = w0_batch.reshape(-1, 6)
    if T_total is None:
        Tb = np.repeat(T_orb, n_real)
        T_total, dt_init = Tb * n_periods, Tb / steps_per_period
    T_total = np.asarray(T_total, dtype=np.float64).reshape(-1)
    dt_init = np.asarray(dt_init, dtype=np.float64).reshape(-1)
    res = integrate_reference(w0, P, -Omega_bar, n_attempts, dt_init, atol, rtol,
                              dt_min, dt_max, store=True)
    ys, dts = res["ys"], res["dts"]
    N = w0.shape[0]
    T = dts.sum(0) + EPSILON
    acc = Accumulator(N, geo)
    acc.add(ys, dts / T[None, :], sym=False)
    rz, cnt, sw, _ = acc.rows()
    valid = ((np.abs(res["EJ_final"] / res["EJ0"] - 1.0) < 0.1) & (res["t_final"] > T_total / 10)).astype(np.float64)
    v = valid[:, None]
    Rz = np.where(v > 0.5, rz, 0.0)
    surf = np.where(v > 0.5, cnt / (geo.num_per_bin * geo.area_pixel + EPSILON), 0.0)
    h = np.where(v[None] > 0.5, sw, 0.0)
    A_rz, A_xy, A_h = realisation_mean(Rz, surf, h, valid, n_part, n_real)
    traj = ys.transpose(1, 0, 2).copy()
    traj[..., 3:] *= KPCGYR_TO_KMS
    return dict(A_Rzphi=A_rz, A_xy=A_xy, A_h=A_h, valid=valid.reshape(n_part, n_real),
                y_traj=traj.reshape(n_part, n_real, n_attempts, 6),
                t_traj=np.cumsum(dts, axis=0).T.reshape(n_part, n_real, n_attempts), integ=res)
