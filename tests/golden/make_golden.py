"""Generate golden vectors by running the reference's own Python modules.

JAX and astropy are not installed here, so the reference modules are imported
with ``tests/golden/jaxshim`` first on ``sys.path``: a NumPy float64
restatement of the JAX primitives they call (jit, vmap, grad, lax.scan/cond/
map, ops.segment_sum, scipy.linalg.cho_solve, scipy.integrate.trapezoid,
random) and of the two astropy unit conversions in constants.py.  Everything
else executed is the reference's code, unmodified, read from REF below.

Each case is small enough for a pure-Python run and is written to
``tests/golden/<case>.npz`` together with its inputs, including every random
draw the reference made (jax.random draws are logged by the shim), so that the
oracle can be replayed on the same numbers.

Usage:  python tests/golden/make_golden.py REF [case ...]
REF is the path of the reference checkout (required); the cases default to the
list at the end of this file.
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) < 2 or not os.path.isdir(sys.argv[1]):
    sys.exit("usage: python tests/golden/make_golden.py REF [case ...]   (REF: the reference checkout)")
REF = sys.argv[1]
sys.path[:0] = [os.path.join(HERE, "jaxshim"), REF]

import jax  # noqa: E402  (the shim)
import jax.numpy as jnp  # noqa: E402
import constants  # noqa: E402
import ghmoments  # noqa: E402
import integrates  # noqa: E402
import likelihood  # noqa: E402
import model  # noqa: E402
import nnls  # noqa: E402
import utils  # noqa: E402

OUT = HERE


def params_pair(scale=1.0):
    pb = dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3 * scale, logM_bar=10.0, L_bar=4.0 * scale,
              a_bar=0.8 * scale, b_bar=0.3 * scale, x_origin=0.0, y_origin=0.0, z_origin=0.0,
              dirx=0.0, diry=0.0, dirz=1.0)
    ph = dict(logM=12.0, Rs=20.6, a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0, z_origin=0.0,
              dirx=0.0, diry=0.0, dirz=1.0)
    return pb, ph


def flat_params(pb, ph):
    return np.array([pb["logM_disc"], pb["Rs_disc"], pb["Hs_disc"], pb["logM_bar"], pb["L_bar"],
                     pb["a_bar"], pb["b_bar"], ph["logM"], ph["Rs"]])


def save(name, **arrs):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
    print(f"  wrote {name}.npz ({', '.join(sorted(arrs))})")


def case_potential():
    rng = np.random.default_rng(1)
    out = {}
    for tag, sc in (("a", 1.0), ("b", 1.2)):
        pb, ph = params_pair(sc)
        x = rng.uniform(-12, 12, 96)
        y = rng.uniform(-12, 12, 96)
        z = rng.uniform(-3, 3, 96)
        x[:4] = [0.01, 4.0, -4.0, 15.0]
        y[:4] = [0.02, 0.0, 0.3, -2.0]
        z[:4] = [0.0, 0.0, -0.05, 2.5]
        phi = np.asarray(likelihood.potential_func(x, y, z, pb, ph))
        rho = np.asarray(likelihood.density_func(x, y, z, pb))

        def _pot(pos):
            return likelihood.potential_func(pos[0], pos[1], pos[2], pb, ph)

        acc = np.stack([-jax.grad(_pot)(jnp.array([x[i], y[i], z[i]])) for i in range(x.size)])
        out.update({f"{tag}_x": x, f"{tag}_y": y, f"{tag}_z": z, f"{tag}_phi": phi, f"{tag}_rho": rho,
                    f"{tag}_acc": acc, f"{tag}_params": flat_params(pb, ph)})
    save("potential", **out)


def case_small_funcs():
    rng = np.random.default_rng(2)
    v = rng.normal(0, 150, 64)
    v0 = rng.normal(0, 30, 64)
    s = rng.uniform(60, 200, 64)
    yv, gau = ghmoments.gauss(v, v0, s)
    H = np.stack([f(yv) for f in (ghmoments.H0, ghmoments.H1, ghmoments.H2, ghmoments.H3, ghmoments.H4)])
    h = rng.normal(0, 0.1, (4, 64))
    V, sig = ghmoments.h_to_V_sigma(h[0], h[1], v0, s, h3=h[2], h4=h[3])
    pos = np.concatenate([rng.uniform(-1, 11, (60, 3)), np.array([[0.0, -3.0, -math.pi], [10.0, 0.0, 0.0],
                                                               [5.0, 3.0, 1.0], [-1e-9, 0.0, 0.0]])])
    lo = np.array([0.0, -3.0, -math.pi])
    hi = np.array([10.0, 3.0, math.pi])
    nb = np.array([10, 6, 8])
    strides = np.concatenate([[1], np.cumprod(nb[:-1])])
    idx = np.asarray(utils.assign_regular_grid(pos, lo, hi, nb, strides))
    angles = np.array([[30.0, 60.0, 45.0], [25.0, 65.0, 45.0], [0.0, 0.0, 0.0], [170.0, 10.0, -80.0]])
    rots = np.stack([np.asarray(utils.makeRotationMatrix(*a)) for a in angles])
    menc = np.array([[10.76, math.log10(7.76)], [11.0, 1.0], [10.3, 0.7]])
    conv = np.array([utils.logMenc_logc_to_logM_logRs(a, b) for a, b in menc], dtype=np.float64)
    back = np.array([utils.logM_logRs_to_logMenc_logc(a, b) for a, b in conv], dtype=np.float64)
    pb, ph = params_pair()
    R = rng.uniform(0.05, 12, 32)
    z = rng.uniform(-1, 1, 32)
    T = np.asarray(jax.vmap(utils.estimate_orbital_timescale, in_axes=(0, None, None, 0))(
        R, likelihood.potential_func, (pb, ph), z))
    Vc = np.asarray(jax.vmap(utils.get_rotation_curve, in_axes=(0, None, None, 0))(
        R, likelihood.potential_func, (pb, ph), z))
    save("small_funcs", v=v, v0=v0, s=s, gh_y=yv, gh_gau=gau, gh_H=H, h=h, V=V, sig=sig,
         grid_pos=pos, grid_lo=lo, grid_hi=hi, grid_n=nb, grid_idx=idx, angles=angles, rots=rots,
         menc=menc, conv=conv, back=back, orb_R=R, orb_z=z, orb_T=T, orb_Vc=Vc,
         params=flat_params(pb, ph))


def case_jeans():
    rng = np.random.default_rng(3)
    pb, ph = params_pair()
    n = 5
    w0 = np.stack([rng.uniform(-6, 6, n), rng.uniform(-6, 6, n), rng.uniform(0, 0.6, n)], -1)
    jax.random.DRAWS.clear()
    k1, k2, k3 = jax.random.PRNGKey(42), jax.random.PRNGKey(109), jax.random.PRNGKey(2026)
    w = np.asarray(model.get_w0_new(w0, k1, k2, k3, n, pb, ph, likelihood.potential_func,
                                    likelihood.density_func))
    normals = np.stack([d[2] for d in jax.random.DRAWS if d[0] == "normal"])
    save("jeans", w0=w0, normals=normals, w0_new=w, params=flat_params(pb, ph))


def geometry():
    nX, nY = 8, 6
    X = np.array([-6.0, 6.0])
    Y = np.array([-4.0, 4.0])
    # 4 apertures: nearest of 4 generator pixels; sentinel -1 at index nX*nY
    gen = np.array([[1, 1], [6, 1], [2, 4], [5, 4]])
    ix, iy = np.meshgrid(np.arange(nX), np.arange(nY), indexing="xy")
    pix = np.stack([ix.ravel(), iy.ravel()], -1)          # idx = ix + iy*nX
    d2 = ((pix[:, None, :] - gen[None]) ** 2).sum(-1)
    bm = np.concatenate([np.argmin(d2, 1), [-1]]).astype(np.int32)
    npb = np.bincount(bm[:-1], minlength=4)
    return dict(nXY=np.array([nX, nY]), X=X, Y=Y, bin_mapping=bm, num_per_bin=npb,
                v0=np.array([10.0, -20.0, 5.0, 0.0]), s=np.array([120.0, 150.0, 90.0, 200.0]),
                nRzphi=np.array([5, 4, 6]), Rzphi_lim=np.array([[0.0, 10.0], [-3.0, 3.0], [-math.pi, math.pi]]))


def _acc_pot(pb, ph):
    def acc_fn(x, y, z):
        def _pot(pos):
            return likelihood.potential_func(pos[0], pos[1], pos[2], pb, ph)
        return -jax.grad(_pot)(jnp.array([x, y, z]))

    def pot_fn(x, y, z):
        return likelihood.potential_func(x, y, z, pb, ph)
    return acc_fn, pot_fn


def case_integrate():
    rng = np.random.default_rng(4)
    pb, ph = params_pair()
    g = geometry()
    n_p, n_r = 3, 2
    R = rng.uniform(1.0, 5.0, n_p)
    th = rng.uniform(0, 2 * math.pi, n_p)
    vc = np.array([180.0, 200.0, 160.0])
    w = np.zeros((n_p, n_r, 6))
    for i in range(n_p):
        for r in range(n_r):
            w[i, r] = [R[i] * math.cos(th[i]) + 0.05 * r, R[i] * math.sin(th[i]), 0.1 + 0.05 * r,
                       vc[i] * math.sin(th[i]) * 0.9, -vc[i] * math.cos(th[i]) * 0.9, 10.0 + 5 * r]
    Torb = 2 * math.pi * R / vc * np.ones((n_r, 1))
    Torb = Torb.T
    T_total = 50 * Torb
    T_total[2, 1] = 1e6        # invalid by the time rule
    dt_init = Torb / 100
    Omega_bar = 35.0 * 1.0227121650537077
    rot = np.asarray(utils.makeRotationMatrix(30.0, 60.0, 45.0))
    acc_fn, pot_fn = _acc_pot(pb, ph)
    N_max, chunk = 400, 100
    t0 = time.time()
    out = integrates._integrate_adaptive_batch_chunked_vmap(
        w, acc_fn, pot_fn, N_max, T_total, dt_init, -Omega_bar, 1e-7, 1e-4, 1e-5, 0.3,
        4, g["bin_mapping"], g["num_per_bin"], g["Rzphi_lim"], np.array([g["X"], g["Y"]]),
        g["nRzphi"], g["nXY"], int(np.prod(g["nRzphi"])), g["v0"], g["s"], rot, chunk)
    print(f"  integrate: {time.time() - t0:.1f}s")
    names = ["Rzphi", "surface", "h0", "h1", "h2", "h3", "h4", "n_valid"]
    res = {k: np.asarray(v) for k, v in zip(names, out)}
    save("integrate", w0=w, T_total=T_total, dt_init=dt_init, Omega_bar=np.array(Omega_bar),
         N_max=np.array(N_max), chunk=np.array(chunk), rot=rot, params=flat_params(pb, ph),
         **{"geo_" + k: v for k, v in g.items()}, **res)

    # trajectory variant, one realisation, no symmetry
    t0 = time.time()
    w1 = w[:2, :1]
    out = integrates._integrate_adaptive_withtraj_batch_vmap(
        w1, acc_fn, pot_fn, 300, T_total[:2, :1], dt_init[:2, :1], -Omega_bar, 1e-7, 1e-4, 1e-5, 0.3,
        4, g["bin_mapping"], g["num_per_bin"], g["Rzphi_lim"], np.array([g["X"], g["Y"]]),
        g["nRzphi"], g["nXY"], int(np.prod(g["nRzphi"])), g["v0"], g["s"], rot)
    print(f"  withtraj: {time.time() - t0:.1f}s")
    names = ["Rzphi", "surface", "h0", "h1", "h2", "h3", "h4", "n_valid", "y_traj", "t_traj"]
    res = {k: np.asarray(v) for k, v in zip(names, out)}
    save("withtraj", w0=w1, T_total=T_total[:2, :1], dt_init=dt_init[:2, :1], Omega_bar=np.array(Omega_bar),
         N_max=np.array(300), rot=rot, params=flat_params(pb, ph), **{"geo_" + k: v for k, v in g.items()}, **res)


def case_nnls():
    rng = np.random.default_rng(5)
    nrz, nb, n, B = 12, 5, 16, 4
    A_rz = rng.uniform(0, 1, (nrz, n)) * (rng.uniform(0, 1, (nrz, n)) > 0.3)
    A_xy = rng.uniform(0, 1e-4, (nb, n))
    A_h = [rng.normal(0, 1e-3, (nb, n)) for _ in range(4)]
    y_rz = A_rz @ rng.uniform(0.5, 1.5, n)
    y_xy = A_xy @ rng.uniform(0.5, 1.5, n) * 1.05
    gamma = rng.uniform(1e-3, 2e-3, nb)
    gamma[0] = 1e-9                          # exercises the |gamma| floor
    y_h = [rng.normal(0, 0.05, nb) for _ in range(4)]
    sig_rz = 0.02 * y_rz + 1e-10
    sig_xy = 0.05 * y_xy
    sig_h = [rng.uniform(0.02, 0.04, nb) for _ in range(4)]
    y_xy_b = y_xy[None] + rng.normal(0, 1, (B, nb)) * sig_xy[None]
    y_h_b = [y_h[k][None] + rng.normal(0, 1, (B, nb)) * sig_h[k][None] for k in range(4)]
    maxiter = 80
    Wb = np.asarray(nnls.solve_nnls_admm_bootstrap(A_rz, A_xy, *A_h, y_rz, y_xy, gamma, y_xy_b, *y_h_b,
                                                   sig_rz, sig_xy, *sig_h, lambda_reg=1.0, maxiter=maxiter,
                                                   w_rzphi=math.sqrt(5.0), w_xy=math.sqrt(5.0), w_h=1.0))
    W1 = np.asarray(nnls.solve_nnls_admm(A_rz, A_xy, *A_h, y_rz, y_xy, gamma, *y_h, sig_rz, sig_xy, *sig_h,
                                         lambda_reg=0.5, maxiter=maxiter))
    v0 = rng.normal(0, 20, nb)
    s = rng.uniform(80, 150, nb)
    maps = model.compute_model_single_vmap(Wb, A_rz, A_xy, *A_h, gamma, v0, s)
    save("nnls", A_rz=A_rz, A_xy=A_xy, A_h=np.stack(A_h), y_rz=y_rz, y_xy=y_xy, gamma=gamma,
         y_h=np.stack(y_h), sig_rz=sig_rz, sig_xy=sig_xy, sig_h=np.stack(sig_h), y_xy_b=y_xy_b,
         y_h_b=np.stack(y_h_b), maxiter=np.array(maxiter), W_boot=Wb, W_single=W1, v0=v0, s=s,
         **{f"map{i}": np.asarray(m) for i, m in enumerate(maps)})


def tiny_dict_data(rng, n_part=2, n_boot=3):
    from scipy.stats import qmc
    g = geometry()
    nb = 4
    n_R, n_z, n_phi = 4, 3, 4
    Re = np.linspace(0.0, 10.0, n_R + 1)
    ze = np.linspace(-3.0, 3.0, n_z + 1)
    pe = np.linspace(-math.pi, math.pi, n_phi + 1)
    mids = [0.5 * (e[:-1] + e[1:]) for e in (Re, ze, pe)]
    RR, ZZ, PP = np.meshgrid(*mids, indexing="ij")
    mid = np.stack([RR.ravel(), ZZ.ravel(), PP.ravel()], -1)
    lim = np.array([[0.0, 10.0], [-3.0, 3.0], [-math.pi, math.pi]])
    nR = np.array([n_R, n_z, n_phi])
    idx = np.asarray(utils.assign_regular_grid(mid, lim[:, 0], lim[:, 1], nR, np.array([1, n_R, n_R * n_z])))
    o = np.argsort(idx)
    sd = rng.uniform(500.0, 2000.0, nb)
    h = [rng.normal(0, 0.03, nb) for _ in range(4)]
    herr = [np.full(nb, 0.03) for _ in range(4)]
    normals = [rng.normal(size=(n_boot, nb)) for _ in range(5)]
    for a in normals:
        a[0] = 0.0
    R = rng.uniform(1.0, 4.0, n_part)
    ph = rng.uniform(0, 2 * math.pi, n_part)
    w0 = np.stack([R * np.cos(ph), R * np.sin(ph), rng.uniform(0.0, 0.4, n_part)], -1)
    d = dict(v0=g["v0"], s=g["s"], XY_density_data=sd, XY_density_data_err=0.01 * sd + 1e-12,
             num_per_bin=g["num_per_bin"], bin_mapping=g["bin_mapping"], total_bins=nb,
             XY_standard_normal=normals[0], R_grid=mid[o, 0], z_grid=mid[o, 1], phi_grid=mid[o, 2],
             R_minmax=[0.0, 10.0], z_minmax=[-3.0, 3.0], phi_minmax=[-math.pi, math.pi],
             Rzphi_n_tot=int(nR.prod()), Rzphi_n_grid=nR, dR=Re[1] - Re[0], dz=ze[1] - ze[0],
             dphi=pe[1] - pe[0], sample_for_integration=qmc.Sobol(d=3, scramble=False).random_base2(m=10),
             X_minmax=g["X"], Y_minmax=g["Y"], nX_nY=g["nXY"], w0=w0)
    for k in range(4):
        d[f"h{k + 1}_data"] = h[k]
        d[f"h{k + 1}_data_err"] = herr[k]
        d[f"h{k + 1}_standard_normal"] = normals[k + 1]
    return d


def case_end_to_end():
    rng = np.random.default_rng(6)
    d = tiny_dict_data(rng)
    theta = np.array([10.76, 10.83, 10.2, math.log10(7.76), math.log10(3.0), math.log10(0.3),
                      math.log10(4.0), 30 * math.pi / 180, 60 * math.pi / 180, 45 * math.pi / 180,
                      0.05, math.log10(35.79)])
    jax.random.DRAWS.clear()
    t0 = time.time()
    logl = float(likelihood.model_likelihood(theta, d, 4, 48, sigma_amplify=1.3))
    print(f"  model_likelihood: {time.time() - t0:.1f}s  logL={logl}")
    normals = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "normal"][:3])
    unif = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "uniform"][:6])
    # build_model outputs at the same parameters (same draws: keys are fixed)
    halo = likelihood.logMenc_logc_to_logM_logRs(theta[0], theta[3], r_enc=10.0, Delta=200., rho_crit=277.54)
    pb = dict(logM_disc=theta[1], Rs_disc=10 ** theta[4], Hs_disc=10 ** theta[5], logM_bar=theta[2],
              L_bar=10 ** theta[6], a_bar=10 ** theta[6] / 5, b_bar=10 ** theta[5],
              mass_to_light_ratio=10 ** theta[10], Omega_bar=10 ** theta[11], x_origin=0.0, y_origin=0.0,
              z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0, alpha=theta[7] * 180 / math.pi,
              beta=theta[8] * 180 / math.pi, gamma=theta[9] * 180 / math.pi)
    phh = dict(logM=halo[0], Rs=10 ** halo[1], a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0,
               z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    t0 = time.time()
    md = model.build_model(likelihood.density_func, likelihood.potential_func, phh, pb, d, 4, 48,
                           np.asarray(d["Rzphi_n_grid"]), np.array([d["R_minmax"], d["z_minmax"], d["phi_minmax"]]),
                           np.array([d["X_minmax"], d["Y_minmax"]]), np.asarray(d["nX_nY"]), nnls_maxiter=60)
    print(f"  build_model: {time.time() - t0:.1f}s")
    t0 = time.time()
    dchi2 = float(likelihood.calculate_delta_chi2(theta, d, 4, 48))
    print(f"  calculate_delta_chi2: {time.time() - t0:.1f}s  dchi2={dchi2}")
    arrays = {"dd_" + k: np.asarray(v) for k, v in d.items()}
    arrays.update({"bm_" + k: np.asarray(v) for k, v in md.items()})
    save("end_to_end", theta=theta, logL=np.array(logl), delta_chi2=np.array(dchi2), sigma_amplify=np.array(1.3),
         jeans_normals=normals, jitter_uniforms=unif, **arrays)


def case_with_orbit():
    """get_model_with_orbit on the end_to_end data; it draws its own jitter
    (shape (n, 1)), which is logged separately."""
    rng = np.random.default_rng(6)
    d = tiny_dict_data(rng)
    g = np.load(os.path.join(OUT, "end_to_end.npz"))
    theta = g["theta"]
    halo = likelihood.logMenc_logc_to_logM_logRs(theta[0], theta[3], r_enc=10.0, Delta=200., rho_crit=277.54)
    pb = dict(logM_disc=theta[1], Rs_disc=10 ** theta[4], Hs_disc=10 ** theta[5], logM_bar=theta[2],
              L_bar=10 ** theta[6], a_bar=10 ** theta[6] / 5, b_bar=10 ** theta[5],
              mass_to_light_ratio=10 ** theta[10], Omega_bar=10 ** theta[11], x_origin=0.0, y_origin=0.0,
              z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0, alpha=theta[7] * 180 / math.pi,
              beta=theta[8] * 180 / math.pi, gamma=theta[9] * 180 / math.pi)
    phh = dict(logM=halo[0], Rs=10 ** halo[1], a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0,
               z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    jax.random.DRAWS.clear()
    t0 = time.time()
    mo = model.get_model_with_orbit(likelihood.density_func, likelihood.potential_func, phh, pb, d, 4, 48,
                                    np.asarray(d["Rzphi_n_grid"]),
                                    np.array([d["R_minmax"], d["z_minmax"], d["phi_minmax"]]),
                                    np.array([d["X_minmax"], d["Y_minmax"]]), np.asarray(d["nX_nY"]), nnls_maxiter=60)
    print(f"  get_model_with_orbit: {time.time() - t0:.1f}s")
    normals = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "normal"][:3])
    unif = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "uniform"][:6])
    save("with_orbit", theta=theta, jeans_normals=normals, jitter_uniforms=unif,
         **{"mo_" + k: np.asarray(mo[k]) for k in ("weights", "weights_all_boot", "y_traj", "t_traj",
                                                     "mass_per_orbit", "density_3d", "density_3d_model",
                                                     "surface_density", "h1", "h2", "h3", "h4", "V", "sigma")})


def case_example_data():
    """The reference's loader (utils.py:572-743) on the example galaxy of its
    checkout (example/mock_Nbody_galaxy_beta65_gamma45_D50.pkl: 609 Voronoi
    apertures on a 60 x 40 pixel map).  Saved: the pickle's arrays as inputs
    (in_*), and the loader's outputs (out_*) with the first two rows of each
    bootstrap draw; the threefry-drawn w0 is left out (the device path draws its
    own)."""
    import pickle
    name = "mock_Nbody_galaxy_beta65_gamma45_D50.pkl"
    path = os.path.join(REF, "example") + os.sep
    with open(path + name, "rb") as f:
        raw = pickle.load(f)               # jax arrays come back as NumPy through the shim
    d = utils.load_data_bootstrap(path, name)
    out = {}
    for k, v in d.items():
        a = np.asarray(v)
        if k == "w0":
            continue
        out["out_" + k] = a[:2] if k.endswith("_standard_normal") else a
    save("example_data", **{"in_" + k: np.asarray(v) for k, v in raw.items()}, **out)


def case_example_end_to_end():
    """model_likelihood and build_model on the example galaxy's apertures and grids
    (609 bins on 60 x 40 pixels, 10 x 6 x 10 cells), with the loader's n_samples = 2
    particles and N_BOOTSTRAP = 3, at the example's viewing angles (25, 65, 45 deg)."""
    name = "mock_Nbody_galaxy_beta65_gamma45_D50.pkl"
    d = utils.load_data_bootstrap(os.path.join(REF, "example") + os.sep, name, N_BOOTSTRAP=3, n_samples=2)
    nb, nc = int(d["total_bins"]), int(d["Rzphi_n_tot"])
    theta = np.array([10.76, 10.83, 10.2, math.log10(7.76), math.log10(3.0), math.log10(0.3),
                      math.log10(4.0), 25 * math.pi / 180, 65 * math.pi / 180, 45 * math.pi / 180,
                      0.05, math.log10(35.79)])
    jax.random.DRAWS.clear()
    t0 = time.time()
    logl = float(likelihood.model_likelihood(theta, d, nb, nc, sigma_amplify=1.3))
    print(f"  model_likelihood: {time.time() - t0:.1f}s  logL={logl}")
    normals = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "normal"][:3])
    unif = np.stack([x[2] for x in jax.random.DRAWS if x[0] == "uniform"][:6])
    halo = likelihood.logMenc_logc_to_logM_logRs(theta[0], theta[3], r_enc=10.0, Delta=200., rho_crit=277.54)
    pb = dict(logM_disc=theta[1], Rs_disc=10 ** theta[4], Hs_disc=10 ** theta[5], logM_bar=theta[2],
              L_bar=10 ** theta[6], a_bar=10 ** theta[6] / 5, b_bar=10 ** theta[5],
              mass_to_light_ratio=10 ** theta[10], Omega_bar=10 ** theta[11], x_origin=0.0, y_origin=0.0,
              z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0, alpha=theta[7] * 180 / math.pi,
              beta=theta[8] * 180 / math.pi, gamma=theta[9] * 180 / math.pi)
    phh = dict(logM=halo[0], Rs=10 ** halo[1], a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0,
               z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    t0 = time.time()
    md = model.build_model(likelihood.density_func, likelihood.potential_func, phh, pb, d, nb, nc,
                           np.asarray(d["Rzphi_n_grid"]), np.array([d["R_minmax"], d["z_minmax"], d["phi_minmax"]]),
                           np.array([d["X_minmax"], d["Y_minmax"]]), np.asarray(d["nX_nY"]), nnls_maxiter=60)
    print(f"  build_model: {time.time() - t0:.1f}s")
    arrays = {"dd_" + k: np.asarray(v) for k, v in d.items()}
    arrays.update({"bm_" + k: np.asarray(v) for k, v in md.items()})
    save("example_end_to_end", theta=theta, logL=np.array(logl), sigma_amplify=np.array(1.3), jeans_normals=normals,
         jitter_uniforms=unif, **arrays)


def case_example_jackknife():
    """calculate_delta_chi2 (leave-one-bin-out over the 609 apertures) on the
    example_end_to_end data and parameters, with the same draws."""
    g = np.load(os.path.join(OUT, "example_end_to_end.npz"))
    d = {k[3:]: g[k] for k in g.files if k.startswith("dd_")}
    d["total_bins"] = int(d["total_bins"])
    d["Rzphi_n_tot"] = int(d["Rzphi_n_tot"])
    jax.random.DRAWS.clear()
    t0 = time.time()
    dchi2 = float(likelihood.calculate_delta_chi2(g["theta"], d, d["total_bins"], d["Rzphi_n_tot"]))
    print(f"  calculate_delta_chi2: {time.time() - t0:.1f}s  dchi2={dchi2}")
    save("example_jackknife", theta=g["theta"], delta_chi2=np.array(dchi2))


def case_dehnen_types():
    """Potential, density and -grad Phi (jax.grad) of every Dehnen & Aly model T1..T4 and
    V1..V4 of the reference (dehnen_bar.py:1272-1568), each with its own (M, a, b, L,
    gamma), at 64 points."""
    import dehnen_bar as db
    rng = np.random.default_rng(9)
    out = {}
    specs = {"T1": (1e10, 0.8, 0.3, 3.0, 0.4), "T2": (2e10, 1.0, 0.4, 4.0, 1.0), "T3": (1e10, 0.8, 0.3, 4.0, 0.7),
             "T4": (1.5e10, 0.6, 0.5, 2.5, 0.0), "V1": (5e9, 0.5, 0.6, 0.4, 0.3), "V2": (5e9, 0.4, 0.5, 0.1, 0.0),
             "V3": (8e9, 0.7, 0.3, 1.5, 0.5), "V4": (5e9, 0.5, 0.5, 0.1, 0.0)}
    for name, (M, a, b, L, gam) in specs.items():
        fphi = getattr(db, name + "_potential")
        frho = getattr(db, name + "_density")
        x = rng.uniform(-8, 8, 64)
        y = rng.uniform(-6, 6, 64)
        z = rng.uniform(-2, 2, 64)
        x[:3] = [0.05, 3.0, -9.0]
        y[:3] = [0.0, 0.01, 1.0]
        z[:3] = [0.0, -0.02, 0.5]
        phi = np.array([float(fphi(x[i], y[i], z[i], M, a, b, L, gam)) for i in range(64)])
        rho = np.array([float(frho(x[i], y[i], z[i], M, a, b, L, gam)) for i in range(64)])

        def _p(pos, f=fphi, M=M, a=a, b=b, L=L, gam=gam):
            return f(pos[0], pos[1], pos[2], M, a, b, L, gam)

        acc = np.stack([-jax.grad(_p)(jnp.array([x[i], y[i], z[i]])) for i in range(64)])
        out.update({f"{name}_params": np.array([M, a, b, L, gam]), f"{name}_x": x, f"{name}_y": y, f"{name}_z": z,
                    f"{name}_phi": phi, f"{name}_rho": rho, f"{name}_acc": acc})
    save("dehnen_types", **out)


def case_analysis():
    """build_Lcirc_of_E (utils.py:275-341) of the canonical potential on a 400-point
    table with its interpolator at a set of energies, and compute_transfer_matrix
    (utils.py:413-485) on the example galaxy's 609 apertures (60 x 40 pixels) on a
    150 x 150 fine grid with a 0.3 kpc PSF."""
    pb, ph = params_pair()
    interp, E, L = utils.build_Lcirc_of_E(likelihood.potential_func, (pb, ph), R_min=1e-2, R_max=1e2, n_grid=400)
    rng = np.random.default_rng(5)
    Eq = np.concatenate([rng.uniform(E[0], E[-1], 300), E[[0, 7, 100, -1]], [E[0] - 10.0, E[-1] + 10.0]])
    Lq = np.asarray(interp(Eq))
    g = np.load(os.path.join(OUT, "example_data.npz"))
    bm = g["out_bin_mapping"]
    nX, nY = (int(v) for v in g["out_nX_nY"])
    P = utils.compute_transfer_matrix(0.3, nX, nY, g["out_X_minmax"], g["out_Y_minmax"], bm, int(g["out_total_bins"]),
                                      grid_res=150)
    save("analysis", params=flat_params(pb, ph), E_circ=E, L_circ=L, E_query=Eq, L_query=Lq, psf_sigma=np.array(0.3),
         psf_grid_res=np.array(150), psf_P=P)


def case_cylspline():
    """evaluate_phi and get_acc (CylindricalSpline.py:354-519) on a table in the format
    of get_phi_m (CylindricalSpline.py:270-352): the azimuthal modes m = 0..4 of the
    canonical potential on get_phi_m's (R, z) grid (R geometric in [0.01, 30], z = 0 and
    geometric in [0.01, 10], R0 = R[NR // 2], both in asinh(./R0)), with the second
    derivatives from the reference's own jax_precompute_splines (CubicSpline.py:55-97),
    evaluated at 160 points inside and 8 outside the grid."""
    import CubicSpline as cub
    import CylindricalSpline as cs
    pb, ph = params_pair()
    NR, NZ, Mmax, Nphi = 24, 16, 4, 32
    R = np.geomspace(1e-2, 30.0, NR)
    Z = np.concatenate([[0.0], np.geomspace(1e-2, 10.0, NZ)])
    R0 = R[NR // 2]
    Rt, Zt = np.arcsinh(R / R0), np.arcsinh(Z / R0)
    ang = np.linspace(0.0, 2 * np.pi, Nphi, endpoint=False)
    Rg, Zg, Ag = np.meshgrid(R, Z, ang, indexing="ij")
    Phi = np.asarray(likelihood.potential_func((Rg * np.cos(Ag)).ravel(), (Rg * np.sin(Ag)).ravel(), Zg.ravel(),
                                               pb, ph)).reshape(Rg.shape)
    modes = np.fft.fft(Phi, axis=2)[..., :Mmax + 1] / Nphi          # Phi_m = mean of Phi e^{-i m phi}
    tab = {k: np.zeros((Mmax + 1, NR, NZ + 1)) for k in ("Phi_m_real", "Phi_m_img", "Mx_real", "My_real",
                                                         "Mx_img", "My_img")}
    for m in range(Mmax + 1):
        for part, vals in (("real", modes[..., m].real), ("img", modes[..., m].imag)):
            tab[f"Phi_m_{part}"][m] = vals
            Mx, My = cub.jax_precompute_splines((Rt, Zt), vals)
            tab[f"Mx_{part}"][m] = np.asarray(Mx)
            tab[f"My_{part}"][m] = np.asarray(My)
    d = dict(Rgrid=Rt, Zgrid=Zt, R0=np.array([R0]), m=np.arange(Mmax + 1), **tab)
    rng = np.random.default_rng(11)
    n = 160
    Rq = np.exp(rng.uniform(np.log(0.02), np.log(25.0), n))
    aq = rng.uniform(-np.pi, np.pi, n)
    zq = rng.uniform(-8.0, 8.0, n) * rng.uniform(0, 1, n) ** 2
    x, y = Rq * np.cos(aq), Rq * np.sin(aq)
    x[:4], y[:4], zq[:4] = [3.0, 0.0, -2.0, 1e-3], [0.0, 2.5, -2.0, 0.0], [0.0, 0.0, -1.5, 0.3]
    # outside the grid: fill value 0 for Phi and its derivatives
    x = np.concatenate([x, [40.0, 0.0, -35.0, 5.0, 0.0, 3.0, 20.0, -1.0]])
    y = np.concatenate([y, [0.0, 45.0, 10.0, 1.0, 0.0, 0.0, 25.0, 0.5]])
    zq = np.concatenate([zq, [0.0, 1.0, -2.0, 12.0, -15.0, 11.0, 0.0, -10.5]])
    phi = np.asarray(cs.evaluate_phi(x, y, zq, d))
    acc = np.asarray(cs.get_acc(x, y, zq, d))
    save("cylspline", x=x, y=y, z=zq, phi=phi, acc=acc, params=flat_params(pb, ph), **d)


if __name__ == "__main__":
    print("G =", constants.G, "KPCGYR_TO_KMS =", constants.KPCGYR_TO_KMS)
    cases = sys.argv[2:] or ["potential", "small_funcs", "jeans", "integrate", "nnls", "end_to_end", "with_orbit",
                             "example_data"]
    for c in cases:
        print("case", c)
        globals()["case_" + c]()
