"""Algebra of a batched leave-group-out jackknife, checked against the oracle's
per-replicate solves (model.py:290-603 via oracle.model.model_deltaChi2_jackknife:
replicate g sets sigma of the xy and h1..h4 rows of the bins with bin % n_groups == g
to 1e20 and re-runs the single-RHS ADMM of nnls.py:6-66).

The batched form needs one m x m inverse X = G^-1 of the full problem,
G = k I + U U^T with k = lambda/n + (|U|_F^2 + lambda)/n, for every replicate:
  * replicate g drops the rows d (their scaled entries are 1e-20 of the others, far
    below FP64 rounding), so its Woodbury matrix is k_g I + S_KK on the kept rows K
    (S = U U^T) and k_g I on d, with k_g = k - delta, delta = |U_d|_F^2 / n;
  * G_KK^-1 = X_KK - X_Kd X_dd^-1 X_dK (Schur complement of the dropped rows);
  * (G_KK - delta I)^-1 = sum_j delta^j G_KK^-(j+1), a Neumann series whose ratio is at
    most delta / k (the eigenvalues of G_KK are >= k);
  * each ADMM x-update in residual form: w = D + U_g^T (k_g I + U_g U_g^T)^-1 (y_g - U_g D),
    D = (rho_g / k_g)(z - u).
So all replicates iterate together on products with the same U and X (as extra right-hand
sides), with no factorisation per replicate.  This test pins the algebra in FP64 NumPy
before the split tensor-core kernels take it over."""
import numpy as np

from oracle import nnls as onnls


def _problem(seed=0, n=150, nc=40, nb=12):
    rng = np.random.default_rng(seed)
    occ = rng.random((nc + nb, n)) * (rng.random((nc + nb, n)) < 0.4)
    A_rz, A_xy = occ[:nc], occ[nc:]
    A_h = [rng.normal(0, 0.05, (nb, n)) * (A_xy > 0) for _ in range(4)]
    w_true = rng.random(n) * (rng.random(n) < 0.3)
    y_rz = A_rz @ w_true + 1e-3
    y_xy = A_xy @ w_true * (1 + 0.05 * rng.normal(size=nb)) + 1e-3
    gamma = A_xy @ w_true + 1e-3
    yh = [A @ w_true / gamma + 0.01 * rng.normal(size=nb) for A in A_h]
    sig_rz = 0.1 * y_rz
    sig_xy = 0.1 * y_xy
    sh = [np.full(nb, 0.03) for _ in range(4)]
    return dict(A_rz=A_rz, A_xy=A_xy, A_h=A_h, y_rz=y_rz, y_xy=y_xy, gamma=gamma, yh=yh, sig_rz=sig_rz,
                sig_xy=sig_xy, sh=sh, nc=nc, nb=nb, n=n)


W = dict(w_rzphi=np.sqrt(5.0), w_xy=np.sqrt(5.0), w_h=1.0)


def _reference(p, n_groups, lam, maxiter):
    """The oracle's replicate loop (sigma of the dropped rows = 1e20)."""
    grp = np.arange(p["nb"]) % n_groups
    out = []
    for g in range(n_groups):
        drop = grp == g
        sxy = np.where(drop, 1e20, p["sig_xy"])
        sh = [np.where(drop, 1e20, x) for x in p["sh"]]
        out.append(onnls.solve_nnls_admm(p["A_rz"], p["A_xy"], *p["A_h"], p["y_rz"], p["y_xy"], p["gamma"], *p["yh"],
                                         p["sig_rz"], sxy, *sh, lambda_reg=lam, maxiter=maxiter, **W))
    return np.array(out)


def _batched(p, n_groups, lam, maxiter, tol=1e-17, max_terms=200):
    U = onnls.design(p["A_rz"], p["A_xy"], *p["A_h"], p["gamma"], p["sig_rz"], p["sig_xy"], *p["sh"], **W)
    y = onnls.rhs_vector(p["y_rz"], p["y_xy"], *p["yh"], p["sig_rz"], p["sig_xy"], *p["sh"], **W)
    m, n = U.shape
    nc, nb = p["nc"], p["nb"]
    nrm2 = float(np.sum(U * U))
    k = lam / n + (nrm2 + lam) / n
    X = np.linalg.inv(k * np.eye(m) + U @ U.T)
    grp = np.arange(nb) % n_groups
    w0 = np.sum(p["y_rz"]) / n
    Z = np.full((n_groups, n), w0)
    Uu = np.zeros((n_groups, n))
    reps = []
    for g in range(n_groups):
        bins = np.nonzero(grp == g)[0]
        d = np.concatenate([nc + j * nb + bins for j in range(5)])   # xy, h1..h4 rows of the bins
        keep = np.ones(m, bool)
        keep[d] = False
        nd2 = float(np.sum(U[d] ** 2))
        rho = (nrm2 - nd2 + lam) / n
        kg = lam / n + rho
        reps.append(dict(d=d, keep=keep, rho=rho, kg=kg, delta=k - kg, Xdd_inv=np.linalg.inv(X[np.ix_(d, d)])))

    def gkk_inv(r, v):                       # G_KK^-1 v (v zero on d)
        t = X @ v
        corr = X[:, r["d"]] @ (r["Xdd_inv"] @ t[r["d"]])
        out = t - corr
        out[r["d"]] = 0.0
        return out

    terms = []
    for _ in range(maxiter):
        for g, r in enumerate(reps):
            Ug = U * r["keep"][:, None]
            yg = y * r["keep"]
            D = (r["rho"] / r["kg"]) * (Z[g] - Uu[g])
            e = yg - Ug @ D
            a = gkk_inv(r, e)
            v = a.copy()
            for j in range(max_terms):
                a = gkk_inv(r, r["delta"] * a)
                v += a
                if np.abs(a).max() <= tol * np.abs(v).max():
                    break
            terms.append(j + 2)
            w = D + Ug.T @ v
            wh = 1.6 * w - 0.6 * Z[g]
            zn = np.maximum(0.0, wh + Uu[g])
            Uu[g] = Uu[g] + wh - zn
            Z[g] = zn
    return Z, max(r["delta"] / k for r in reps), max(terms)


def _batched_h(p, n_groups, lam, maxiter, tol=1e-12):
    """The form the kernels iterate: H = X U once, then per replicate and iteration
    W = sum_t (delta S)^t E (S = G_KK^-1, E = y_g - U_g D, zero on d) and
    w = D + U^T S W = D + H^T W - H_d^T X_dd^-1 (X W)_d, since W vanishes on d."""
    U = onnls.design(p["A_rz"], p["A_xy"], *p["A_h"], p["gamma"], p["sig_rz"], p["sig_xy"], *p["sh"], **W)
    y = onnls.rhs_vector(p["y_rz"], p["y_xy"], *p["yh"], p["sig_rz"], p["sig_xy"], *p["sh"], **W)
    m, n = U.shape
    nc, nb = p["nc"], p["nb"]
    nrm2 = float(np.sum(U * U))
    k = lam / n + (nrm2 + lam) / n
    X = np.linalg.inv(k * np.eye(m) + U @ U.T)
    H = X @ U
    grp = np.arange(nb) % n_groups
    w0 = np.sum(p["y_rz"]) / n
    Z = np.full((n_groups, n), w0)
    Uu = np.zeros((n_groups, n))
    reps = []
    for g in range(n_groups):
        bins = np.nonzero(grp == g)[0]
        d = np.concatenate([nc + j * nb + bins for j in range(5)])
        keep = np.ones(m, bool)
        keep[d] = False
        rho = (nrm2 - float(np.sum(U[d] ** 2)) + lam) / n
        kg = lam / n + rho
        reps.append(dict(d=d, keep=keep, rho=rho, kg=kg, delta=k - kg, Xdd_inv=np.linalg.inv(X[np.ix_(d, d)])))
    q = max(r["delta"] / k for r in reps)
    terms = 1
    while q ** terms > tol:
        terms += 1

    def s_apply(r, v):                      # S v = X v - X_{:,d} X_dd^-1 (X v)_d, zero on d
        t = X @ v
        return t - X[:, r["d"]] @ (r["Xdd_inv"] @ t[r["d"]])

    for _ in range(maxiter):
        for g, r in enumerate(reps):
            D = (r["rho"] / r["kg"]) * (Z[g] - Uu[g])
            e = (y - U @ D) * r["keep"]
            v, Wg = e, e.copy()
            for _t in range(1, terms):
                v = r["delta"] * s_apply(r, v)
                Wg += v
            c = r["Xdd_inv"] @ (X[r["d"]] @ Wg)
            w = D + H.T @ Wg - H[r["d"]].T @ c
            wh = 1.6 * w - 0.6 * Z[g]
            zn = np.maximum(0.0, wh + Uu[g])
            Uu[g] = Uu[g] + wh - zn
            Z[g] = zn
    return Z, terms


def test_h_form_of_the_batched_jackknife():
    p = _problem(seed=2, nb=16)
    lam, it = 1.0, 120
    ref = _reference(p, p["nb"], lam, it)
    got, terms = _batched_h(p, p["nb"], lam, it)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    assert terms >= 2


def test_batched_jackknife_matches_per_replicate_solves():
    p = _problem()
    lam, it = 1.0, 200
    ref = _reference(p, 4, lam, it)
    got, ratio, terms = _batched(p, 4, lam, it)
    scale = np.abs(ref).max()
    assert ratio < 0.5                                   # the Neumann series converges
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * scale)


def test_leave_one_bin_out_needs_few_neumann_terms():
    p = _problem(seed=1, nb=20)
    lam, it = 1.0, 60
    ref = _reference(p, p["nb"], lam, it)
    got, ratio, terms = _batched(p, p["nb"], lam, it)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    # one bin's five rows hold a small share of |U|_F^2: a few terms reach 1e-17
    assert ratio < 0.2 and terms <= 40
