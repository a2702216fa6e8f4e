"""Canonical SchwarMAX potential and stellar density (oracle restatement).

Phi = NFW halo + Miyamoto-Nagai disc + Dehnen-Aly T3 bar (gamma=1)
      + Dehnen-Aly V4 bulge (a=b=0.5, L=0.1, gamma=0)
rho = Miyamoto-Nagai + T3 + V4 (stellar only)

Follows likelihood.py:10-71 (model assembly, V4 constants, V4 mass tied to the
bar mass), potentials.py:18-65 (NFW, MN potential and density, including the
EPSILON offsets), dehnen_bar.py:104-157 (A/B/Ax recurrence), 211-241 (needle
convolution), 269-278 (C = x*A - B), 1318-1326 (T3 Phi), 1371-1383 (V4 Phi),
1425-1438 (T3 rho), 1526-1543 (V4 rho).  Only the canonical configuration is
supported: halo/disc origin 0 and symmetry axis (0,0,1), for which
utils.get_mat (utils.py:70-99) is the identity.

All routines accept ndarrays or oracle.dual.Dual values, so the acceleration
is the exact gradient of the same expression (the reference uses jax.grad).
"""
import math

from . import dual as D
from .constants import G, EPSILON

V4_A, V4_B, V4_L, V4_GAMMA = 0.5, 0.5, 0.1, 0.0      # likelihood.py:10
GAMMA_BAR = 1.0                                        # likelihood.py:11


def canonical_params(params_baryon, params_halo, bulge_mass=None):
    """Flatten the reference's parameter dicts into the canonical set.

    Raises NotImplementedError for shifted or tilted components (the
    reference's _shift/_rotate path, potentials.py:8-15) since the canonical
    likelihood never uses them.
    """
    for p, keys in ((params_baryon, ("x_origin", "y_origin", "z_origin", "dirx", "diry")),
                    (params_halo, ("x_origin", "y_origin", "z_origin", "dirx", "diry"))):
        for k in keys:
            if k in p and float(p[k]) != 0.0:
                raise NotImplementedError(f"non-canonical component geometry: {k}={p[k]}")
        if "dirz" in p and float(p["dirz"]) <= 0.0:
            raise NotImplementedError("symmetry axis must be +z")
    m_bar = 10.0 ** float(params_baryon["logM_bar"])
    return dict(
        halo_M=10.0 ** float(params_halo["logM"]),
        halo_Rs=float(params_halo["Rs"]),
        halo_qa=float(params_halo.get("a", 1.0)),
        halo_qb=float(params_halo.get("b", 1.0)),
        halo_qc=float(params_halo.get("c", 1.0)),
        disc_M=10.0 ** float(params_baryon["logM_disc"]),
        disc_a=float(params_baryon["Rs_disc"]),
        disc_b=float(params_baryon["Hs_disc"]),
        bar_M=m_bar,
        bar_a=float(params_baryon["a_bar"]),
        bar_b=float(params_baryon["b_bar"]),
        bar_L=float(params_baryon["L_bar"]),
        bar_gamma=GAMMA_BAR,
        bulge_M=m_bar if bulge_mass is None else float(bulge_mass),
        bulge_a=V4_A, bulge_b=V4_B, bulge_L=V4_L, bulge_gamma=V4_GAMMA,
    )


# --------------------------------------------------------------------------
# Dehnen & Aly needle machinery
# --------------------------------------------------------------------------
def _acrn_odd(xp, u2, nmax):
    """A_n, B_n for odd n = 1..nmax at (xp, u2) (dehnen_bar.py:104-142)."""
    R2 = xp * xp + u2
    iR2 = 1.0 / R2
    r = D.sqrt(R2)
    Ax = 1.0 / r
    A = D.log(xp + r)
    B = r
    out = {1: (A, B)}
    cur = 1
    while cur < nmax:
        B_new = -Ax / cur
        A_new = ((cur - 1) * A + xp * Ax) / (cur * u2)
        Ax = Ax * iR2
        A, B = A_new, B_new
        cur += 2
        out[cur] = (A, B)
    return out


def _needle(M, x, y, Zp, L, gamma, orders):
    """Barred M/r^n by needle convolution for each n in `orders`
    (dehnen_bar.py:211-241 with _acrn_A_C, 269-278)."""
    nmax = max(orders)
    c1 = M * (1 - gamma) / (2 * L)
    c2 = M * gamma / (L * L)
    u2 = y * y + Zp * Zp
    tp = _acrn_odd(x + L, u2, nmax)
    tm = _acrn_odd(x - L, u2, nmax)
    t0 = _acrn_odd(x, u2, nmax)
    res = {}
    for n in orders:
        Ap, Bp = tp[n]
        Am, Bm = tm[n]
        A0, B0 = t0[n]
        Cp = (x + L) * Ap - Bp
        Cm = (x - L) * Am - Bm
        C0 = x * A0 - B0
        res[n] = c1 * (Ap - Am) + c2 * (Cp + Cm - 2 * C0)
    return res


def t3_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1318-1326."""
    ze = D.sqrt(z * z + b * b)
    Z = ze + a
    aZ = a * Z
    F = _needle(M, x, y, Z, L, gamma, (1, 3, 5))
    ph = F[1]
    ph = ph + a * (Z - a / 3) * F[3]
    ph = ph + aZ ** 2 * F[5]
    return -G * ph


def v4_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1371-1383."""
    ze = D.sqrt(z * z + b * b)
    Z = ze + a
    aZ = a * Z
    hB2 = 0.5 * b * b
    F = _needle(M, x, y, Z, L, gamma, (1, 3, 5, 7, 9))
    ph = F[1]
    ph = ph + (a * (Z - 0.4 * a) + hB2) * F[3]
    ph = ph + 3 * a * (0.2 * aZ * (Z + Z - a) + hB2 * (Z - 0.2 * a)) * F[5]
    ph = ph + aZ ** 2 * (aZ + 6 * hB2) * F[7]
    ph = ph + (7 * hB2 * aZ ** 3 * Z / ze) * F[9]
    return -G * ph


def t3_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1425-1438."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    Z2 = Z * Z
    A2 = a * a
    F = _needle(M, x, y, Z, L, gamma, (5, 7, 9))
    rh = 3 * ze ** 3 * F[5]
    rh = rh + 5 * a * Z2 * ((3 * ze - 2 * a) * ze + A2) * F[7]
    rh = rh + 35 * A2 * Z2 * Z2 * ze * F[9]
    return (b * b * iz ** 3) * (0.25 / math.pi) * rh


def v4_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1526-1543."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    Z2 = Z * Z
    A2 = a * a
    AZ = a * Z
    F = _needle(M, x, y, Z, L, gamma, (7, 9, 11, 13))
    rh = 5 * ze ** 3 * F[7]
    rh = rh + 7 * a * Z2 * (5 * ze * ze - 4 * a * ze + 3 * A2
                            - 2 * a * A2 * iz + A2 * A2 * iz * iz) * F[9]
    rh = rh + 63 * A2 * Z2 * Z2 * (ze + ze - 2 * a + A2 * iz) * F[11]
    rh = rh + 231 * A2 * AZ * Z2 * Z2 * Z * F[13]
    return (b * b * iz ** 3) * (0.375 * b * b / math.pi) * rh


def t1_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1303-1307."""
    Z = D.sqrt(z * z + b * b) + a
    return -G * _needle(M, x, y, Z, L, gamma, (1,))[1]


def t2_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1309-1316."""
    Z = D.sqrt(z * z + b * b) + a
    F = _needle(M, x, y, Z, L, gamma, (1, 3))
    return -G * (F[1] + a * Z * F[3])


def t4_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1328-1337."""
    Z = D.sqrt(z * z + b * b) + a
    aZ = a * Z
    F = _needle(M, x, y, Z, L, gamma, (1, 3, 5, 7))
    ph = F[1] + a * (Z - 0.4 * a) * F[3] + 0.6 * a * aZ * (Z + Z - a) * F[5] + aZ ** 3 * F[7]
    return -G * ph


def v1_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1339-1346."""
    ze = D.sqrt(z * z + b * b)
    Z = ze + a
    hB2 = 0.5 * b * b
    F = _needle(M, x, y, Z, L, gamma, (1, 3))
    return -G * (F[1] + (hB2 * Z / ze) * F[3])


def v2_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1348-1357."""
    ze = D.sqrt(z * z + b * b)
    Z = ze + a
    aZ = a * Z
    hB2 = 0.5 * b * b
    F = _needle(M, x, y, Z, L, gamma, (1, 3, 5))
    return -G * (F[1] + (aZ + hB2) * F[3] + (3 * hB2 * aZ * Z / ze) * F[5])


def v3_phi(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1359-1369."""
    ze = D.sqrt(z * z + b * b)
    Z = ze + a
    aZ = a * Z
    hB2 = 0.5 * b * b
    F = _needle(M, x, y, Z, L, gamma, (1, 3, 5, 7))
    ph = F[1] + (a * (Z - a / 3) + hB2) * F[3] + aZ * (aZ + 3 * hB2) * F[5] + (5 * hB2 * aZ ** 2 * Z / ze) * F[7]
    return -G * ph


def t1_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1399-1409."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    F = _needle(M, x, y, Z, L, gamma, (3, 5))
    return (b * b * iz ** 3) * (0.25 / math.pi) * (a * F[3] + 3 * Z * Z * ze * F[5])


def t2_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1411-1423."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    F = _needle(M, x, y, Z, L, gamma, (5, 7))
    rh = (a * a * a + ze ** 3) * F[5] + 5 * a * Z * Z * Z * ze * F[7]
    return (b * b * iz ** 3) * (0.75 / math.pi) * rh


def t4_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1440-1456."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    Z2, A2, AZ = Z * Z, a * a, a * Z
    F = _needle(M, x, y, Z, L, gamma, (5, 7, 9, 11))
    rh = (3 * F[5] + 15 * AZ * F[7]) * ze ** 3
    rh = rh + 7 * A2 * Z * Z2 * ((6 * ze - 3 * a) * ze + A2) * F[9]
    rh = rh + 63 * A2 * AZ * Z2 * Z2 * ze * F[11]
    return (b * b * iz ** 3) * (0.25 / math.pi) * rh


def v1_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1480-1493."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    F = _needle(M, x, y, Z, L, gamma, (3, 5, 7))
    rh = a * iz * iz * F[3] + 3 * a * Z * iz * F[5] + 5 * Z * Z * Z * F[7]
    return (b * b * iz ** 3) * (0.375 * b * b / math.pi) * rh


def v2_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1495-1508."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    Z2, A2 = Z * Z, a * a
    F = _needle(M, x, y, Z, L, gamma, (5, 7, 9))
    rh = 3 * a * A2 * iz * iz * F[5] + 5 * Z2 * (ze * ze - 2 * a * ze + 3 * A2) * iz * F[7] + 35 * a * Z2 * Z2 * F[9]
    return (b * b * iz ** 3) * (0.375 * b * b / math.pi) * rh


def v3_rho(x, y, z, M, a, b, L, gamma):
    """dehnen_bar.py:1510-1524."""
    ze = D.sqrt(z * z + b * b)
    iz = 1.0 / ze
    Z = ze + a
    Z2, A2, AZ = Z * Z, a * a, a * Z
    F = _needle(M, x, y, Z, L, gamma, (7, 9, 11))
    rh = 3 * ze ** 3 * (1 + (a * iz) ** 5) * F[7]
    rh = rh + 7 * AZ * Z2 * iz * ((3 * ze - 4 * a) * ze + 3 * A2) * F[9]
    rh = rh + 63 * A2 * Z * Z2 * Z2 * F[11]
    return (b * b * iz ** 3) * (0.625 * b * b / math.pi) * rh


DEHNEN_PHI = {1: t1_phi, 2: t2_phi, 3: t3_phi, 4: t4_phi, 11: v1_phi, 12: v2_phi, 13: v3_phi, 14: v4_phi}
DEHNEN_RHO = {1: t1_rho, 2: t2_rho, 3: t3_rho, 4: t4_rho, 11: v1_rho, 12: v2_rho, 13: v3_rho, 14: v4_rho}
DEHNEN_CODES = {"T1": 1, "T2": 2, "T3": 3, "T4": 4, "V1": 11, "V2": 12, "V3": 13, "V4": 14}


# --------------------------------------------------------------------------
# NFW and Miyamoto-Nagai
# --------------------------------------------------------------------------
def nfw_phi(x, y, z, M, Rs, qa=1.0, qb=1.0, qc=1.0):
    """potentials.py:18-27 (identity rotation, zero shift)."""
    r = D.sqrt((x / qa) ** 2 + (y / qb) ** 2 + (z / qc) ** 2 + EPSILON)
    return -G * M * D.log(1 + r / Rs) / (r + EPSILON)


def mn_phi(x, y, z, M, a, b):
    """potentials.py:51-65; the EPSILON offset is added to each coordinate."""
    rx, ry, rz = x + EPSILON, y + EPSILON, z + EPSILON
    R = D.sqrt(rx * rx + ry * ry)
    denom2 = R ** 2 + (a + D.sqrt(rz * rz + b * b)) ** 2
    return -G * M / D.sqrt(denom2)


def mn_rho(x, y, z, M, a, b):
    """potentials.py:29-49."""
    rx, ry, rz = x + EPSILON, y + EPSILON, z + EPSILON
    R = D.sqrt(rx * rx + ry * ry)
    beta = D.sqrt(rz * rz + b * b)
    D2 = R * R + (a + beta) ** 2
    num = a * R * R + (a + 3.0 * beta) * (a + beta) ** 2
    den = beta ** 3 * D2 ** 2.5
    return (b * b * M / (4 * math.pi)) * (num / den)


# --------------------------------------------------------------------------
# Totals
# --------------------------------------------------------------------------
def phi(x, y, z, P):
    """potential_func (likelihood.py:46-71)."""
    p = nfw_phi(x, y, z, P["halo_M"], P["halo_Rs"], P["halo_qa"], P["halo_qb"], P["halo_qc"])
    p = p + mn_phi(x, y, z, P["disc_M"], P["disc_a"], P["disc_b"])
    fb = DEHNEN_PHI[P.get("bar_type", 3) or 3]
    fu = DEHNEN_PHI[P.get("bulge_type", 14) or 14]
    p = p + fb(x, y, z, P["bar_M"], P["bar_a"], P["bar_b"], P["bar_L"], P["bar_gamma"])
    p = p + fu(x, y, z, P["bulge_M"], P["bulge_a"], P["bulge_b"], P["bulge_L"], P["bulge_gamma"])
    return p


def rho(x, y, z, P):
    """density_func (likelihood.py:13-43)."""
    r = mn_rho(x, y, z, P["disc_M"], P["disc_a"], P["disc_b"])
    fb = DEHNEN_RHO[P.get("bar_type", 3) or 3]
    fu = DEHNEN_RHO[P.get("bulge_type", 14) or 14]
    r = r + fb(x, y, z, P["bar_M"], P["bar_a"], P["bar_b"], P["bar_L"], P["bar_gamma"])
    r = r + fu(x, y, z, P["bulge_M"], P["bulge_a"], P["bulge_b"], P["bulge_L"], P["bulge_gamma"])
    return r


def acc(x, y, z, P):
    """-grad Phi (model.py:152-157), exact forward-mode derivative."""
    _, ax, ay, az = phi_acc(x, y, z, P)
    return ax, ay, az


def phi_acc(x, y, z, P):
    """Phi and -grad Phi; P["cylspline"] (get_phi_m's table, optional) adds the
    cylindrical-spline component (oracle/cylspline.py)."""
    X, Y, Zc = D.seed(x, y, z)
    p = phi(X, Y, Zc, P)
    out = (p.v, -p.d[0], -p.d[1], -p.d[2])
    if P.get("cylspline") is not None:
        from . import cylspline
        cp, ca = cylspline.phi_and_acc(x, y, z, P["cylspline"])
        out = (out[0] + cp, out[1] + ca[0], out[2] + ca[1], out[3] + ca[2])
    return out
