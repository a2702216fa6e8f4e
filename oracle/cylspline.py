"""Test infrastructure (the oracle): FP64 NumPy restatement of the cylindrical-spline
potential of the reference, evaluation only.

* second_derivatives:  not-a-knot cubic-spline second derivatives
                        (CubicSpline.py:5-52)
* precompute_splines:  M_x along the first grid axis for every column, M_y along the
                        second for every row (CubicSpline.py:55-97)
* spline_with_derivs:  the separable bicubic value and its two first derivatives,
                        0 outside the grid (CubicSpline.py:202-305)
* phi_and_acc:         Phi = sum_m f_m (Re Phi_m cos m phi - Im Phi_m sin m phi),
                        f_0 = 1, f_m = 2, on (asinh(R/R0), asinh(|z|/R0)), and
                        -grad Phi by the chain rule of get_acc
                        (CylindricalSpline.py:418-519)

The table follows get_phi_m's dictionary (CylindricalSpline.py:340-350): Rgrid, Zgrid
(scaled), R0, m = 0..M, and (M+1, NR, NZ) arrays Phi_m_real, Phi_m_img, Mx_real, My_real,
Mx_img, My_img."""
import numpy as np


def second_derivatives(x, y):
    """CubicSpline.py:5-52: the tridiagonal system with not-a-knot end rows."""
    n = len(x)
    h = np.diff(x)
    A = np.zeros((n, n))
    b = np.zeros(n)
    A[0, 0], A[0, 1], A[0, 2] = h[1], -(h[0] + h[1]), h[0]
    for i in range(1, n - 1):
        A[i, i - 1], A[i, i], A[i, i + 1] = h[i - 1], 2.0 * (h[i - 1] + h[i]), h[i]
        b[i] = 6.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    A[n - 1, n - 3], A[n - 1, n - 2], A[n - 1, n - 1] = h[n - 2], -(h[n - 3] + h[n - 2]), h[n - 3]
    return np.linalg.solve(A, b)


def precompute_splines(gx, gy, values):
    """CubicSpline.py:55-97."""
    nx, ny = values.shape
    Mx = np.zeros((nx, ny))
    My = np.zeros((nx, ny))
    for j in range(ny):
        Mx[:, j] = second_derivatives(gx, values[:, j])
    for i in range(nx):
        My[i, :] = second_derivatives(gy, values[i, :])
    return Mx, My


def spline_with_derivs(px, py, gx, gy, v, Mx, My):
    """CubicSpline.py:202-305 (fill value 0 outside the grid, derivatives 0 there)."""
    px, py = np.asarray(px, np.float64), np.asarray(py, np.float64)
    out = (px < gx[0]) | (px > gx[-1]) | (py < gy[0]) | (py > gy[-1])
    px = np.clip(px, gx[0], gx[-1])
    py = np.clip(py, gy[0], gy[-1])
    ix = np.clip(np.searchsorted(gx, px) - 1, 0, len(gx) - 2)
    iy = np.clip(np.searchsorted(gy, py) - 1, 0, len(gy) - 2)
    hx = gx[ix + 1] - gx[ix]
    hy = gy[iy + 1] - gy[iy]
    tx = (px - gx[ix]) / hx
    ty = (py - gy[iy]) / hy
    ux, uy = 1.0 - tx, 1.0 - ty
    z00, z10, z01, z11 = v[ix, iy], v[ix + 1, iy], v[ix, iy + 1], v[ix + 1, iy + 1]
    a00, a10, a01, a11 = Mx[ix, iy], Mx[ix + 1, iy], Mx[ix, iy + 1], Mx[ix + 1, iy + 1]
    b00, b10, b01, b11 = My[ix, iy], My[ix + 1, iy], My[ix, iy + 1], My[ix + 1, iy + 1]
    cx = hx ** 2 / 6.0
    cy = hy ** 2 / 6.0
    f0 = ux * z00 + tx * z10 + ((ux ** 3 - ux) * a00 + (tx ** 3 - tx) * a10) * cx
    f1 = ux * z01 + tx * z11 + ((ux ** 3 - ux) * a01 + (tx ** 3 - tx) * a11) * cx
    df0 = (z10 - z00) + ((-3.0 * ux ** 2 + 1.0) * a00 + (3.0 * tx ** 2 - 1.0) * a10) * cx
    df1 = (z11 - z01) + ((-3.0 * ux ** 2 + 1.0) * a01 + (3.0 * tx ** 2 - 1.0) * a11) * cx
    m0 = ux * b00 + tx * b10
    m1 = ux * b01 + tx * b11
    value = uy * f0 + ty * f1 + ((uy ** 3 - uy) * m0 + (ty ** 3 - ty) * m1) * cy
    dvx = (uy * df0 + ty * df1 + ((uy ** 3 - uy) * (b10 - b00) + (ty ** 3 - ty) * (b11 - b01)) * cy) / hx
    dvy = ((f1 - f0) + ((-3.0 * uy ** 2 + 1.0) * m0 + (3.0 * ty ** 2 - 1.0) * m1) * cy) / hy
    return np.where(out, 0.0, value), np.where(out, 0.0, dvx), np.where(out, 0.0, dvy)


def phi_and_acc(x, y, z, t):
    """Phi and -grad Phi (CylindricalSpline.py:418-519) at arrays x, y, z for table t."""
    x, y, z = (np.asarray(a, np.float64) for a in (x, y, z))
    R = np.sqrt(x * x + y * y)
    ph = np.arctan2(y, x)
    za = np.abs(z)
    R0 = float(np.asarray(t["R0"]).reshape(-1)[0])
    Rs, zs = np.arcsinh(R / R0), np.arcsinh(za / R0)
    phi = np.zeros_like(R)
    dR = np.zeros_like(R)
    dz = np.zeros_like(R)
    dph = np.zeros_like(R)
    for m in np.asarray(t["m"]).astype(int):
        re, dre_R, dre_z = spline_with_derivs(Rs, zs, t["Rgrid"], t["Zgrid"], t["Phi_m_real"][m], t["Mx_real"][m],
                                              t["My_real"][m])
        im, dim_R, dim_z = spline_with_derivs(Rs, zs, t["Rgrid"], t["Zgrid"], t["Phi_m_img"][m], t["Mx_img"][m],
                                              t["My_img"][m])
        c, s = np.cos(m * ph), np.sin(m * ph)
        f = 1.0 if m == 0 else 2.0
        phi += f * (re * c - im * s)
        dR += f * (dre_R * c - dim_R * s)
        dz += f * (dre_z * c - dim_z * s)
        dph += f * (-m * re * s - m * im * c)
    dphi_dR = dR / np.sqrt(R * R + R0 * R0)
    dphi_dz = dz / np.sqrt(za * za + R0 * R0) * np.sign(z)
    ok = R > 1e-12
    with np.errstate(divide="ignore", invalid="ignore"):
        invR = np.where(ok, 1.0 / np.where(ok, R, 1.0), 0.0)
    gx = dphi_dR * np.where(ok, x * invR, 0.0) + dph * np.where(ok, -y * invR * invR, 0.0)
    gy = dphi_dR * np.where(ok, y * invR, 0.0) + dph * np.where(ok, x * invR * invR, 0.0)
    return phi, -np.stack([gx, gy, dphi_dz])
