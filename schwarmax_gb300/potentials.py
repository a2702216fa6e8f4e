"""The canonical SchwarMAX potential and stellar density, as descriptors.

The reference passes ``density_func`` and ``potential_func`` as Python
callables into jitted code (likelihood.py:13-71).  Callables cannot cross a C
ABI, so this package exposes the canonical pair as descriptor objects: they
are recognised by ``build_model`` and friends, which then run the inline
sm_103a kernels; calling them directly on CUDA tensors evaluates the model
through ``smx_potential_eval``.  Any other callable is rejected with
NotImplementedError.

Model (likelihood.py:10-71): NFW halo (potentials.py:18-27) + Miyamoto-Nagai
disc (potentials.py:29-65) + Dehnen-Aly T3 bar with gamma = 1
(dehnen_bar.py:1318-1326, 1425-1438) + Dehnen-Aly V4 bulge with a = b = 0.5,
L = 0.1, gamma = 0 (dehnen_bar.py:1371-1383, 1526-1543) whose mass is tied to
the bar mass unless ``bulge_mass`` is given.
"""
import torch

from . import _lib, kernels
from ._lib import SmxPotential

V4_A, V4_B, V4_L, V4_GAMMA = 0.5, 0.5, 0.1, 0.0
GAMMA_BAR = 1.0


DEHNEN_TYPES = _lib.DEHNEN_TYPES


def _type_code(t, default):
    if t is None:
        return 0
    if isinstance(t, str):
        if t not in DEHNEN_TYPES:
            raise NotImplementedError(f"Dehnen model {t} is not built (T1-T4, V1-V4)")
        return 0 if DEHNEN_TYPES[t] == default else DEHNEN_TYPES[t]
    return int(t)


class CylSplineTable:
    """A cylindrical-spline potential table (CylindricalSpline.py:270-352, the dictionary
    get_phi_m returns: Rgrid, Zgrid, R0, m, Phi_m_real, Phi_m_img, Mx_real, My_real,
    Mx_img, My_img) in device memory, for the smx_potential fields cyl_*.  The modes must
    be m = 0, 1, .., M in order, as get_phi_m makes them."""

    KEYS = ("Phi_m_real", "Phi_m_img", "Mx_real", "My_real", "Mx_img", "My_img")

    def __init__(self, dict_phi_m):
        import numpy as np
        d = {k: np.asarray(dict_phi_m[k].cpu() if isinstance(dict_phi_m[k], torch.Tensor) else dict_phi_m[k])
             for k in ("Rgrid", "Zgrid", "R0", "m") + self.KEYS}
        m = d["m"].astype(int).reshape(-1)
        if not np.array_equal(m, np.arange(len(m))):
            raise NotImplementedError("cylindrical spline modes must be m = 0, 1, .., M (get_phi_m's order)")
        nr, nz = len(d["Rgrid"]), len(d["Zgrid"])
        coef = np.stack([d[k][:len(m)] for k in self.KEYS], axis=1)          # (modes, 6, nr, nz)
        if coef.shape != (len(m), 6, nr, nz):
            raise ValueError(f"cylindrical spline table of shape {coef.shape}, expected {(len(m), 6, nr, nz)}")
        self.r0 = float(d["R0"].reshape(-1)[0])
        self.r = torch.as_tensor(d["Rgrid"], dtype=torch.float64, device="cuda").contiguous()
        self.z = torch.as_tensor(d["Zgrid"], dtype=torch.float64, device="cuda").contiguous()
        self.coef = torch.as_tensor(coef, dtype=torch.float64, device="cuda").contiguous()
        self.n_modes, self.n_r, self.n_z = len(m), nr, nz

    def attach(self, pot):
        pot.cyl_n_r, pot.cyl_n_z, pot.cyl_n_modes, pot.cyl_r0 = self.n_r, self.n_z, self.n_modes, self.r0
        pot.cyl_r_grid, pot.cyl_z_grid, pot.cyl_coef = self.r.data_ptr(), self.z.data_ptr(), self.coef.data_ptr()
        pot._cyl = self            # keeps the device table alive with the struct
        return pot


def cylspline_only(table):
    """smx_potential holding the cylindrical-spline component alone (the analytic ones
    at zero mass)."""
    pot = SmxPotential(halo_M=0.0, halo_Rs=1.0, halo_qa=1.0, halo_qb=1.0, halo_qc=1.0, disc_M=0.0, disc_a=1.0,
                       disc_b=0.3, bar_M=0.0, bar_a=0.8, bar_b=0.3, bar_L=4.0, bar_gamma=GAMMA_BAR, bulge_M=0.0,
                       bulge_a=V4_A, bulge_b=V4_B, bulge_L=V4_L, bulge_gamma=V4_GAMMA)
    t = table if isinstance(table, CylSplineTable) else CylSplineTable(table)
    return t.attach(pot)


def potential_struct(params_baryon, params_halo, bulge_mass=None, bar_type=None, bulge_type=None, cylspline=None):
    """Reference parameter dicts -> smx_potential.  Shifted or tilted components
    (potentials.py:8-15) are not part of the canonical model.  bar_type / bulge_type
    ("T1".."T4", "V1".."V4", default T3 / V4) choose another Dehnen & Aly model
    (dehnen_bar.py:1272-1555) for either slot.  cylspline (a CylSplineTable or
    get_phi_m's dictionary) adds a cylindrical-spline component to the potential."""
    for p in (params_baryon, params_halo):
        for k in ("x_origin", "y_origin", "z_origin", "dirx", "diry"):
            if k in p and float(p[k]) != 0.0:
                raise NotImplementedError(f"non-canonical component geometry: {k}={float(p[k])}")
        if "dirz" in p and float(p["dirz"]) <= 0.0:
            raise NotImplementedError("the symmetry axis must be +z")
    m_bar = 10.0 ** float(params_baryon["logM_bar"])
    pot = SmxPotential(
        halo_M=10.0 ** float(params_halo["logM"]), halo_Rs=float(params_halo["Rs"]),
        halo_qa=float(params_halo.get("a", 1.0)), halo_qb=float(params_halo.get("b", 1.0)),
        halo_qc=float(params_halo.get("c", 1.0)),
        disc_M=10.0 ** float(params_baryon["logM_disc"]), disc_a=float(params_baryon["Rs_disc"]),
        disc_b=float(params_baryon["Hs_disc"]),
        bar_M=m_bar, bar_a=float(params_baryon["a_bar"]), bar_b=float(params_baryon["b_bar"]),
        bar_L=float(params_baryon["L_bar"]), bar_gamma=GAMMA_BAR,
        bulge_M=m_bar if bulge_mass is None else float(bulge_mass), bulge_a=V4_A, bulge_b=V4_B, bulge_L=V4_L,
        bulge_gamma=V4_GAMMA, bar_type=_type_code(bar_type, 3), bulge_type=_type_code(bulge_type, 14))
    if cylspline is not None:
        (cylspline if isinstance(cylspline, CylSplineTable) else CylSplineTable(cylspline)).attach(pot)
    return pot


class _Canonical:
    kind = None

    def __init__(self, bar_type="T3", bulge_type="V4"):
        self.bar_type, self.bulge_type = bar_type, bulge_type

    @property
    def types(self):
        return dict(bar_type=self.bar_type, bulge_type=self.bulge_type)

    def __repr__(self):
        return f"<schwarmax_gb300 {self.kind} (bar {self.bar_type}, bulge {self.bulge_type})>"


class DensityFunc(_Canonical):
    """density_func(x, y, z, params) -> rho, CUDA tensors in and out."""
    kind = "density_func"

    def __call__(self, x, y, z, params):
        pot = potential_struct(params, dict(logM=0.0, Rs=1.0), **self.types)
        return kernels.potential_eval(pot, x, y, z, want_phi=False, want_acc=False, want_rho=True)["rho"]


class PotentialFunc(_Canonical):
    """potential_func(x, y, z, params_baryon, params_halo) -> Phi, CUDA tensors in and out."""
    kind = "potential_func"

    def __call__(self, x, y, z, params_baryon, params_halo):
        pot = potential_struct(params_baryon, params_halo, **self.types)
        return kernels.potential_eval(pot, x, y, z, want_phi=True, want_acc=False)["phi"]

    def acceleration(self, x, y, z, params_baryon, params_halo):
        """-grad Phi (the reference's acc_fn, model.py:152-157) as a (3, n) tensor."""
        pot = potential_struct(params_baryon, params_halo, **self.types)
        return kernels.potential_eval(pot, x, y, z, want_phi=False, want_acc=True)["acc"]


density_func = DensityFunc()
potential_func = PotentialFunc()


def dehnen_model(bar="T3", bulge="V4"):
    """(density_func, potential_func) of the model NFW + MN + a Dehnen & Aly bar of type
    `bar` + a bulge of type `bulge` (any of T1..T4, V1..V4; the reference builds such
    models from dehnen_bar.py's T*_potential / V*_potential functions).  The pair is
    accepted by build_model, get_model_with_orbit and model_deltaChi2_jackknife like the
    canonical one."""
    for t in (bar, bulge):
        _type_code(t, 0)
    return DensityFunc(bar, bulge), PotentialFunc(bar, bulge)


def model_types(density, potential):
    """bar_type / bulge_type of a descriptor pair (they must agree)."""
    if density is not None and potential is not None and density.types != potential.types:
        raise ValueError("density_func and potential_func describe different Dehnen models")
    d = potential if potential is not None else density
    return d.types if d is not None else {}


def require_canonical(density, potential):
    if density is not None and not isinstance(density, DensityFunc):
        raise NotImplementedError("only the descriptor density_func (MN + Dehnen bar + bulge) has a GB300 kernel")
    if potential is not None and not isinstance(potential, PotentialFunc):
        raise NotImplementedError("only the descriptor potential_func (NFW + MN + Dehnen bar + bulge) has a GB300 "
                                  "kernel")


def as_cuda(x, dtype):
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(x, dtype=dtype, device="cuda").contiguous()
