"""Cylindrical-spline potential (CylindricalSpline.py), evaluation on the GPU.

``evaluate_phi(x, y, z, dict_phi_m)`` and ``get_acc(x, y, z, params)`` keep the
reference's names and arguments (CylindricalSpline.py:354-387, 489-519): dict_phi_m is
the table get_phi_m builds (CylindricalSpline.py:270-352).  They run the same inline
device code as the integrator (smx_potential_eval with the cyl_* fields of
smx_potential), so a table can also be added to any potential with
``potentials.potential_struct(..., cylspline=dict_phi_m)`` and integrated through."""
import torch

from . import kernels
from .potentials import CylSplineTable, cylspline_only

__all__ = ["CylSplineTable", "evaluate_phi", "get_acc"]


def _xyz(x, y, z, dtype):
    return [(t if isinstance(t, torch.Tensor) else torch.as_tensor(t)).to(device="cuda", dtype=dtype).contiguous()
            .reshape(-1) for t in (x, y, z)]


def evaluate_phi(x, y, z, dict_phi_m, dtype=torch.float64):
    """Phi at the points (CylindricalSpline.py:354-387); 0 outside the table's grid."""
    X, Y, Z = _xyz(x, y, z, dtype)
    return kernels.potential_eval(cylspline_only(dict_phi_m), X, Y, Z, want_phi=True, want_acc=False)["phi"]


def get_acc(x, y, z, params, dtype=torch.float64):
    """-grad Phi as a (3, n) tensor (CylindricalSpline.py:489-519)."""
    X, Y, Z = _xyz(x, y, z, dtype)
    return kernels.potential_eval(cylspline_only(params), X, Y, Z, want_phi=False, want_acc=True)["acc"]
