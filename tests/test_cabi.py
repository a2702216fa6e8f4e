"""The C-ABI library loads and exports every symbol include/schwarmax.h declares (CPU only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "schwarmax.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(smx_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("smx_integrate", "smx_project_bin", "smx_nnls_admm", "smx_model_maps", "smx_initial_conditions",
              "smx_density_target", "smx_potential_eval", "smx_sample_cells"):
        assert n in names


def test_library_exports_declared_symbols():
    from schwarmax_gb300 import _lib
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:   # no nvcc on this machine
        if not os.path.exists(_lib.LIB_PATH):
            pytest.skip(f"library not built: {e}")
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for n in _declared():
        assert hasattr(lib, n), n
    assert set(_lib.EXPORTS) == set(_declared())
    lib.smx_version.restype = ctypes.c_int
    assert lib.smx_version() >= 100
    lib.smx_status_string.restype = ctypes.c_char_p
    lib.smx_status_string.argtypes = [ctypes.c_int]
    assert lib.smx_status_string(0) == b"ok"


def test_argument_errors_without_gpu():
    """Argument validation returns status codes before touching the device."""
    from schwarmax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    pot = _lib.SmxPotential(halo_M=1e12, halo_Rs=20, halo_qa=1, halo_qb=1, halo_qc=1, disc_M=5e10, disc_a=3,
                            disc_b=0.3, bar_M=1e10, bar_a=0.8, bar_b=0.3, bar_L=0.0, bar_gamma=1,
                            bulge_M=1e10, bulge_a=0.5, bulge_b=0.5, bulge_L=0.1, bulge_gamma=0)
    st = lib.smx_potential_eval(ctypes.byref(pot), 0, None, None, None, 10, None, None, None, None, None, None)
    assert st == 2   # L = 0 is the axisymmetric model, not built
    assert "L" in _lib.last_error()
    pot.bar_L = 4.0
    st = lib.smx_potential_eval(ctypes.byref(pot), 0, None, None, None, 10, None, None, None, None, None, None)
    assert st == 1
    st = lib.smx_potential_eval(ctypes.byref(pot), 7, None, None, None, 0, None, None, None, None, None, None)
    assert st == 0   # n = 0 is a no-op
