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
    # every entry point has ctypes argument types (no default int conversion of 64-bit arguments)
    assert set(_lib._SIGS) == set(_lib.EXPORTS)
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


def _geo(**kw):
    from schwarmax_gb300 import _lib
    g = _lib.SmxBinning(n_part=5, n_real=4, nR=4, nz=3, nphi=2, R_lo=0.0, R_hi=10.0, z_lo=-3.0, z_hi=3.0,
                        phi_lo=-3.14159, phi_hi=3.14159, nX=8, nY=8, X_lo=-1.0, X_hi=1.0, Y_lo=-1.0, Y_hi=1.0,
                        n_bins=5, symmetry=1)
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def test_soft_projection_argument_errors_without_gpu():
    """smx_soft_project / _adjoint check sizes, sigma, the velocity scale and their
    buffers before any device call."""
    from schwarmax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    fake = ctypes.c_void_p(256)          # never dereferenced: every case below returns first

    def proj(geo, sigma=0.5, vscale=1.0, bufs=fake):
        return lib.smx_soft_project(geo if geo is None else ctypes.byref(geo), 1, sigma, vscale, bufs, bufs, 10,
                                    bufs, bufs, bufs, bufs, bufs, bufs, bufs, None)

    assert proj(None) == 1
    assert proj(_geo(n_real=9)) == 1                  # realisations 1..8
    assert proj(_geo(nX=0)) == 1
    assert proj(_geo(X_hi=-1.0)) == 1                 # empty sky grid
    assert proj(_geo(), sigma=0.01) == 1              # window of +-3 pixels needs sigma in [0.05, 1]
    assert proj(_geo(), sigma=1.5) == 1
    assert proj(_geo(), vscale=0.0) == 1
    assert "velocity scale" in _lib.last_error()
    assert proj(_geo(n_part=0)) == 0                  # nothing to do
    assert proj(_geo(), bufs=None) == 1               # buffers missing
    assert lib.smx_soft_project(ctypes.byref(_geo()), 9, 0.5, 1.0, fake, fake, 10, fake, fake, fake, fake, fake,
                                fake, fake, None) == 1     # precision
    drot = (ctypes.c_double * 27)()
    grad = fake

    def adj(geo, d=drot, g=grad):
        return lib.smx_soft_project_adjoint(ctypes.byref(geo), 1, 0.5, 1.0, d, fake, fake, 10, fake, fake, fake,
                                            fake, fake, fake, fake, g, None)

    assert adj(_geo(), d=None) == 1
    assert adj(_geo(), g=None) == 1
    assert adj(_geo(n_part=0)) == 0


def test_split_product_argument_errors_without_gpu():
    from schwarmax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    nbytes = ctypes.c_size_t(0)
    assert lib.smx_split_gemm_workspace_size(300, 100, 1000, 4, 5, ctypes.byref(nbytes)) == 0
    need = nbytes.value
    assert need >= 300 * 100 * 12                    # int64 + float accumulator per output at least
    assert lib.smx_split_gemm_workspace_size(0, 100, 1000, 4, 5, ctypes.byref(nbytes)) == 1
    assert lib.smx_split_gemm_workspace_size(300, 100, 1000, 4, 5, None) == 1
    assert lib.smx_split_gemm_workspace_size(300, 100, 1000, 3, 3, ctypes.byref(nbytes)) == 2   # no 3-slice kernel
    assert lib.smx_split_gemm_workspace_size(300, 200, 1000, 4, 5, ctypes.byref(nbytes)) == 2   # 4 x 5 needs N <= 112
    fake = ctypes.c_void_p(256)
    assert lib.smx_split_gemm(300, 100, 1000, 4, 5, 0, fake, fake, fake, fake, need - 1, None) == 6   # workspace
    assert lib.smx_split_gemm(300, 100, 1000, 4, 5, 0, None, fake, fake, fake, need, None) == 1
    assert lib.smx_split_gemm(300, 200, 1000, 4, 4, 1, fake, fake, fake, fake, 1 << 40, None) == 1    # lower: M == N
    assert lib.smx_split_gemm(1 << 17, 1 << 15, 64, 4, 4, 0, fake, fake, fake, fake, 1 << 40, None) == 2  # too large


def test_seed_inverse_argument_errors_without_gpu():
    from schwarmax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    nbytes = ctypes.c_size_t(0)
    assert lib.smx_spd_inverse_seed_workspace_size(6608, ctypes.byref(nbytes)) == 0
    assert nbytes.value > 6608 * 6608 * (8 + 8 + 4)    # accumulators and the scratch block at least
    assert lib.smx_spd_inverse_seed_workspace_size(12000, ctypes.byref(nbytes)) == 0
    need = nbytes.value
    assert need > 2 ** 32                               # passed as a size_t, not an int
    assert lib.smx_spd_inverse_seed_workspace_size(0, ctypes.byref(nbytes)) == 1
    assert lib.smx_spd_inverse_seed_workspace_size(100, None) == 1
    fake = ctypes.c_void_p(256)
    assert lib.smx_spd_inverse_seed(fake, 12000, fake, fake, need - 1, None) == 6   # workspace too small
    assert lib.smx_spd_inverse_seed(None, 12000, fake, fake, need, None) == 1
    assert lib.smx_spd_inverse_seed(fake, 0, fake, fake, need, None) == 1


def test_nnls_argument_errors_without_gpu():
    """smx_nnls_admm checks the problem and its buffers before creating any handle."""
    from schwarmax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    fake = ctypes.c_void_p(256)

    def prob(**kw):
        p = _lib.SmxNnlsProblem(n=100, m=60, n_rhs=4, ld_lib=80, lib_precision=_lib.SMX_FP32,
                                mode=_lib.SMX_NNLS_MIXED, maxiter=10, lambda_reg=1.0, w_init=0.1)
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def run(p, bufs=fake):
        return lib.smx_nnls_admm(None if p is None else ctypes.byref(p), bufs, bufs, bufs, bufs, bufs, bufs, 1 << 40,
                                 None)

    assert run(None) == 1
    assert run(prob(n=0)) == 1
    assert run(prob(n_rhs=0)) == 1
    assert run(prob(maxiter=-1)) == 1
    assert run(prob(m=50000)) == 2                    # G = c I + U U^T would exceed 2^31 entries
    assert run(prob(mode=7)) == 1
    assert run(prob(), bufs=None) == 1
    assert run(prob(lambda_reg=-1.0)) == 1
    nbytes = ctypes.c_size_t(0)
    assert lib.smx_nnls_workspace_size(None, ctypes.byref(nbytes)) == 1
    assert lib.smx_nnls_workspace_size(ctypes.byref(prob(m=0)), ctypes.byref(nbytes)) == 1
