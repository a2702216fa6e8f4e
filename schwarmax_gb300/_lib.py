"""Build and load the C-ABI library ``libschwarmax_gb300.so`` (include/schwarmax.h).

The library is compiled in-tree for sm_103a with nvcc (one object per .cu,
compiled in parallel, then linked with cuBLAS and cuSOLVER).  ``load()``
returns the ctypes handle; every entry point goes through ``call()``, which
raises SmxError with the library's own message when a status is not SMX_OK.
There is no fallback: without the built library and a CUDA device the
package's GPU entry points raise.
"""
import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libschwarmax_gb300.so")
SOURCES = ["api.cu", "pointkernels.cu", "integrate.cu", "project_bin.cu", "soft_project.cu", "nnls.cu", "split_gemm.cu",
           "maps.cu", "analysis.cu", "spd_inverse.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SMX_FP32, SMX_FP64 = 0, 1
SMX_MODE_REFERENCE, SMX_MODE_SAMPLED = 0, 1
SMX_NNLS_FP64, SMX_NNLS_MIXED = 0, 1
INFO_T, INFO_EJ0, INFO_EJ, INFO_WSUM, INFO_NACC, INFO_NATT, INFO_FIELDS = range(7)

EXPORTS = ["smx_version", "smx_kernel_launches", "smx_status_string", "smx_last_error", "smx_potential_eval",
           "smx_initial_conditions", "smx_density_target", "smx_integrate", "smx_integrate_batch", "smx_integrate_noalloc",
           "smx_project_bin", "smx_project_bin_batch",
           "smx_sample_cells", "smx_soft_project", "smx_soft_project_adjoint", "smx_nnls_workspace_size",
           "smx_nnls_admm", "smx_nnls_jackknife_workspace_size", "smx_nnls_jackknife", "smx_split_gemm_workspace_size",
           "smx_split_gemm", "smx_model_maps", "smx_model_maps_workspace_size", "smx_lcirc_table", "smx_spline_eval",
           "smx_circularity", "smx_histogram2d", "smx_psf_transfer_workspace_size", "smx_psf_transfer",
           "smx_rmh_propose", "smx_rmh_accept", "smx_spd_inverse_f32_workspace_size", "smx_spd_inverse_f32",
           "smx_spd_inverse_seed_workspace_size", "smx_spd_inverse_seed"]


class SmxError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"schwarmax status {status}: {message}")
        self.status = status


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "schwarmax.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile the CUDA sources into LIB_PATH (sm_103a).  Returns LIB_PATH."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ----------------------------------------------------------------- structs
class SmxPotential(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "halo_M", "halo_Rs", "halo_qa", "halo_qb", "halo_qc", "disc_M", "disc_a", "disc_b",
        "bar_M", "bar_a", "bar_b", "bar_L", "bar_gamma",
        "bulge_M", "bulge_a", "bulge_b", "bulge_L", "bulge_gamma")] + [
        ("bar_type", ctypes.c_int), ("bulge_type", ctypes.c_int),
        ("cyl_n_r", ctypes.c_int), ("cyl_n_z", ctypes.c_int), ("cyl_n_modes", ctypes.c_int), ("cyl_r0", ctypes.c_double),
        ("cyl_r_grid", ctypes.c_void_p), ("cyl_z_grid", ctypes.c_void_p), ("cyl_coef", ctypes.c_void_p)]


DEHNEN_TYPES = {"T1": 1, "T2": 2, "T3": 3, "T4": 4, "V1": 11, "V2": 12, "V3": 13, "V4": 14}


class SmxPoint(ctypes.Structure):
    _fields_ = [("pot", SmxPotential), ("omega", ctypes.c_double)]


class SmxIntegrator(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("store_all", ctypes.c_int), ("n_attempts", ctypes.c_int),
                ("n_samples", ctypes.c_int), ("max_attempts", ctypes.c_int64), ("atol", ctypes.c_double),
                ("rtol", ctypes.c_double), ("dt_min", ctypes.c_double), ("dt_max", ctypes.c_double),
                ("omega", ctypes.c_double), ("order", ctypes.c_void_p)]


class SmxBinning(ctypes.Structure):
    _fields_ = [("n_part", ctypes.c_int), ("n_real", ctypes.c_int), ("nR", ctypes.c_int), ("nz", ctypes.c_int),
                ("nphi", ctypes.c_int), ("R_lo", ctypes.c_double), ("R_hi", ctypes.c_double),
                ("z_lo", ctypes.c_double), ("z_hi", ctypes.c_double), ("phi_lo", ctypes.c_double),
                ("phi_hi", ctypes.c_double), ("nX", ctypes.c_int), ("nY", ctypes.c_int),
                ("X_lo", ctypes.c_double), ("X_hi", ctypes.c_double), ("Y_lo", ctypes.c_double),
                ("Y_hi", ctypes.c_double), ("n_bins", ctypes.c_int), ("symmetry", ctypes.c_int),
                ("rot", ctypes.c_double * 9)]


class SmxNnlsProblem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("n_rhs", ctypes.c_int64),
                ("ld_lib", ctypes.c_int64), ("lib_precision", ctypes.c_int), ("mode", ctypes.c_int),
                ("maxiter", ctypes.c_int), ("lambda_reg", ctypes.c_double), ("w_init", ctypes.c_double)]


class SmxMapsProblem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("n_rhs", ctypes.c_int64), ("ld_lib", ctypes.c_int64),
                ("lib_precision", ctypes.c_int), ("n_cells", ctypes.c_int), ("n_bins", ctypes.c_int),
                ("lum_factor", ctypes.c_double), ("sigma_amplify", ctypes.c_double)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_SIGS = {
    "smx_version": ([], ctypes.c_int),
    "smx_kernel_launches": ([], ctypes.c_ulonglong),
    "smx_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "smx_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_size_t),
    "smx_potential_eval": ([ctypes.POINTER(SmxPotential), ctypes.c_int, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P],
                           ctypes.c_int),
    "smx_initial_conditions": ([ctypes.POINTER(SmxPotential), ctypes.c_int, _P, _P, _P, _I64, ctypes.c_int,
                                ctypes.c_double, ctypes.c_double, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_density_target": ([ctypes.POINTER(SmxPotential), ctypes.c_int, _P, _P, _P, _I64, ctypes.c_double,
                            ctypes.c_double, ctypes.c_double, _P, ctypes.c_int, _P, _P], ctypes.c_int),
    "smx_integrate": ([ctypes.POINTER(SmxPotential), ctypes.POINTER(SmxIntegrator), ctypes.c_int, _P, _P, _P, _I64,
                       _I64, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_integrate_batch": ([_P, ctypes.c_int, _I64, ctypes.POINTER(SmxIntegrator), ctypes.c_int, _P, _P, _P, _I64,
                             _P, _P, _P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "smx_project_bin_batch": ([ctypes.POINTER(SmxBinning), ctypes.c_int, _P, ctypes.c_int, _P, _P, _I64, _P, _P, _P,
                               _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_integrate_noalloc": ([ctypes.POINTER(SmxPotential), ctypes.POINTER(SmxIntegrator), ctypes.c_int, _P, _P, _P,
                               _I64, _I64, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_project_bin": ([ctypes.POINTER(SmxBinning), ctypes.c_int, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P],
                        ctypes.c_int),
    "smx_sample_cells": ([ctypes.POINTER(SmxBinning), ctypes.c_int, _P, _I64, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_soft_project": ([ctypes.POINTER(SmxBinning), ctypes.c_int, ctypes.c_double, ctypes.c_double, _P, _P,
                          ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_soft_project_adjoint": ([ctypes.POINTER(SmxBinning), ctypes.c_int, ctypes.c_double, ctypes.c_double, _P, _P,
                                  _P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "smx_nnls_workspace_size": ([ctypes.POINTER(SmxNnlsProblem), ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "smx_nnls_admm": ([ctypes.POINTER(SmxNnlsProblem), _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "smx_nnls_jackknife_workspace_size": ([ctypes.POINTER(SmxNnlsProblem), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "smx_nnls_jackknife": ([ctypes.POINTER(SmxNnlsProblem), _P, _P, _P, _P, _P, ctypes.c_int, _P, _P, ctypes.c_size_t,
                            _P], ctypes.c_int),
    "smx_lcirc_table": ([ctypes.POINTER(SmxPotential), ctypes.c_double, ctypes.c_double, ctypes.c_int,
                         ctypes.c_double, _P, _P, _P], ctypes.c_int),
    "smx_spline_eval": ([_P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_double, _P, _I64, _P, _P], ctypes.c_int),
    "smx_circularity": ([ctypes.POINTER(SmxPotential), ctypes.c_int, _P, _I64, _P, _P, ctypes.c_int, ctypes.c_double,
                         ctypes.c_double, _P, _P, _P, _P], ctypes.c_int),
    "smx_histogram2d": ([ctypes.c_int, _P, _P, _P, _I64, _P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_double, _P, _P,
                         _P], ctypes.c_int),
    "smx_psf_transfer_workspace_size": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)],
                                        ctypes.c_int),
    "smx_psf_transfer": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                          ctypes.c_double, ctypes.c_double, _P, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_size_t,
                          _P], ctypes.c_int),
    "smx_rmh_propose": ([_P, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_double, _P, _P, _P], ctypes.c_int),
    "smx_rmh_accept": ([_P, _P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P], ctypes.c_int),
    "smx_spd_inverse_f32_workspace_size": ([_I64, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "smx_spd_inverse_f32": ([_P, _I64, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "smx_spd_inverse_seed_workspace_size": ([_I64, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "smx_spd_inverse_seed": ([_P, _I64, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "smx_split_gemm_workspace_size": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "smx_split_gemm": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                        _P, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "smx_model_maps_workspace_size": ([ctypes.POINTER(SmxMapsProblem), ctypes.POINTER(ctypes.c_size_t)],
                                      ctypes.c_int),
    "smx_model_maps": ([ctypes.POINTER(SmxMapsProblem), _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                        ctypes.c_size_t, _P], ctypes.c_int),
}

_lib = None
_lock = threading.Lock()


def load(path=None):
    """Load the library (building it first if it is missing or stale and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if path is None and _stale():
            build()
        lib = ctypes.CDLL(p)
        for name, (args, res) in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
        return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(2048)
    lib.smx_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def kernel_launches():
    """Kernels launched so far by this process through the library."""
    return int(load().smx_kernel_launches())


def call(name, *args):
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        raise SmxError(st, f"{name}: {last_error()}")
    return st
