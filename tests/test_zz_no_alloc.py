"""smx_integrate_noalloc: the integrator entry point for callers that cannot
allocate device memory (its work counter lives in a static device array of the
library).  Its output must equal smx_integrate's on the same inputs, on two
calls in a row (the shared counter is re-zeroed by every call).  Collected last
on purpose: it runs after every other GPU test, and also passes alone."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _inputs(n, dtype):
    rng = np.random.default_rng(21)
    R = rng.uniform(1.0, 7.0, n)
    th = rng.uniform(0, 2 * np.pi, n)
    vc = 200.0
    w = np.stack([R * np.cos(th), R * np.sin(th), rng.normal(0, 0.2, n), vc * np.sin(th) * 0.9,
                  -vc * np.cos(th) * 0.9, rng.normal(0, 15, n)])
    To = 2 * np.pi * R / vc
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")  # noqa: E731
    return dev(w), dev(To / 100), dev(To * 2)


def _outputs(n, slots, dtype):
    return dict(samples=torch.full((7, n, slots), float("nan"), dtype=dtype, device="cuda"),
                n_stored=torch.full((n,), -1, dtype=torch.int32, device="cuda"),
                info=torch.full((6, n), float("nan"), dtype=dtype, device="cuda"),
                status=torch.full((n,), -1, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("mode,dtype", [(1, torch.float32), (0, torch.float64)])
def test_noalloc_integrator_matches_allocating_entry_point(mode, dtype):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import _lib
    from schwarmax_gb300.potentials import potential_struct
    lib = _lib.load()
    pot = potential_struct(dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3, logM_bar=10.0, L_bar=4.0, a_bar=0.8,
                                b_bar=0.3), dict(logM=12.0, Rs=20.6))
    n, slots = 777, 64
    cfg = _lib.SmxIntegrator(mode=mode, store_all=0, n_attempts=slots, n_samples=slots, max_attempts=50000,
                             atol=1e-7, rtol=1e-5, dt_min=1e-5, dt_max=0.3, omega=-35.79)
    prec = _lib.SMX_FP32 if dtype == torch.float32 else _lib.SMX_FP64
    w0, dt0, tt = _inputs(n, dtype)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = _outputs(n, slots, dtype)
    queue = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("smx_integrate", ctypes.byref(pot), ctypes.byref(cfg), prec, P(w0), P(dt0), P(tt), n, slots,
              P(ref["samples"]), P(ref["n_stored"]), P(ref["info"]), P(ref["status"]), P(queue), stream)
    fn = lib.smx_integrate_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_lib.SmxPotential), ctypes.POINTER(_lib.SmxIntegrator), ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for call in range(2):
        out = _outputs(n, slots, dtype)
        st = fn(ctypes.byref(pot), ctypes.byref(cfg), prec, P(w0), P(dt0), P(tt), n, slots, P(out["samples"]),
                P(out["n_stored"]), P(out["info"]), P(out["status"]), stream)
        assert st == 0, _lib.last_error()
        torch.cuda.synchronize()
        ns = ref["n_stored"].cpu().numpy()
        np.testing.assert_array_equal(out["n_stored"].cpu().numpy(), ns)
        np.testing.assert_array_equal(out["status"].cpu().numpy(), ref["status"].cpu().numpy())
        np.testing.assert_allclose(out["info"].cpu().numpy(), ref["info"].cpu().numpy(), rtol=0, atol=0)
        a, b = out["samples"].cpu().numpy(), ref["samples"].cpu().numpy()
        for o in range(n):
            np.testing.assert_allclose(a[:, o, :ns[o]], b[:, o, :ns[o]], rtol=0, atol=0)


def test_noalloc_rejects_sizes_beyond_its_counter():
    from schwarmax_gb300 import _lib
    from schwarmax_gb300.potentials import potential_struct
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    pot = potential_struct(dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3, logM_bar=10.0, L_bar=4.0, a_bar=0.8,
                                b_bar=0.3), dict(logM=12.0, Rs=20.6))
    cfg = _lib.SmxIntegrator(mode=0, store_all=0, n_attempts=10, n_samples=0, max_attempts=0, atol=1e-7,
                             rtol=1e-5, dt_min=1e-5, dt_max=0.3, omega=0.0)
    fn = lib.smx_integrate_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_lib.SmxPotential), ctypes.POINTER(_lib.SmxIntegrator), ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    st = fn(ctypes.byref(pot), ctypes.byref(cfg), 0, None, None, None, 1 << 31, 10, None, None, None, None, None)
    assert st == 2 and "limit" in _lib.last_error()
