"""The cylindrical-spline potential component (CylindricalSpline.py:354-519) on the GPU:
Phi and -grad Phi of a table in get_phi_m's format against the reference's own
evaluate_phi / get_acc (golden vectors), the component added to the canonical model, and
orbits in that potential against the oracle integrator."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def table():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return dict(golden("cylspline"))


def test_cylspline_matches_reference(table):
    from schwarmax_gb300 import cylspline
    g = table
    phi = cylspline.evaluate_phi(g["x"], g["y"], g["z"], g).cpu().numpy()
    acc = cylspline.get_acc(g["x"], g["y"], g["z"], g).cpu().numpy()
    np.testing.assert_allclose(phi, g["phi"], rtol=0, atol=1e-12 * np.abs(g["phi"]).max())
    np.testing.assert_allclose(acc, g["acc"], rtol=0, atol=1e-12 * np.abs(g["acc"]).max())
    # FP32: the same formulas in single precision on the double table
    p32 = cylspline.evaluate_phi(g["x"], g["y"], g["z"], g, dtype=torch.float32).double().cpu().numpy()
    a32 = cylspline.get_acc(g["x"], g["y"], g["z"], g, dtype=torch.float32).double().cpu().numpy()
    np.testing.assert_allclose(p32, g["phi"], rtol=0, atol=2e-6 * np.abs(g["phi"]).max())
    np.testing.assert_allclose(a32, g["acc"], rtol=0, atol=2e-4 * np.abs(g["acc"]).max())


def test_cylspline_adds_to_the_canonical_model(table):
    from oracle import potential as op
    from schwarmax_gb300 import kernels
    from schwarmax_gb300.potentials import potential_struct
    g = table
    pb = dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3, logM_bar=10.0, L_bar=4.0, a_bar=0.8, b_bar=0.3)
    ph = dict(logM=12.0, Rs=20.6)
    pot = potential_struct(pb, ph, cylspline=g)
    x, y, z = (torch.as_tensor(g[k], device="cuda") for k in ("x", "y", "z"))
    out = kernels.potential_eval(pot, x, y, z, want_phi=True, want_acc=True)
    P = op.canonical_params(pb, ph)
    P["cylspline"] = g
    phi, ax, ay, az = op.phi_acc(g["x"], g["y"], g["z"], P)
    np.testing.assert_allclose(out["phi"].cpu().numpy(), phi, rtol=1e-11)
    ref = np.stack([ax, ay, az])
    np.testing.assert_allclose(out["acc"].cpu().numpy(), ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def test_orbits_with_a_cylspline_component_match_oracle(table):
    """Reference-mode orbits (300 attempts, FP64) in NFW + MN + T3 + V4 + the spline
    component against the oracle integrator (identical accepted counts)."""
    from oracle import integrate as oi, potential as op
    from schwarmax_gb300 import kernels as kern
    from schwarmax_gb300._lib import SMX_MODE_REFERENCE, SmxIntegrator
    from schwarmax_gb300.potentials import potential_struct
    g = table
    pb = dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3, logM_bar=10.0, L_bar=4.0, a_bar=0.8, b_bar=0.3)
    ph = dict(logM=12.0, Rs=20.6)
    pot = potential_struct(pb, ph, cylspline=g)
    P = op.canonical_params(pb, ph)
    P["cylspline"] = g
    rng = np.random.default_rng(5)
    n = 12
    R = rng.uniform(1.0, 8.0, n)
    phi0 = rng.uniform(0, 2 * np.pi, n)
    w0 = np.stack([R * np.cos(phi0), R * np.sin(phi0), rng.normal(0, 0.2, n), -200 * np.sin(phi0),
                   200 * np.cos(phi0), rng.normal(0, 20, n)], -1)
    om = -30.0
    cfg = SmxIntegrator(mode=SMX_MODE_REFERENCE, store_all=0, n_attempts=300, n_samples=0, max_attempts=300,
                        atol=1e-7, rtol=1e-4, dt_min=1e-5, dt_max=0.3, omega=om)
    dt0 = np.full(n, 1e-3)
    bufs = kern.IntegratorBuffers(n, 300, torch.float64, torch.device("cuda"))
    kern.integrate(pot, cfg, torch.as_tensor(w0.T.copy(), device="cuda"), torch.as_tensor(dt0, device="cuda"),
                   torch.as_tensor(np.ones(n), device="cuda"), bufs)
    ref = oi.integrate_reference(w0, P, om, 300, dt0, 1e-7, 1e-4, 1e-5, 0.3, store=True)
    nst = bufs.n_stored.cpu().numpy()
    np.testing.assert_array_equal(nst, ref["n_acc"])
    np.testing.assert_allclose(bufs.info.cpu().numpy()[1], ref["EJ0"], rtol=1e-12)
    # the spline sums of the kernel and of NumPy round differently (1e-16), and 300
    # attempts through a barred potential grow that to about 1e-7 of the state
    samples = bufs.samples.cpu().numpy()
    for o in range(n):
        acc = ref["dts"][:, o] > 0
        np.testing.assert_allclose(samples[:6, o, :nst[o]].T, ref["ys"][acc, o], rtol=1e-6, atol=1e-7)
