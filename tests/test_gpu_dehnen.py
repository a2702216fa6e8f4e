"""The other Dehnen & Aly models (T1..T4, V1..V4) in the bar and bulge slots of the
device potential: Phi, -grad Phi and rho against the reference's own functions, and an
integration with a non-default model against the oracle."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NAMES = ["T1", "T2", "T3", "T4", "V1", "V2", "V3", "V4"]


@pytest.fixture(scope="module")
def kern():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import kernels
    return kernels


def _slot_pot(slot, name, M, a, b, L, gam):
    from schwarmax_gb300._lib import DEHNEN_TYPES, SmxPotential
    kw = dict(halo_M=0.0, halo_Rs=1.0, halo_qa=1.0, halo_qb=1.0, halo_qc=1.0, disc_M=0.0, disc_a=1.0, disc_b=0.3,
              bar_M=0.0, bar_a=0.8, bar_b=0.3, bar_L=4.0, bar_gamma=1.0, bulge_M=0.0, bulge_a=0.5, bulge_b=0.5,
              bulge_L=0.1, bulge_gamma=0.0)
    kw.update({f"{slot}_M": M, f"{slot}_a": a, f"{slot}_b": b, f"{slot}_L": L, f"{slot}_gamma": gam,
               f"{slot}_type": DEHNEN_TYPES[name]})
    return SmxPotential(**kw)


@pytest.mark.parametrize("slot", ["bar", "bulge"])
@pytest.mark.parametrize("name", NAMES)
def test_dehnen_model_matches_reference(kern, name, slot):
    g = golden("dehnen_types")
    M, a, b, L, gam = (float(v) for v in g[name + "_params"])
    pot = _slot_pot(slot, name, M, a, b, L, gam)
    x, y, z = (torch.as_tensor(g[name + k], device="cuda") for k in ("_x", "_y", "_z"))
    out = kern.potential_eval(pot, x, y, z, want_phi=True, want_acc=True, want_rho=True)
    np.testing.assert_allclose(out["phi"].cpu().numpy(), g[name + "_phi"], rtol=1e-11)
    acc = g[name + "_acc"].T
    np.testing.assert_allclose(out["acc"].cpu().numpy(), acc, rtol=1e-9, atol=1e-10 * np.abs(acc).max())
    rho = g[name + "_rho"]
    np.testing.assert_allclose(out["rho"].cpu().numpy(), rho, rtol=1e-8, atol=1e-11 * np.abs(rho).max())
    # FP32: the same formulas in single precision.  The needle sums alternate in sign
    # (V1 reaches 6e-5 relative at 2 of the 64 points, a cancellation of about 1,000
    # float ulp), so Phi gets 1.5e-4; the forces that drive the orbits keep 2e-3 of |a|.
    o32 = kern.potential_eval(pot, x.float(), y.float(), z.float(), want_phi=True, want_acc=True)
    np.testing.assert_allclose(o32["phi"].double().cpu().numpy(), g[name + "_phi"], rtol=1.5e-4)
    np.testing.assert_allclose(o32["acc"].double().cpu().numpy(), acc, rtol=2e-3, atol=2e-4 * np.abs(acc).max())


def test_orbits_in_a_non_default_model_match_oracle(kern):
    """A T2 bar and a V2 bulge in the full potential: reference-mode orbits (300 attempts)
    of the FP64 kernel against the oracle integrator."""
    from oracle import integrate as oi, potential as op
    from schwarmax_gb300._lib import SMX_MODE_REFERENCE, SmxIntegrator
    from schwarmax_gb300.potentials import potential_struct
    pb = dict(logM_disc=10.7, Rs_disc=3.0, Hs_disc=0.3, logM_bar=10.0, L_bar=4.0, a_bar=0.8, b_bar=0.3)
    ph = dict(logM=12.0, Rs=20.6)
    pot = potential_struct(pb, ph, bar_type="T2", bulge_type="V2")
    P = op.canonical_params(pb, ph)
    P["bar_type"], P["bulge_type"] = 2, 12
    rng = np.random.default_rng(4)
    n = 16
    R = rng.uniform(1.0, 8.0, n)
    phi0 = rng.uniform(0, 2 * np.pi, n)
    w0 = np.stack([R * np.cos(phi0), R * np.sin(phi0), rng.normal(0, 0.2, n), -150 * np.sin(phi0),
                   150 * np.cos(phi0), rng.normal(0, 20, n)], -1)
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
    samples = bufs.samples.cpu().numpy()
    for o in range(n):
        acc = ref["dts"][:, o] > 0
        np.testing.assert_allclose(samples[:6, o, :nst[o]].T, ref["ys"][acc, o], rtol=1e-8, atol=1e-9)
