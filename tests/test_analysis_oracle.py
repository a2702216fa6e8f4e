"""Post-analysis on the CPU: the oracle restatement and the package's host-side
spline against the reference's own build_Lcirc_of_E and compute_transfer_matrix
(golden vectors from tests/golden/make_golden.py, case 'analysis')."""
import numpy as np
import pytest

from conftest import golden, params_from_flat


def test_oracle_lcirc_matches_reference():
    from oracle import analysis as oa, potential as op
    g = golden("analysis")
    pb, ph = params_from_flat(g["params"])
    interp, E, L = oa.build_Lcirc_of_E(op.canonical_params(pb, ph), n_grid=400)
    # the central difference with dR = 1e-3 amplifies rounding of Phi (|Phi| eps / dR)
    np.testing.assert_allclose(E, g["E_circ"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(L, g["L_circ"], rtol=1e-9, atol=1e-12 * np.abs(g["L_circ"]).max())
    np.testing.assert_allclose(interp(g["E_query"]), g["L_query"], rtol=1e-10, atol=1e-10 * np.abs(g["L_query"]).max())


def test_oracle_transfer_matrix_matches_reference():
    from oracle import analysis as oa
    g = golden("analysis")
    d = golden("example_data")
    nX, nY = (int(v) for v in d["out_nX_nY"])
    P = oa.compute_transfer_matrix(float(g["psf_sigma"]), nX, nY, d["out_X_minmax"], d["out_Y_minmax"],
                                   d["out_bin_mapping"], int(d["out_total_bins"]), grid_res=int(g["psf_grid_res"]))
    np.testing.assert_allclose(P, g["psf_P"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(P.sum(axis=0)[P.sum(axis=0) > 0], 1.0, rtol=1e-12)


@pytest.mark.parametrize("n", [4, 7, 400])
def test_not_a_knot_spline_is_interp1d_cubic(n):
    """The host-side spline of schwarmax_gb300.analysis against scipy's interp1d(kind='cubic')."""
    from scipy.interpolate import interp1d

    from schwarmax_gb300.analysis import not_a_knot_spline
    g = golden("analysis")
    rng = np.random.default_rng(n)
    if n == 400:
        x, y = g["E_circ"], g["L_circ"]
    else:
        x = np.sort(rng.uniform(-3, 5, n))
        y = rng.normal(size=n)
    c = not_a_knot_spline(x, y)
    q = np.sort(rng.uniform(x[0], x[-1], 500))
    j = np.clip(np.searchsorted(x, q, side="right") - 1, 0, x.size - 2)
    t = q - x[j]
    mine = ((c[0, j] * t + c[1, j]) * t + c[2, j]) * t + c[3, j]
    ref = interp1d(x, y, kind="cubic")(q)
    np.testing.assert_allclose(mine, ref, rtol=1e-9, atol=1e-9 * np.abs(y).max())
