"""schwarmax_gb300.utils.load_data_bootstrap (utils.py:572-743 without JAX) against
the reference's own loader on the example galaxy of its checkout: 609 Voronoi
apertures on a 60 x 40 pixel map (fixture tests/golden/example_data.npz, made by
tests/golden/make_golden.py).  The pickle's arrays are written back to a pickle here,
read by our loader, and every output of the reference's loader is compared (the
bootstrap draws by their first two rows; the threefry-drawn w0 is not part of it).
The real IFU also checks the grid conventions the binning kernels use."""
import pickle

import numpy as np

from conftest import golden
from oracle import grid as ogrid


def _load(tmp_path):
    g = golden("example_data")
    raw = {k[3:]: g[k] for k in g if k.startswith("in_")}
    with open(tmp_path / "galaxy.pkl", "wb") as f:
        pickle.dump(raw, f)
    from schwarmax_gb300 import utils
    return g, utils.load_data_bootstrap(str(tmp_path) + "/", "galaxy.pkl")


def test_loader_matches_the_reference_loader(tmp_path):
    g, d = _load(tmp_path)
    names = [k[4:] for k in g if k.startswith("out_")]
    assert len(names) > 40
    for name in names:
        ref = np.asarray(g["out_" + name], dtype=np.float64)
        got = np.asarray(d[name], dtype=np.float64)
        if name.endswith("_standard_normal"):
            got = got[:2]
        assert got.shape == ref.shape, name
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, err_msg=name)


def test_example_ifu_conventions(tmp_path):
    _, d = _load(tmp_path)
    nb = int(d["total_bins"])
    bm = np.asarray(d["bin_mapping"])
    nX, nY = (int(v) for v in d["nX_nY"])
    # one entry per pixel plus the sentinel slot that out-of-map samples index
    assert bm.shape == (nX * nY + 1,) and bm[-1] == -1
    assert bm.min() >= -1 and bm.max() == nb - 1
    np.testing.assert_array_equal(np.bincount(bm[:-1][bm[:-1] >= 0], minlength=nb), d["num_per_bin"])
    # pixel centres land on their own pixel index (X fastest), cell centres on their own cell
    lo = np.array([d["X_minmax"][0], d["Y_minmax"][0]])
    hi = np.array([d["X_minmax"][1], d["Y_minmax"][1]])
    XY = np.stack([np.asarray(d["X_regular_grid"], np.float64), np.asarray(d["Y_regular_grid"], np.float64)], -1)
    np.testing.assert_array_equal(ogrid.assign_regular_grid(XY, lo, hi, d["nX_nY"]), np.arange(nX * nY))
    cells = ogrid.assign_regular_grid(np.stack([d["R_grid"], d["z_grid"], d["phi_grid"]], -1),
                                      np.array([d["R_minmax"][0], d["z_minmax"][0], d["phi_minmax"][0]]),
                                      np.array([d["R_minmax"][1], d["z_minmax"][1], d["phi_minmax"][1]]),
                                      d["Rzphi_n_grid"])
    np.testing.assert_array_equal(cells, np.arange(int(d["Rzphi_n_tot"])))
    # bootstrap row 0 is the unperturbed data
    for k in ("XY", "V", "sigma", "h1", "h2", "h3", "h4"):
        assert not np.any(d[k + "_standard_normal"][0])
