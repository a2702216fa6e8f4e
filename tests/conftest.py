import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: longer CPU test")


def golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip(f"golden fixture {name}.npz missing")
    return dict(np.load(path, allow_pickle=False))


def params_from_flat(p):
    """Inverse of make_golden.flat_params -> (params_baryon, params_halo)."""
    pb = dict(logM_disc=p[0], Rs_disc=p[1], Hs_disc=p[2], logM_bar=p[3], L_bar=p[4], a_bar=p[5],
              b_bar=p[6], x_origin=0.0, y_origin=0.0, z_origin=0.0, dirx=0.0, diry=0.0, dirz=1.0)
    ph = dict(logM=p[7], Rs=p[8], a=1.0, b=1.0, c=1.0, x_origin=0.0, y_origin=0.0, z_origin=0.0,
              dirx=0.0, diry=0.0, dirz=1.0)
    return pb, ph


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def tiny_dict_data(g):
    """dict_data of the end_to_end golden case, with the reference's draws."""
    dd = {k[3:]: g[k] for k in g if k.startswith("dd_")}
    dd["total_bins"] = int(dd["total_bins"])
    dd["Rzphi_n_tot"] = int(dd["Rzphi_n_tot"])
    dd["jeans_normals"] = g["jeans_normals"]
    dd["jitter_uniforms"] = g["jitter_uniforms"]
    return dd
