"""GB300-native (sm_103a) SchwarMAX model evaluation.

Drop-in entry points of the reference's model-evaluation path:
  build_model, get_model_with_orbit, model_deltaChi2_jackknife   (model.py)
  model_likelihood, calculate_delta_chi2, chi2_func               (likelihood.py)
  model_likelihood_batch: jax.vmap(model_likelihood) over parameter points
  solve_nnls_admm, solve_nnls_admm_bootstrap                      (nnls.py)
  density_func, potential_func (canonical descriptors)
The compute runs in hand-written CUDA kernels behind the C ABI of
include/schwarmax.h (libschwarmax_gb300.so, built in-tree by _lib.build()).
"""
from ._lib import SmxError, build, load  # noqa: F401
from .engine import Settings  # noqa: F401
from .likelihood import (calculate_delta_chi2, chi2_func, model_likelihood, model_likelihood_batch,  # noqa: F401
                         unpack_params)
from .model import build_model, compute_model_single, get_model_with_orbit, model_deltaChi2_jackknife  # noqa: F401
from .nnls import solve_nnls_admm, solve_nnls_admm_bootstrap  # noqa: F401
from .potentials import density_func, potential_func  # noqa: F401

__version__ = "0.1.0"
