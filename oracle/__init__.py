"""FP64 CPU oracle for the SchwarMAX model-evaluation path.

TEST INFRASTRUCTURE ONLY.  This package is a plain NumPy (float64, with a
float32 mode for the integer binning arithmetic) restatement of the
reference's algorithm.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and
only to check results or as the timed CPU baseline.  The product package
``schwarmax_gb300`` never imports it and has no CPU fallback.

Parity pin: the restatement is checked against golden vectors produced by the
reference's own Python modules (``tests/golden/make_golden.py`` imports them
under a NumPy restatement of the JAX primitives they call, since JAX is not
installed).  JAX's own float32 rounding and its threefry random streams are
not reproduced: random draws are explicit inputs everywhere.

Module map (reference file:line in each docstring):
  constants   constants.py:5-11
  dual        forward-mode derivatives standing in for jax.grad (model.py:152-157)
  potential   likelihood.py:13-71, potentials.py:18-65, dehnen_bar.py:104-157,211-278,1318-1543
  grid        utils.py:10-42
  ghmoments   ghmoments.py:6-78
  orbits      utils.py:144-273, model.py:117-148
  jeans       jeans.py:8-93
  integrate   integrates.py:8-313 (chunked library) and 319-570 (trajectory)
  target      model.py:192-213
  nnls        nnls.py:6-166
  model       model.py:14-850
  likelihood  likelihood.py:73-336, utils.py:514-569
"""
