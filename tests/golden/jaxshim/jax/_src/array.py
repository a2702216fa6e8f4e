"""Unpickling of JAX arrays without JAX.  A pickled jax.Array is reduced to
``_reconstruct_array(fun, args, state, aval)`` whose ``fun(*args)`` builds a NumPy
array and ``state`` is that array's own pickle state, so the NumPy array is the
value."""


def _reconstruct_array(fun, args, state, aval=None):
    a = fun(*args)
    a.__setstate__(state)
    return a
