"""Internal modules of the shim: only what unpickling JAX arrays needs."""
