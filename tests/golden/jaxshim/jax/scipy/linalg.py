import scipy.linalg as _sla


def cho_solve(c_and_lower, b):
    c, lower = c_and_lower
    return _sla.cho_solve((c, lower), b)
