import numpy as _np


def _stack(outs):
    first = outs[0]
    if first is None:
        return None
    if isinstance(first, dict):
        return {k: _stack([o[k] for o in outs]) for k in first}
    if isinstance(first, (tuple, list)):
        return type(first)(_stack([o[i] for o in outs]) for i in range(len(first)))
    return _np.stack([_np.asarray(o) for o in outs])


def _slice(xs, i):
    if xs is None:
        return None
    if isinstance(xs, (tuple, list)):
        return type(xs)(_slice(x, i) for x in xs)
    if isinstance(xs, dict):
        return {k: _slice(v, i) for k, v in xs.items()}
    return _np.asarray(xs)[i]


def _len(xs):
    if isinstance(xs, (tuple, list)):
        return _len(xs[0])
    if isinstance(xs, dict):
        return _len(next(iter(xs.values())))
    return _np.asarray(xs).shape[0]


def scan(f, init, xs=None, length=None):
    n = length if length is not None else _len(xs)
    carry = init
    ys = []
    for i in range(n):
        carry, y = f(carry, _slice(xs, i))
        ys.append(y)
    return carry, (_stack(ys) if ys else None)


def map(f, xs):
    return _stack([f(_slice(xs, i)) for i in range(_len(xs))])


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def switch(index, branches, *operands):
    return branches[int(index)](*operands)


def stop_gradient(x):
    return x


def fori_loop(lower, upper, body_fun, init_val):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val
