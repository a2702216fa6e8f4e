"""Autotuner of the batched evaluation's launch choices, with a JSON cache.

The integrator is one persistent launch over a work queue, so its speed depends on how
many blocks share an SM (registers and latency hiding against the tail of the queue)
and on the order in which the queue hands out orbits (orbits sorted by cost keep the
lanes of a warp busy for similar times).  ``tune_integrator`` times the candidates on a
short horizon of the actual batch (a fraction of every orbit's integration time, so the
relative cost of the orbits is that of the real run) and returns the fastest; the
choice is stored per (device, orbit count, sample count, tolerance) in
``$SCHWARMAX_AUTOTUNE`` (default ``~/.cache/schwarmax_gb300/autotune.json``).  No
result depends on the choice.
"""
import json
import os
import time

import torch

from . import kernels
from ._lib import INFO_NATT, SMX_MODE_SAMPLED, SmxIntegrator

CACHE = os.environ.get("SCHWARMAX_AUTOTUNE", os.path.join(os.path.expanduser("~"), ".cache", "schwarmax_gb300",
                                                            "autotune.json"))


def _key(n_orb, n_samples, rtol):
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|orbits={n_orb}|samples={n_samples}|rtol={rtol:g}"


def load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save(cache):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def lookup(n_orb, n_samples, rtol):
    return load().get(_key(n_orb, n_samples, rtol))


def tune_integrator(points, n_points, per_point, w0, dt_init, t_total, st, horizon=0.04, candidates=(0, 3, 2, 1),
                    repeats=2):
    """Times smx_integrate_batch on `horizon` of every orbit's integration time for each
    blocks-per-SM cap in `candidates` (0 = as many as fit), with the natural queue order
    and with the orbits sorted by the cost of the first candidate's run (longest first).
    Returns the best {"blocks_per_sm", "order", "ms"} and stores it in the cache."""
    n_orb = w0.shape[1]
    ns = max(1, int(round(st.n_samples * horizon)))
    tt = (t_total * horizon).contiguous()
    bufs = kernels.IntegratorBuffers(n_orb, ns, w0.dtype, w0.device)
    cfg = SmxIntegrator(mode=SMX_MODE_SAMPLED, store_all=0, n_attempts=0, n_samples=ns,
                        max_attempts=max(1, int(st.max_attempts * horizon)), atol=st.atol, rtol=st.rtol,
                        dt_min=st.dt_min, dt_max=st.dt_max, omega=0.0)

    def run(bps, order):
        cfg.order = 0 if order is None else order.data_ptr()
        best = float("inf")
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            kernels.integrate_batch(points, n_points, per_point, cfg, w0, dt_init, tt, bufs, bps)
            torch.cuda.synchronize()
            best = min(best, (time.perf_counter() - t0) * 1e3)
        return best

    results = []
    for bps in candidates:
        results.append({"blocks_per_sm": bps, "order": "natural", "ms": run(bps, None)})
    cost = bufs.info[INFO_NATT]
    order = torch.argsort(cost, descending=True).to(torch.int32).contiguous()
    for bps in candidates:
        results.append({"blocks_per_sm": bps, "order": "cost", "ms": run(bps, order)})
    best = min(results, key=lambda r: r["ms"])
    cache = load()
    cache[_key(n_orb, st.n_samples, st.rtol)] = dict(best, candidates=results, horizon=horizon)
    save(cache)
    return best


def cost_order(points, n_points, per_point, w0, dt_init, t_total, st, horizon=0.02):
    """Queue order of a batch, longest first, from a probe over `horizon` of every
    orbit's integration time."""
    n_orb = w0.shape[1]
    ns = max(1, int(round(st.n_samples * horizon)))
    bufs = kernels.IntegratorBuffers(n_orb, ns, w0.dtype, w0.device)
    cfg = SmxIntegrator(mode=SMX_MODE_SAMPLED, store_all=0, n_attempts=0, n_samples=ns,
                        max_attempts=max(1, int(st.max_attempts * horizon)), atol=st.atol, rtol=st.rtol,
                        dt_min=st.dt_min, dt_max=st.dt_max, omega=0.0)
    kernels.integrate_batch(points, n_points, per_point, cfg, w0, dt_init, (t_total * horizon).contiguous(), bufs)
    return torch.argsort(bufs.info[INFO_NATT], descending=True).to(torch.int32).contiguous()
