#!/usr/bin/env python
"""Model evaluations per second on one GB300.

Default (config 2, the batched workload): one step = one batch of 64 parameter
points, each a full model evaluation (model_likelihood_batch): Jeans ICs ->
16,384 particles x 4 jitter realisations integrated for 50 circular periods
(adaptive BS23, rtol 1e-6, 1,000 uniform-time samples each) -> projection and
binning into an 80x80-pixel / 400-aperture IFU and a 24x16x12 (R, z, phi)
grid -> 3-D density target -> 100 bootstrap ADMM NNLS solves (200 iterations)
-> model maps -> chi^2 -> log-mean-exp.  --config 1, 4 or small: one evaluation
of that configuration per step (model_likelihood).  Inputs are seeded synthetic
data (schwarmax_gb300.synthetic); working sets are larger than L2 (the sample
store of one evaluation alone is 1.8 GB), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 1|2|4|small]

--impl reference times the CPU restatement of the same evaluation (oracle/,
all host cores) on a bounded sample of the workload and scales it to evals/s.
Multi-GPU runs are independent replicas (one evaluation stream per GPU).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "model evals/sec at Δχ²≤0.1, batched mixed-precision vs plain FP64, 1 GB300"
UNIT = "evals/s"


def workload(cfg):
    """One evaluation of a configuration, in words."""
    nR, nz, nphi = cfg.n_grid
    return (f"{cfg.name}: {cfg.n_part:,} particles x {cfg.n_real} realisations, {cfg.n_periods:g} circular periods, "
            f"rtol {cfg.rtol:g}, {cfg.n_samples:,} uniform-time samples per orbit, {cfg.n_pix}x{cfg.n_pix} px / "
            f"{cfg.n_bins:,} Voronoi apertures, {nR}x{nz}x{nphi} Rzphi grid, {cfg.n_boot} bootstrap ADMM NNLS "
            f"({cfg.admm_iters} iterations)")


WORKLOAD_BATCH = ("config2: {P} parameter points per batch (potential within +-20% of config 1, Omega_p in "
                  "[25, 45] km/s/kpc), each 16,384 particles x 4 realisations, 50 circular periods, rtol 1e-6, "
                  "1,000 uniform-time samples per orbit, 80x80 px / 400 Voronoi apertures, 24x16x12 Rzphi grid, "
                  "100 bootstrap ADMM NNLS (200 iterations){jk}; one integrator launch over all points' orbits")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, device=None):
    """The slowest rank's timed milliseconds (the job ends with its slowest replica);
    ms itself when there is one process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, steps, ms):
    """Evaluations per second of all replicas together: world x steps in the slowest rank's time."""
    return world * steps / (ms / 1e3)


def clock_sampler(path):
    try:
        return subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"], stdout=open(path, "w"), stderr=subprocess.DEVNULL)
    except FileNotFoundError:
        return None


def clock_summary(path, gpu_index):
    rows = []
    try:
        for line in open(path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9 and f[0] == str(gpu_index):
                rows.append(f)
    except OSError:
        return None
    if not rows:
        return None
    sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
    reasons = set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for r in rows:
        for nm, v in zip(names, r[5:9]):
            if v.strip().lower() in ("active", "yes", "1"):
                reasons.add(nm)
    return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": float(rows[0][2]) if rows else None,
            "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


# FP32 operations of one canonical force evaluation (gradient of NFW + MN +
# T3 needle (3 positions, orders 1-7) + V4 needle (2 positions, orders 1-11))
# and of one BS23 attempt outside the three force calls (stage inputs, frame
# terms, error norm, step control, amortised dense output), counted from the
# kernel source with add/sub/mul = 1, FMA = 2 and each sqrt/rsqrt/rcp/log/
# log1p/cbrt call = 1.
FLOPS_PER_FORCE = 462
FLOPS_PER_STEP = 192


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import schwarmax_gb300 as smx
    from schwarmax_gb300 import _lib, engine, synthetic
    from schwarmax_gb300.likelihood import grid_of, log_likelihoods, log_mean_exp, unpack_params

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg = synthetic.CONFIGS[args.config]
    t0 = time.time()
    dict_data, theta = synthetic.make_dataset(cfg, seed=args.seed)
    setup_s = time.time() - t0
    st = cfg.settings("mixed")
    st.bootstrap = args.bootstrap
    dd = engine.DeviceData(dict_data, n_real=st.n_real)
    nb = cfg.n_bins
    nc = cfg.n_grid[0] * cfg.n_grid[1] * cfg.n_grid[2]
    kw = dict(settings=st, nnls_maxiter=cfg.admm_iters)

    def step(i, timers=None):
        th = theta.copy()
        th[10] = theta[10] + 0.002 * ((i % 5) - 2)          # M/L walk, MCMC-like
        logl, r = log_likelihoods(th, dd, nb, nc, **kw)
        return log_mean_exp(logl), r

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    # --- device-resident throughput -------------------------------------------------
    sampler = clock_sampler(os.path.join(args.out, f"clocks_rank{rank}.csv")) if rank == 0 else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for i in range(args.steps):
        val, r = step(i)
    ev1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches = _lib.kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev)
    if sampler:
        sampler.terminate()
    value = whole_job_rate(world, args.steps, ms)
    # --- per-stage device time of one evaluation (outside the timed region) ---------
    stages = stage_breakdown(lambda: step(0))
    # --- integrator kernel alone, for the roofline ----------------------------------
    halo, bary = unpack_params(theta)
    pot = smx.potentials.potential_struct(bary, halo, st.bulge_mass)
    grid = grid_of(dict_data)
    libd = engine.build_library(pot, bary, dd, grid, st)
    torch.cuda.synchronize()
    ic = libd["ic"]
    bufs = libd["bufs"]
    from schwarmax_gb300 import kernels
    from schwarmax_gb300._lib import SmxIntegrator, SMX_MODE_SAMPLED
    icfg = SmxIntegrator(mode=SMX_MODE_SAMPLED, store_all=0, n_attempts=st.n_attempts, n_samples=st.n_samples,
                         max_attempts=st.max_attempts, atol=st.atol, rtol=st.rtol, dt_min=st.dt_min,
                         dt_max=st.dt_max, omega=-float(bary["Omega_bar"]))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    kernels.integrate(pot, icfg, ic["w0"], ic["dt_init"], ic["t_total"], bufs)
    e1.record()
    torch.cuda.synchronize()
    k_ms = e0.elapsed_time(e1)
    n_att = float(bufs.info[_lib.INFO_NATT].double().sum().item())
    flops = n_att * (3 * FLOPS_PER_FORCE + FLOPS_PER_STEP)
    peaks = measured_peaks() or {}
    clocks = clock_summary(os.path.join(args.out, f"clocks_rank{rank}.csv"), local) if rank == 0 else None
    max_mhz = (clocks or {}).get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * max_mhz * 1e6 / 1e12     # TFLOP/s, FMA = 2
    achieved = flops / (k_ms / 1e3) / 1e12
    roofline = {"kernel": "integrate_kernel<float>", "bound": "fp32", "achieved": round(achieved, 3),
                "peak": round(fp32_peak, 1), "unit": "TFLOP/s", "frac": round(achieved / fp32_peak, 4),
                "peak_source": "nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 at the max SM clock "
                               "(MEASURED_PEAKS.json holds no FP32 figure)",
                "traffic": None, "ms_per_launch": round(k_ms, 3), "attempts": n_att,
                "flops_per_attempt": 3 * FLOPS_PER_FORCE + FLOPS_PER_STEP}
    # --- precision: mixed NNLS vs FP64 NNLS on the same library, and plain FP64 -------
    prec = {}
    if rank == 0 and not args.skip_fp64 and args.bootstrap == "gaussian":
        prec = precision_and_fp64(cfg, dd, grid, nb, theta, st, step, value / world)
    # --- end to end through the public API with host buffers ------------------------------
    e2e = None
    if not args.skip_e2e:
        host, h2d = pinned_host_data(dict_data)
        if world > 1:
            torch.distributed.barrier()    # rank 0 has just run the FP64 comparison alone
        torch.cuda.synchronize()
        t1 = time.time()
        for i in range(args.e2e_steps):
            th = theta.copy()
            th[10] += 0.002 * ((i % 5) - 2)
            smx.model_likelihood(th, host, nb, grid.n_cells, settings=st, nnls_maxiter=cfg.admm_iters, cache=False)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks((time.time() - t1) * 1e3, dev)
        e2e = {"value": whole_job_rate(world, args.e2e_steps, e2e_ms), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": 8 * 3}
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_baseline(cfg, quick=True)
    adj = None
    if rank == 0 and args.adjoint:
        adj = adjoint_timing(dict_data, theta, cfg, st)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (orbits, binning) / bf16 split products + f64 (NNLS)",
                "data": "synthetic (seeded; schwarmax_gb300.synthetic)",
                "config": {"workload": workload(cfg), "bootstrap": args.bootstrap, "parallelism": f"replicas x{world}",
                           "l2": "working set > L2 (no flush)", "setup_s": round(setup_s, 1)},
                "gpu_launches": int(launches), "roofline": roofline, "stages_ms": stages, "precision": prec, "e2e": e2e,
                "cpu_baseline": cpu, "clocks": clocks, "logL_last": float(val.item())}
        if adj is not None:
            line["adjoint"] = adj
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch(args, rank, world, local):
    """Config 2, the metric's batched workload: one step = one batch of P parameter points
    (jax.vmap(model_likelihood) of the reference's notebooks), each a full model
    evaluation; value = evaluations per second.  Every point's orbits run in one
    integrator launch fed by one work queue (autotuned launch shape and cost-ordered
    queue), one projection launch bins all points, then the NNLS and maps of every point.
    Reported beside it: per-stage times of one batch, the integrator's FP32 roofline, the
    precision of point 0 against the plain FP64 kernels (same library and end to end),
    the plain-FP64 rate of one evaluation, the end-to-end rate through
    model_likelihood_batch with host buffers, and the 400-replicate jackknife of one point."""
    import torch

    from schwarmax_gb300 import _lib, engine, kernels, synthetic
    from schwarmax_gb300.likelihood import grid_of, log_likelihoods, log_likelihoods_batch, log_mean_exp

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg = synthetic.CONFIGS[2]
    P = args.points
    t0 = time.time()
    dict_data, theta = synthetic.make_dataset(cfg, seed=args.seed)
    setup_s = time.time() - t0
    st = cfg.settings("mixed")
    st.autotune = not args.no_autotune
    st.bootstrap = args.bootstrap
    dd = engine.DeviceData(dict_data, n_real=st.n_real)
    nb = cfg.n_bins
    nc = cfg.n_grid[0] * cfg.n_grid[1] * cfg.n_grid[2]
    grid = grid_of(dict_data)
    kw = dict(settings=st, nnls_maxiter=cfg.admm_iters)
    points = synthetic.points_for(cfg, P, seed=args.seed + rank)

    def batch(i, keep=False):
        th = points.copy()
        th[:, 10] = th[:, 10] + 0.002 * ((i % 5) - 2)          # M/L walk, MCMC-like
        logl, r = log_likelihoods_batch(th, dd, nb, nc, keep=keep, max_points=args.points_per_launch, **kw)
        m = torch.max(logl, dim=1, keepdim=True).values
        return m[:, 0] + torch.log(torch.mean(torch.exp(logl - m), dim=1)), r

    for i in range(args.warmup):
        batch(i)
    torch.cuda.synchronize()
    # stage launches inside the timed region: CUDA events recorded on the launching stream
    # (no synchronisation), and the integrator's buffers for its attempt count
    names = ["initial_conditions", "integrate_batch", "project_bin_batch", "density_target", "nnls_admm",
             "model_maps"]
    events = {n: [] for n in names}
    integ = []
    orig = {n: getattr(kernels, n) for n in names}

    def wrap(n):
        def f(*a, **k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = orig[n](*a, **k)
            e1.record()
            events[n].append((e0, e1))
            # the integrator launch of the batch (a[7]: its IntegratorBuffers), not the queue-order probe's
            if n == "integrate_batch" and a[7].slots == cfg.n_samples:
                integ.append((e0, e1, a[7]))
            return out
        return f

    sampler = clock_sampler(os.path.join(args.out, f"clocks_rank{rank}.csv")) if rank == 0 else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.kernel_launches()
    for n in names:
        setattr(kernels, n, wrap(n))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        ev0.record()
        for i in range(args.steps):
            val, _ = batch(i)
        ev1.record()
        torch.cuda.synchronize()
    finally:
        for n in names:
            setattr(kernels, n, orig[n])
    if world > 1:
        torch.distributed.barrier()
    launches = _lib.kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev)
    if sampler:
        sampler.terminate()
    stages = {n: round(sum(a.elapsed_time(b) for a, b in events[n]) / args.steps, 3) for n in names}
    stages["batch"] = round(ev0.elapsed_time(ev1) / args.steps, 3)
    value = whole_job_rate(world, args.steps * P, ms)
    # integrator roofline: arithmetic flops of the attempts / launch time, FP32 pipe
    k_ms = sum(a.elapsed_time(b) for a, b, _ in integ) / max(len(integ), 1)
    n_att = float(integ[-1][2].info[_lib.INFO_NATT].double().sum().item()) if integ else 0.0
    flops = n_att * (3 * FLOPS_PER_FORCE + FLOPS_PER_STEP)
    peaks = measured_peaks() or {}
    clocks = clock_summary(os.path.join(args.out, f"clocks_rank{rank}.csv"), local) if rank == 0 else None
    max_mhz = (clocks or {}).get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * max_mhz * 1e6 / 1e12
    achieved = flops / (k_ms / 1e3) / 1e12 if k_ms > 0 else 0.0
    roofline = {"kernel": "integrate_kernel<float, BATCH> (one launch per batch)", "bound": "fp32",
                "achieved": round(achieved, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                "frac": round(achieved / fp32_peak, 4),
                "peak_source": "nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 at the max SM clock "
                               "(MEASURED_PEAKS.json holds no FP32 figure)",
                "traffic": None, "ms_per_launch": round(k_ms, 3), "launches": len(integ), "attempts": n_att,
                "flops_per_attempt": 3 * FLOPS_PER_FORCE + FLOPS_PER_STEP}
    extra = {"stages_ms_per_batch": stages}
    # --- end to end through the public API with host buffers (before the large workspaces below)
    e2e = None
    if not args.skip_e2e:
        from schwarmax_gb300 import model_likelihood_batch
        host, h2d = pinned_host_data(dict_data)
        h2d += points.nbytes
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t1 = time.time()
        for i in range(args.e2e_steps):
            th = points.copy()
            th[:, 10] += 0.002 * ((i % 5) - 2)
            model_likelihood_batch(th, host, nb, nc, settings=st, nnls_maxiter=cfg.admm_iters, cache=False)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks((time.time() - t1) * 1e3, dev)
        e2e = {"value": whole_job_rate(world, args.e2e_steps * P, e2e_ms), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 8 * P, "steps": args.e2e_steps}
    if rank == 0:
        torch.cuda.empty_cache()
        # precision and the plain FP64 denominator on point 0 of the batch
        if not args.skip_fp64 and args.bootstrap == "gaussian":
            th0 = points[0].copy()

            def single(i):
                th = th0.copy()
                th[10] = th0[10] + 0.002 * ((i % 5) - 2)
                logl, r = log_likelihoods(th, dd, nb, nc, **kw)
                return log_mean_exp(logl), r
            extra["precision"] = precision_and_fp64(cfg, dd, grid, nb, th0, st, single, value / world)
            extra["precision"]["point"] = "point 0 of the batch"
        if args.jackknife_points > 0:
            # calculate_delta_chi2 (400 leave-one-bin-out replicates) on the libraries of the
            # first points of the batch, timed after one untimed call on the same library
            torch.cuda.empty_cache()
            jp = min(args.jackknife_points, P)
            _, r = batch(0, keep=True)
            libs = {"libraries": [r["libraries"][0][:jp]]}
            jackknife_batch(points[:1], libs, dd, nb, st, cfg.admm_iters)
            torch.cuda.synchronize()
            t1 = time.time()
            dc = jackknife_batch(points[:jp], libs, dd, nb, st, cfg.admm_iters)
            torch.cuda.synchronize()
            extra["jackknife"] = {"points": jp, "replicates_per_point": nb,
                                  "s_per_point": round((time.time() - t1) / jp, 3),
                                  "delta_chi2": [float(v) for v in dc]}
            del r, libs
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_baseline(cfg, quick=True)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (orbits, binning) / bf16 split products + f64 (NNLS)",
                "data": "synthetic (seeded; schwarmax_gb300.synthetic)",
                "config": {"workload": WORKLOAD_BATCH.format(P=P, jk=""), "bootstrap": args.bootstrap,
                           "evals_per_step": P,
                           "parallelism": f"replicas x{world}", "l2": "working set > L2 (no flush)",
                           "setup_s": round(setup_s, 1), "autotune": st.autotune},
                "gpu_launches": int(launches), "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu,
                "clocks": clocks, "logL_last": [float(v) for v in val.cpu().numpy()[:4]]}
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def critical_path(args):
    """The integrator of one evaluation against the critical path of its longest orbits:
    one launch over all orbits in queue order and in exact cost order (attempts of that
    run, longest first), then the k longest orbits alone.  Prints one JSON object."""
    import numpy as np
    import torch

    from schwarmax_gb300 import _lib, engine, kernels, synthetic
    from schwarmax_gb300._lib import SMX_MODE_SAMPLED, SmxIntegrator
    from schwarmax_gb300.likelihood import unpack_params
    from schwarmax_gb300.potentials import potential_struct
    cfg = synthetic.CONFIGS[args.config]
    dict_data, theta = synthetic.make_dataset(cfg, seed=args.seed)
    st = cfg.settings("mixed")
    dd = engine.DeviceData(dict_data, n_real=st.n_real)
    halo, bary = unpack_params(theta)
    pot = potential_struct(bary, halo, st.bulge_mass)
    pos, normals, uni = dd.cast(st.dtype, st.n_real)
    ic = kernels.initial_conditions(pot, pos, normals, uni, st.n_real, st.n_periods, st.steps_per_period)
    icfg = SmxIntegrator(mode=SMX_MODE_SAMPLED, store_all=0, n_attempts=st.n_attempts, n_samples=st.n_samples,
                         max_attempts=st.max_attempts, atol=st.atol, rtol=st.rtol, dt_min=st.dt_min,
                         dt_max=st.dt_max, omega=-float(bary["Omega_bar"]))

    def timed(idx=None, order=None, reps=2):
        w0, dt0, tt = ic["w0"], ic["dt_init"], ic["t_total"]
        if idx is not None:
            w0, dt0, tt = w0[:, idx].contiguous(), dt0[idx].contiguous(), tt[idx].contiguous()
        bufs = kernels.IntegratorBuffers(w0.shape[1], st.n_samples, st.dtype, torch.device("cuda"))
        icfg.order = 0 if order is None else order.data_ptr()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            kernels.integrate(pot, icfg, w0, dt0, tt, bufs)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best, bufs

    out = {"workload": f"config {args.config}: {ic['w0'].shape[1]} orbits, {st.n_samples} samples"}
    out["queue_order_ms"], bufs = timed()
    att = bufs.info[_lib.INFO_NATT].double().cpu().numpy()
    order = np.argsort(-att, kind="stable")
    out["attempts"] = {"total": float(att.sum()), "mean": float(att.mean()), "median": float(np.median(att)),
                       "p99": float(np.percentile(att, 99)), "max": float(att.max())}
    w = att.reshape(-1, 32)
    ws = att[order].reshape(-1, 32)
    out["lane_use_queue_order"] = float(w.sum() / (32 * w.max(axis=1)).sum())
    out["lane_use_cost_order"] = float(ws.sum() / (32 * ws.max(axis=1)).sum())
    out["cost_order_ms"], _ = timed(order=torch.as_tensor(order.astype(np.int32), device="cuda"))
    for k in (32, 152 * 32, 608 * 32):
        if k < len(order):
            out[f"longest_{k}_alone_ms"], _ = timed(idx=torch.as_tensor(order[:k].astype(np.int64), device="cuda"))
    out["us_per_attempt_longest_alone"] = 1e3 * out["longest_32_alone_ms"] / float(att.max())
    print(json.dumps(out))


def pinned_host_data(dict_data):
    """dict_data with its arrays in pinned host memory, and their bytes."""
    import numpy as np
    import torch
    host, h2d = {}, 0
    for k, v in dict_data.items():
        a = np.asarray(v)
        if a.dtype.kind in "fi" and a.size > 8:
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            host[k] = t
            h2d += t.numel() * t.element_size()
        else:
            host[k] = v
    return host, h2d


def jackknife_batch(thetas, r, dd, nb, st, maxiter):
    """calculate_delta_chi2 (leave-one-bin-out jackknife, one replicate per bin) at every
    point of a batch, on the libraries the batch built: each point's replicates run as
    one batched mixed-precision solve."""
    from schwarmax_gb300.likelihood import chi2_func, grid_of, unpack_params
    from schwarmax_gb300.model import jackknife_of_library
    from schwarmax_gb300.potentials import potential_struct
    grid = grid_of(dd)
    libs = [lib for chunk in r["libraries"] for lib in chunk]
    out = []
    for th, lib in zip(thetas, libs):
        halo, bary = unpack_params(th)
        pot = potential_struct(bary, halo, st.bulge_mass)
        out.append(float(jackknife_of_library(chi2_func, lib, pot, bary, dd, grid, st, maxiter, 1.0, nb)))
    return out


def precision_and_fp64(cfg, dd, grid, nb, theta, st, step, mixed_evals_per_s):
    """Errors of the mixed evaluation against plain FP64, and the plain-FP64 rate.

    * same library: the mixed NNLS + maps against the FP64 NNLS + maps on the float
      library of the mixed run (the solver's contract, Delta chi^2 <= 0.1);
    * the full FP64 evaluation (FP64 ICs, orbits, binning, target, NNLS, maps), timed
      stage by stage with CUDA events; against it: the end-to-end Delta chi^2, the
      orbits' end states, their Jacobi-integral drift, and the per-bin moments of the
      two libraries under the same (FP64) weights;
    * bin indices: the FP32 kernel's (R, z, phi) cells and sky pixels of every stored
      sample image against the same float operations with a correctly rounded atan2."""
    import torch

    from schwarmax_gb300 import _lib, engine, kernels
    from schwarmax_gb300.likelihood import log_mean_exp, unpack_params
    from schwarmax_gb300.potentials import potential_struct

    val_m, r_m = step(0)
    logl_m = r_m["logl"].clone()
    lib32 = r_m["lib"]["library"]
    lib64 = lib32.double()
    d = r_m["data"]
    n = lib64.shape[0]
    nc = grid.n_cells
    row_scale, Y = engine.nnls_inputs(d, dd, nc, (math.sqrt(5.0), math.sqrt(5.0), 1.0))
    w_init = float((d["y_rz"].sum() / n).item())
    W64 = kernels.nnls_admm(lib64, engine.row_map(nc, nb), row_scale, Y, cfg.admm_iters, 1.0, w_init, mixed=False)
    y_xy_b, y_h_b, sh = engine.likelihood_data(dd)
    lum = float(d["mmpo"].item()) * d["l2m"]
    _, logl_64 = kernels.model_maps(lib64, nc, nb, W64, d["gamma"].contiguous(), dd.v0, dd.s,
                                    d["y_rz"].contiguous(), dd.xy, y_xy_b, y_h_b, sh, lum, 1.0, want_maps=False)
    dchi2 = (2 * (logl_m - logl_64)).abs()
    wm = r_m["W"]
    out = {"precision_ok": bool(float(dchi2.max().item()) <= 0.1),
           "dchi2_max_same_library": float(dchi2.max().item()),
           "dchi2_median_same_library": float(dchi2.median().item()),
           "dchi2_marginal_same_library": abs(2 * float((log_mean_exp(logl_m) - log_mean_exp(logl_64)).item())),
           "chi2_scale": float((-2 * logl_64).median().item()),
           "weights_max_rel_same_library": float(((wm - W64).abs().max() / W64.abs().max()).item())}
    # ---- the plain FP64 evaluation, every stage at full size
    halo, bary = unpack_params(theta)
    st64 = engine.Settings(**{**st.__dict__, "precision": "fp64"})
    pot = potential_struct(bary, halo, st64.bulge_mass)
    holder = {}

    def run64():
        holder["r"] = engine.evaluate(pot, bary, dd, grid, st64, cfg.admm_iters, 1.0, want_maps=True)

    stages64 = stage_breakdown(run64)
    r64 = holder["r"]
    total64 = stages64["total"] / 1e3
    out.update({"fp64_evals_per_s": 1.0 / total64, "mixed_over_fp64": mixed_evals_per_s * total64,
                "fp64_stage_ms": stages64})
    out["dchi2_end_to_end_vs_fp64"] = {"max": float((2 * (logl_m - r64["logl"])).abs().max()),
                                       "median": float((2 * (logl_m - r64["logl"])).abs().median())}
    # ---- orbit end states and Jacobi drift (FP32 vs FP64 orbits from the same draws)
    b32, b64 = r_m["lib"]["bufs"], r64["lib"]["bufs"]
    last32 = b32.samples[:6, torch.arange(b32.n_orb, device="cuda"), (b32.n_stored.long() - 1).clamp(min=0)].double()
    last64 = b64.samples[:6, torch.arange(b64.n_orb, device="cuda"), (b64.n_stored.long() - 1).clamp(min=0)]
    pos_err = (last32[:3] - last64[:3]).norm(dim=0) / last64[:3].norm(dim=0).clamp(min=1e-30)
    q = torch.tensor([0.5, 0.9, 0.99], dtype=torch.float64, device="cuda")

    def quant(x):
        v = torch.quantile(x[torch.isfinite(x)][:1_000_000], q)
        return {"median": float(v[0]), "p90": float(v[1]), "p99": float(v[2]), "max": float(x[torch.isfinite(x)].max())}

    drift32 = (b32.info[_lib.INFO_EJ].double() / b32.info[_lib.INFO_EJ0].double() - 1).abs()
    drift64 = (b64.info[_lib.INFO_EJ] / b64.info[_lib.INFO_EJ0] - 1).abs()
    out["orbit_end_state_rel_error"] = quant(pos_err)
    out["jacobi_drift_fp32"] = quant(drift32)
    out["jacobi_drift_fp64"] = quant(drift64)
    # ---- per-bin moments of the two libraries under the FP64 weights
    W = r64["W"]
    m32, _ = kernels.model_maps(lib64, nc, nb, W, r64["data"]["gamma"].contiguous(), dd.v0, dd.s,
                                r64["data"]["y_rz"].contiguous(), dd.xy, y_xy_b, y_h_b, sh, lum, 1.0)
    m64 = r64["maps"]
    mp32, mp64 = engine.split_maps(m32, nc, nb), engine.split_maps(m64, nc, nb)
    sd_rel = ((mp32["surface_density"] - mp64["surface_density"]).abs() / mp64["surface_density"].abs().clamp(min=1e-300))
    mom = {"surface_density_rel": {"median": float(sd_rel.median()), "max": float(sd_rel.max())}}
    for k in range(1, 5):
        dh = (mp32[f"h{k}"] - mp64[f"h{k}"]).abs()
        mom[f"h{k}_abs"] = {"median": float(dh.median()), "max": float(dh.max())}
    out["per_bin_moments_fp32_vs_fp64_orbits"] = mom
    # ---- bin indices of every stored sample image (FP32 kernel vs float ops with a correctly rounded atan2)
    out["cell_index_check"] = index_check(r_m["lib"]["geo"], b32, dd)
    return out


def index_check(geo, bufs, dd, max_samples=20_000_000):
    """Counts the sample images whose Rzphi cell or sky pixel from the FP32 kernel
    differs from the same IEEE float operations (utils.py:10-42, integrates.py:120-146)
    evaluated with torch, where atan2 is the correctly rounded double atan2 rounded to
    float.  Only atan2 may differ (CUDA's atan2f is not correctly rounded)."""
    import torch

    from schwarmax_gb300 import kernels
    slots = bufs.slots
    valid = torch.arange(slots, device="cuda")[None] < bufs.n_stored[:, None].long()     # (n_orb, slots)
    pts = bufs.samples[:6].reshape(6, -1)[:, valid.reshape(-1)][:, :max_samples].contiguous()
    N = pts.shape[1]
    cells, bins, _ = kernels.sample_cells(geo, pts, dd.bin_mapping)
    f = torch.float32
    lo = [geo.R_lo, geo.z_lo, geo.phi_lo]
    hi = [geo.R_hi, geo.z_hi, geo.phi_hi]
    nn = [geo.nR, geo.nz, geo.nphi]
    rot = torch.tensor(list(geo.rot), dtype=f, device="cuda")
    n_cells = geo.nR * geo.nz * geo.nphi
    bad_cell = 0
    bad_pix = 0
    for im in range(4 if geo.symmetry else 1):
        sxy = -1.0 if im >= 2 else 1.0
        sz = -1.0 if im in (1, 3) else 1.0
        x, y, z = pts[0] * sxy, pts[1] * sxy, pts[2] * sz
        R = torch.sqrt(x * x + y * y)
        ph = torch.atan2(y.double(), x.double()).to(f)
        flat = torch.zeros(N, dtype=torch.int64, device="cuda")
        out_ = torch.zeros(N, dtype=torch.bool, device="cuda")
        stride = 1
        for v, a, b, m in zip((R, z, ph), lo, hi, nn):
            span = torch.tensor(b, dtype=f) - torch.tensor(a, dtype=f)
            norm = (v - torch.tensor(a, dtype=f, device="cuda")) / span.to("cuda")
            out_ |= ~(norm < 1) | (norm < 0)
            k = torch.floor(norm * float(m)).clamp(0, m - 1).long()
            flat += k * stride
            stride *= m
        ref_cell = torch.where(out_, torch.full_like(flat, n_cells), flat)
        bad_cell += int((ref_cell != cells[im].long()).sum())
        X = (rot[0] * x + rot[1] * y) + rot[2] * z
        Yv = (rot[3] * x + rot[4] * y) + rot[5] * z
        pix = torch.zeros(N, dtype=torch.int64, device="cuda")
        outp = torch.zeros(N, dtype=torch.bool, device="cuda")
        stride = 1
        for v, a, b, m in zip((X, Yv), (geo.X_lo, geo.Y_lo), (geo.X_hi, geo.Y_hi), (geo.nX, geo.nY)):
            span = torch.tensor(b, dtype=f) - torch.tensor(a, dtype=f)
            norm = (v - torch.tensor(a, dtype=f, device="cuda")) / span.to("cuda")
            outp |= ~(norm < 1) | (norm < 0)
            k = torch.floor(norm * float(m)).clamp(0, m - 1).long()
            pix += k * stride
            stride *= m
        pix = torch.where(outp, torch.full_like(pix, geo.nX * geo.nY), pix)
        ref_bin = dd.bin_mapping.long()[pix]
        bad_pix += int((ref_bin != bins[im].long()).sum())
    images = N * (4 if geo.symmetry else 1)
    return {"images": images, "cell_mismatches": bad_cell, "aperture_mismatches": bad_pix,
            "cell_mismatch_fraction": bad_cell / max(images, 1)}


def stage_breakdown(fn):
    """CUDA-event time of each library stage during one call of fn()."""
    import torch

    from schwarmax_gb300 import kernels
    names = ["initial_conditions", "integrate", "integrate_batch", "project_bin", "project_bin_batch",
             "density_target", "nnls_admm", "model_maps"]
    events = {n: [] for n in names}
    orig = {n: getattr(kernels, n) for n in names}

    def wrap(n):
        def f(*a, **k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = orig[n](*a, **k)
            e1.record()
            events[n].append((e0, e1))
            return r
        return f

    for n in names:
        setattr(kernels, n, wrap(n))
    try:
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        fn()
        t1.record()
        torch.cuda.synchronize()
    finally:
        for n in names:
            setattr(kernels, n, orig[n])
    out = {n: round(sum(a.elapsed_time(b) for a, b in events[n]), 3) for n in names}
    out["total"] = round(t0.elapsed_time(t1), 3)
    return out


def nnls_cpu_seconds(cfg, rng):
    """The oracle ADMM NNLS (nnls.py:68-166 restated, FP64, NumPy/BLAS threads as
    configured) timed on a 1/16-scale problem (n / 16 orbits, m / 16 rows, all
    bootstraps and iterations) and scaled to the full one by its cost
    n^3/3 + m n^2 + maxiter * B * 2 n^2.  Returns (scaled seconds, measured seconds)."""
    import numpy as np
    from oracle import nnls as on
    nf, mf = cfg.n_part, int(np.prod(cfg.n_grid)) + 5 * cfg.n_bins
    ns, ms_ = nf // 16, mf // 16
    B = cfg.n_boot
    U = np.abs(rng.normal(size=(ms_, ns)))
    Y = rng.normal(size=(B, ms_))
    t0 = time.time()
    on.admm(U, Y, 1.0, 1.0, cfg.admm_iters)
    t_n = time.time() - t0
    cost = lambda n_, m_: n_ ** 3 / 3 + m_ * n_ * n_ + cfg.admm_iters * B * 2 * n_ * n_  # noqa: E731
    return t_n * cost(nf, mf) / cost(ns, ms_), t_n


def cpu_baseline(cfg, quick=True, cores=None):
    """The FP64 oracle on a bounded sample of the workload, scaled to evals/s.

    Sample: n orbits of the config (2,048, 10-20 s on one core; the oracle integrates
    all orbits of a call as one vector, and its cost per orbit falls from 16 to 2,048
    orbits by 28x as NumPy's per-step overhead is shared) integrated over 1/25 of the
    horizon (2 of 50 periods) with the same tolerances, per-orbit cost scaled to
    n_part * n_real orbits and 50 periods; plus the oracle NNLS timed at a
    1/16-scale problem and scaled by its cost (nnls_cpu_seconds)."""
    import numpy as np
    from oracle import integrate as oi, orbits as oo, potential as op
    from schwarmax_gb300 import synthetic
    from schwarmax_gb300.likelihood import unpack_params
    theta = synthetic.theta_for(cfg)
    halo, bary = unpack_params(theta)
    P = op.canonical_params(bary, halo, cfg.bulge_mass)
    rng = np.random.default_rng(3)
    n = 2048 if quick else 8192
    pos = synthetic.disc_positions(rng, n)
    R = np.sqrt(pos[:, 0] ** 2 + pos[:, 1] ** 2)
    vc = oo.rotation_curve(R, pos[:, 2], P)
    w = np.concatenate([pos, np.stack([vc * pos[:, 1] / R, -vc * pos[:, 0] / R, np.zeros(n)], -1)], -1)
    To = oo.orbital_timescale(R, pos[:, 2], P)
    periods = 2.0
    t0 = time.time()
    oi.integrate_sampled(w, P, -float(bary["Omega_bar"]), To * periods, int(cfg.n_samples * periods / cfg.n_periods),
                         To / 100, cfg.atol, cfg.rtol, 1e-5, 0.3)
    t_int = time.time() - t0
    per_orbit_period = t_int / (n * periods)
    integ_s = per_orbit_period * cfg.n_part * cfg.n_real * cfg.n_periods
    nnls_s, t_n = nnls_cpu_seconds(cfg, rng)
    total = integ_s + nnls_s
    threads = os.environ.get("OMP_NUM_THREADS")
    return {"value": 1.0 / total, "unit": UNIT, "cores": 1 if quick else (cores or os.cpu_count()),
            "kind": "port",
            "sample": f"FP64 NumPy oracle: {n} orbits x {periods:g} periods of the sampled integrator "
                      f"({t_int:.1f} s, scaled x{cfg.n_part * cfg.n_real * cfg.n_periods / (n * periods):.0f}) + "
                      f"ADMM NNLS at 1/16 scale ({t_n:.1f} s, scaled by cost); BLAS threads={threads or 'default'}",
            "integrator_s": integ_s, "nnls_s": nnls_s}


def _cpu_worker(args):
    """Integrate a share of the sample orbits in a separate process."""
    import numpy as np
    from oracle import integrate as oi
    w, P, om, Tend, ns, dt0, atol, rtol = args
    t0 = time.time()
    oi.integrate_sampled(w, P, om, Tend, ns, dt0, atol, rtol, 1e-5, 0.3)
    return time.time() - t0


def run_reference(args, rank, world):
    """CPU restatement of the evaluation on all host cores (bounded sample: 512 orbits
    per core, so that the oracle's vectorised integrator shares its per-step overhead
    as the reference's vmapped one would)."""
    if rank != 0:
        return
    import multiprocessing as mp

    import numpy as np
    from oracle import orbits as oo, potential as op
    from schwarmax_gb300 import synthetic
    from schwarmax_gb300.likelihood import unpack_params
    cfg = synthetic.CONFIGS[args.config]
    cores = os.cpu_count() or 1
    theta = synthetic.theta_for(cfg)
    halo, bary = unpack_params(theta)
    P = op.canonical_params(bary, halo, cfg.bulge_mass)
    rng = np.random.default_rng(3)
    per = 512
    n = cores * per
    pos = synthetic.disc_positions(rng, n)
    R = np.sqrt(pos[:, 0] ** 2 + pos[:, 1] ** 2)
    vc = oo.rotation_curve(R, pos[:, 2], P)
    w = np.concatenate([pos, np.stack([vc * pos[:, 1] / R, -vc * pos[:, 0] / R, np.zeros(n)], -1)], -1)
    To = oo.orbital_timescale(R, pos[:, 2], P)
    periods = 1.0
    ns = max(1, int(cfg.n_samples * periods / cfg.n_periods))
    jobs = [(w[i::cores], P, -float(bary["Omega_bar"]), To[i::cores] * periods, ns, To[i::cores] / 100, cfg.atol,
             cfg.rtol) for i in range(cores)]
    ctx = mp.get_context("spawn")
    values = []
    for s in range(args.warmup + args.steps):
        t0 = time.time()
        with ctx.Pool(cores) as pool:
            pool.map(_cpu_worker, jobs)
        wall = time.time() - t0
        integ_s = wall * (cfg.n_part * cfg.n_real * cfg.n_periods) / (n * periods)
        if s >= args.warmup:
            values.append(1.0 / integ_s)
    nnls_s, t_n = nnls_cpu_seconds(cfg, rng)
    value = float(1.0 / (1.0 / np.median(values) + nnls_s))
    sample = (f"FP64 NumPy oracle on {cores} processes: {n} orbits x {periods:g} period of the sampled integrator "
              f"per step, wall time scaled to {cfg.n_part * cfg.n_real} orbits x {cfg.n_periods:g} periods; plus the "
              f"ADMM NNLS at 1/16 scale with BLAS threads ({t_n:.1f} s, scaled by cost to {nnls_s:.0f} s). ICs, "
              f"binning and maps are not timed, so this is a lower bound on the CPU cost of one evaluation")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": workload(cfg) + ("; per parameter point of the 64-point batch (on the CPU a "
                                                    "batch costs the sum of its points)" if args.config == 2 else "")},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def adjoint_timing(dict_data, theta, cfg, st):
    """Config 3: the chi^2 gradient with respect to (alpha, beta, gamma, velocity
    scale) on this evaluation's stored orbits (soft apertures, sigma 0.5 pixel), timed
    after one warm-up gradient, and checked against central differences of all four
    components at three points of the config's range: the viewing angles shifted by
    -10, 0 and +10 degrees and the velocity scale 0.8, 1.0 and 1.2.  The difference
    steps are 1e-5 rad and 1e-5 relative; a component whose free set (the orbits with
    non-zero weight) differs between theta + h and theta - h is reported with that flag,
    since chi^2 has a kink there and a central difference across it is not a derivative."""
    import numpy as np
    import torch

    from schwarmax_gb300 import adjoint
    prob, th0 = adjoint.problem_from_evaluation(theta, dict_data, cfg.n_bins,
                                                cfg.n_grid[0] * cfg.n_grid[1] * cfg.n_grid[2], settings=st,
                                                sigma_pix=0.5, precision="mixed")
    prob.admm_iters = 3000      # a converged ADMM start: the active-set steps then have little to do
    th = th0 + np.array([0.05, -0.05, 0.05, 0.05])
    prob.chi2_and_grad(th)
    torch.cuda.synchronize()
    t0 = time.time()
    tim = {}
    c2, g = prob.chi2_and_grad(th, timings=tim)
    torch.cuda.synchronize()
    t_grad = time.time() - t0

    def chi2_and_free_set(t):
        lib = prob.soft_library(t)
        w, idx, _ = prob.solve(lib, prob.design(lib))
        return float(prob.chi2_of_model(lib.t() @ w)), set(idx.cpu().numpy().tolist())

    checks = []
    d10 = np.radians(10.0)
    for shift, vs in ((-d10, 0.8), (0.0, 1.0), (d10, 1.2)):
        t = th0.copy()
        t[:3] += shift
        t[3] = th0[3] * vs
        c, gr = prob.chi2_and_grad(t)
        gr = gr.cpu().numpy()
        settled = bool(prob.kkt_settled)
        rows = []
        for k in range(4):
            h = 1e-5 if k < 3 else 1e-5 * t[3]
            e = np.zeros(4)
            e[k] = h
            (cp, fp), (cm, fm) = chi2_and_free_set(t + e), chi2_and_free_set(t - e)
            fd = (cp - cm) / (2 * h)
            rows.append({"grad": float(gr[k]), "fd": float(fd),
                         "rel_err": float(abs(gr[k] - fd) / max(abs(fd), 1e-300)), "free_set_changes": fp != fm})
        checks.append({"angles_shift_deg": float(np.degrees(shift)), "vscale": float(t[3]), "chi2": c,
                       "kkt_settled": settled,
                       "alpha": rows[0], "beta": rows[1], "gamma": rows[2], "vscale_grad": rows[3]})
    return {"workload": "config3: soft apertures (sigma 0.5 px) on the stored orbits of one config-1 evaluation, "
                        "single data row, FP64 soft projection, ADMM + active-set KKT NNLS; the gradient is that of "
                        "the chi^2 of the converged KKT solution for the unperturbed data",
            "s_per_gradient": round(t_grad, 3), "stages_s": {k: (round(v, 3) if isinstance(v, float) else v)
                                                             for k, v in tim.items()},
            "chi2": c2, "grad_alpha_beta_gamma_vscale": [float(v) for v in g.cpu().numpy()],
            "fd_checks": checks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="2",
                    help="2 (the benchmark: batches of --points parameter points), 1 (one evaluation per step), "
                         "0, 4 or 'small' (profiler captures)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=None, help="end-to-end steps (default 3; 1 batch for --config 2)")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--points", type=int, default=64, help="parameter points per batch (--config 2)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="--config 2: natural integrator launch instead of the tuned one (blocks per SM, queue order)")
    ap.add_argument("--points-per-launch", type=int, default=None,
                    help="--config 2: parameter points per integrator launch (default: engine.MAX_POINTS_PER_LAUNCH)")
    ap.add_argument("--critical-path", action="store_true",
                    help="--config 1: time the integrator launch in queue order and in cost order, and the longest "
                         "orbits alone (32, 4,864 and 19,456 of them), and print them with the attempt statistics")
    ap.add_argument("--bootstrap", default="gaussian", choices=["gaussian", "poisson"],
                    help="gaussian: the reference's perturbed data rows (one shared solve for all resamples); "
                         "poisson: Poisson(1) aperture weights per resample (one solve each)")
    ap.add_argument("--jackknife-points", type=int, default=1,
                    help="--config 2: points of the batch whose 400-replicate leave-one-bin-out jackknife is timed")
    ap.add_argument("--adjoint", action="store_true",
                    help="also time the chi^2 gradient of the differentiable projection + NNLS on this library")
    ap.add_argument("--out", default=os.path.join(ROOT, "bench_out"), help="folder for the clock samples")
    args = ap.parse_args()
    args.config = int(args.config) if args.config.isdigit() else args.config
    os.makedirs(args.out, exist_ok=True)
    if args.e2e_steps is None:
        args.e2e_steps = 1 if args.config == 2 else 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config == 2:
        run_batch(args, rank, world, local)
    elif args.critical_path:
        critical_path(args)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
