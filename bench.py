#!/usr/bin/env python3
"""Benchmark of the qgw time step on GB300.

Workload: the closed double-gyre basin at NX = NY = 1024 (1023^2 interior
points) with 10 stretched layers, biharmonic viscosity 1e9 m^4/s, fixed
dt = 600 s, seeded Gaussian q of std 1e-7 s^-1 (synthetic data).  One bench
step is one model time step (the reference's timestep(), src/timestep.h:114-167).

Metric: layer-gridpoint-steps/s = nl * (NX-1)^2 * steps / seconds, for the
plain FP64 path (``value``), with the FP32-compensated path reported beside it
(``fp32c``).  ``value`` is device-timed with the state resident in HBM;
``e2e`` goes through the C ABI with host buffers: every step takes q in
from pinned host memory and returns q to it (qgw_step_host: the first kernel
reads the host array across the C2C link, q goes out as qgw_get does).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

``--impl reference`` times the reference's CPU step instead: the C
restatement of the reference step (oracle/qgw_port.c), one full-size model
step per worker per bench step, on every host core (independent replicas:
the reference's MPI build cannot run without MPI).  Under torchrun every rank
runs an independent replica (no collective on the data path; the barrier and
the max over ranks are for timing only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--nl", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32c", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--error-steps", type=int, default=2000,
                    help="length of the FP32c-vs-FP64 comparison run (0: skip)")
    ap.add_argument("--variant-steps", type=int, default=50,
                    help="steps of the periodic / forcing variant lines (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=40, help="0: skip the ensemble measurement")
    ap.add_argument("--ensemble-members", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=500, help="0: skip the serving measurement")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-step-scale", type=int, default=50,
                    help="request step counts are U[500, 5000] divided by this factor")
    return ap.parse_args()


def workload(nx, nl):
    from qgw_gb300 import configs
    return configs.cfg2(nx, nl)


def lgp_of(p):
    from qgw_gb300 import configs
    return configs.lgp(p)


# ------------------------------------------------------------- CPU baseline
def _port_worker_init(nx, nl, seed):
    global _PORT
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from qgw_gb300 import configs
    p = workload(nx, nl)
    _PORT = oracle.Port(p)
    _PORT.set_q(configs.noise_ic(p, seed))
    _PORT.fix_dt(600.0)


def _port_worker_step(n):
    t0 = time.perf_counter()
    _PORT.step(n)
    return time.perf_counter() - t0


def cpu_pool(nx, nl, workers):
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)  # the port only: the reference sources never travel
    ctx = mp.get_context("spawn")
    return ctx.Pool(workers, initializer=_port_worker_init, initargs=(nx, nl, 12345))


def cpu_measure(pool, workers, lgp, steps, warmup):
    """Aggregate lgp-steps/s of `workers` concurrent full-size runs."""
    for _ in range(warmup):
        pool.map(_port_worker_step, [1] * workers)
    t0 = time.perf_counter()
    for _ in range(steps):
        pool.map(_port_worker_step, [1] * workers)
    wall = time.perf_counter() - t0
    return workers * lgp * steps / wall, wall


# ------------------------------------------------------------------ clocks
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.gpu), "-lms", "50"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [l.strip().split(",") for l in self.f.read().splitlines() if l.strip()]
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                power.append(float(r[3]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# --------------------------------------------------------------- roofline
def bytes_per_lgp(precision):
    """Algorithmic HBM bytes per layer-gridpoint of each step kernel.
    Plain FP64: rows forward read q, f0, f1, f2 and write q and the spectral
    field (48); columns read/write the spectral field and read the Helmholtz
    table (24); rows inverse read the spectral field and write psi (16); the
    RHS reads psi and q and writes f0 (24).  Compensated FP32 with the
    spectral zeta: rows forward read q hi/lo, f0, f1, f2 and write q hi/lo
    and the spectral field (32); columns read the spectral field and write it
    and the spectral zeta (12); rows inverse read both spectral fields and
    write psi and zeta (16); the RHS reads psi, q hi and zeta and writes f0
    (16)."""
    if precision == 0:
        return [48.0, 24.0, 16.0, 24.0]
    return [32.0, 12.0, 16.0, 16.0]


def fp64_ops_per_lgp(nl, M, nsweep):
    """FP64-pipe instructions (add, mul and fma each count one) per
    layer-gridpoint of each kernel, from the kernels' arithmetic: DST-I of
    length M-1 = pre-processing 2 + complex FFT of M/2 points (radix-8 first
    pass 52/8 per point, later passes 80/8, radix-4/2 tails) / 2 + split 3 +
    prefix sum 1."""
    H = M // 2
    rem, passes = H, []
    while rem >= 8:
        passes.append(8)
        rem //= 8
    if rem > 1:
        passes.append(rem)
    fft = 0.0
    for i, R in enumerate(passes):
        base = {8: 52, 4: 16, 2: 4}[R]
        tw = 0 if i == 0 else 4 * (R - 1)
        fft += (base + tw) / R
    dst = 2 + fft / 2 + 3 + 1
    k1 = 3 + nl + dst
    k2 = 2 * dst + 1
    k3 = dst + nl
    k4 = 4.4 + 10 + 2 + (4 * nsweep * 1.2 + 1 if nsweep else 0) + 2 + 0.5
    return [k1, k2, k3, k4]


def read_measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


KERNEL_IDS = ["k_rows_fwd", "k_cols", "k_rows_inv", "k_rhs"]
KERNEL_NAMES = ["rows_fwd (AB3 + projection + x-DST)", "cols (y-DST, Helmholtz, inverse y-DST)",
                "rows_inv (spectral projection + inverse x-DST)", "rhs (Jacobian, viscosity, forcing, CFL)"]


def read_kernel_profile(precision, kernel):
    """ncu counters of one step kernel at this workload, from the committed
    summary profiles/traffic.json: per-launch DRAM bytes
    (dram__bytes_read.sum + dram__bytes_write.sum) and, for the FP64 kernels,
    the FP64 pipe's active share.  None when that kernel was not captured."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f).get("fp64" if precision == 0 else "fp32c", {})
        return d.get(KERNEL_IDS[kernel])
    except (OSError, ValueError):
        return None


# -------------------------------------------------------------------- ours
def rank_ops(world, device):
    """Replica coordination: a barrier and the maximum of a value over ranks
    (each rank runs its own whole run; no data-path collective)."""
    import torch

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def whole_job_rate(lgp_per_rank, steps, seconds_max, world):
    """lgp-steps/s of all replicas together, timed by the slowest rank."""
    return world * lgp_per_rank * steps / seconds_max


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    from qgw_gb300 import build, capi, configs

    torch.cuda.set_device(local_rank)
    build.build()
    p = workload(args.nx, args.nl)
    lgp = lgp_of(p)
    q0 = configs.noise_ic(p, 2000)

    barrier, max_over_ranks = rank_ops(world, "cuda")

    def timed(precision, K, W, clocks=None):
        run = capi.Run(p, precision)
        run.set_q(q0)
        run.fix_dt(600.0)
        run.step(W)
        stream = torch.cuda.ExternalStream(run.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        e0.record(stream)
        info = run.step(K)
        e1.record(stream)
        e1.synchronize()
        cl = clocks.stop() if clocks else None
        torch.cuda.synchronize()
        barrier()
        assert info.steps_taken == K, (info.steps_taken, K)
        ms = max_over_ranks(e0.elapsed_time(e1))
        kms = run.profile_kernels(5)
        return run, ms, kms, cl

    K, W = args.steps, args.warmup
    clocks = Clocks(local_rank)
    run64, ms64, kms64, cl = timed(0, K, W, clocks)
    value = whole_job_rate(lgp, K, ms64 / 1e3, world)

    hbm_peak, peak_kind = read_measured_peaks()
    fp64_peak, fp32_peak = capi.probe_fp_rates()
    M = args.nx
    nsweep = 3  # n_hyper = 4: n_hyper/2 + 1 Laplacian sweeps
    bpl = bytes_per_lgp(0)
    dom = max(range(4), key=lambda k: kms64[k])
    achieved = bpl[dom] * lgp / (kms64[dom] / 1e3) / 1e9
    ops = fp64_ops_per_lgp(args.nl, M, nsweep)
    fp64_rate = ops[dom] * 2 * lgp / (kms64[dom] / 1e3) / 1e12  # one FMA slot = 2 flops
    prof64 = read_kernel_profile(0, dom) or {}
    # The plain FP64 kernels are bound by the FP64 pipe, not by HBM: the
    # headline roofline is that pipe (achieved = the kernel's FP64 operations
    # from the instruction model, counted as FMA slots, over its CUDA-event
    # time; peak = the FP64 FMA rate measured live on this GPU, which
    # MEASURED_PEAKS.json does not carry), with ncu's FP64-pipe activity of
    # the same kernel beside it and the HBM fraction as a secondary field.
    roofline = {"bound": "fp64", "kernel": KERNEL_NAMES[dom], "achieved": fp64_rate, "peak": fp64_peak,
                "unit": "TFLOP/s (FP64, FMA-slot equivalent)",
                "frac": fp64_rate / fp64_peak if fp64_peak > 0 else None,
                "peak_source": "measured live: qgw_probe_fp_rates (independent FP64 FMA chains)",
                "ops_per_lgp_model": ops[dom],
                "ncu_fp64_pipe_active_pct": prof64.get("fp64_pipe_active_pct"),
                "traffic": prof64.get("dram_bytes"),
                "step_frac": sum(o * 2 * lgp for o in ops) / (ms64 / K / 1e3) / 1e12 / fp64_peak
                if fp64_peak > 0 else None,
                "kernel_ms": kms64[dom], "all_kernels_ms": kms64,
                "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                        "peak_source": peak_kind, "bytes_per_lgp": bpl[dom],
                        "traffic": prof64.get("dram_bytes")}}

    # e2e: per step, q in from pinned host memory, one step, q out
    E = args.e2e_steps or K
    shape = run64.shape
    qh = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    qo = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    run64.get(q=qh, want=("q",))
    for _ in range(2):
        run64.step_host(1, qh, qo)
    barrier()
    t0 = time.perf_counter()
    for _ in range(E):
        run64.step_host(1, qh, qo)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    # the host arrays cross the link whole: the reference layout with its ghost ring
    e2e = {"value": world * lgp * E / e2e_s, "unit": "lgp-steps/s", "steps": E,
           "h2d_bytes_per_step": int(qh.nbytes), "d2h_bytes_per_step": int(qo.nbytes),
           "api": "qgw_step_host(1 step, q in and q out) per step, pinned host buffers"}
    run64.close()

    fp32c = None
    if not args.no_fp32c:
        run32, ms32, kms32, _ = timed(1, K, W)
        run32.close()
        v32 = world * lgp * K / (ms32 / 1e3)
        b32 = bytes_per_lgp(1)
        dom32 = max(range(4), key=lambda k: kms32[k])
        ach32 = b32[dom32] * lgp / (kms32[dom32] / 1e3) / 1e9
        step_bytes = sum(b32) * lgp / (ms32 / K / 1e3) / 1e9
        fracs = [b32[k] * lgp / (kms32[k] / 1e3) / 1e9 / hbm_peak for k in range(4)]
        prof32 = read_kernel_profile(1, dom32) or {}
        errs = precision_errors(capi, p, q0, args.error_steps) if args.error_steps > 0 else None
        fp32c = {"value": v32, "unit": "lgp-steps/s", "ms_per_step": ms32 / K, "speedup_vs_fp64": v32 / value,
                 "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom32], "achieved": ach32, "peak": hbm_peak,
                              "unit": "GB/s", "frac": ach32 / hbm_peak, "peak_source": peak_kind,
                              "traffic": prof32.get("dram_bytes"), "bytes_per_lgp": b32[dom32],
                              "all_kernels_ms": kms32, "all_kernels_frac": fracs,
                              "step_achieved_gbs": step_bytes, "step_frac": step_bytes / hbm_peak},
                 "error_vs_fp64": errs, "dtype": "f32 (q as f32 hi+lo)"}

    # the other boundary kind and the forcing add-ons at the same size
    variants = None
    if args.variant_steps > 0:
        variants = run_variants(args, capi, configs, torch, max_over_ranks, world)

    ensemble = None
    if args.ensemble_steps > 0:
        ensemble = run_ensemble(args, capi, configs, torch, barrier, max_over_ranks, world)

    serving = None
    if args.serve_requests > 0:
        serving = run_serving(args, capi, configs)

    if rank != 0:
        return None
    cpu = None
    if getattr(args, "_cpu", None) is not None:
        cpu = args._cpu
    launches = K * 4 + 3
    out = {
        "metric": "layer-gridpoint-steps/s at 1024^2 x 10 layers (plain FP64 step)",
        "value": value, "unit": "lgp-steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms64 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Gaussian q, std 1e-7 s^-1)",
        "config": {"workload": f"closed double-gyre basin NX=NY={args.nx}, nl={args.nl}, biharmonic 1e9, "
                               f"dt=600 s, fixed-dt mode", "NX": args.nx, "nl": args.nl,
                   "lgp_per_step": lgp, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": f"inputs larger than L2: FP64 working set "
                         f"{7 * args.nl * (args.nx - 1) * args.nx * 8 / 1e6:.0f} MB per step"},
        "roofline": roofline,
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": cl,
        "fp32c": fp32c,
        "variants": variants,
        "ensemble": ensemble,
        "serving": serving,
        "fp64_tflops_measured": fp64_peak, "fp32_tflops_measured": fp32_peak,
    }
    return out


def precision_errors(capi, p, q0, nsteps, sample=50):
    """The precision form against the plain FP64 path from the same initial
    q, both at fixed dt: rel-L2 of q and psi after 10, 100 and 1000 steps
    (those below nsteps) and after nsteps; the mean kinetic energy and the
    mean wind work (qgw_budget, FP64 reductions) over the second half of the
    run, sampled every `sample` steps."""
    import numpy as np
    runs = []
    for prec in (0, 1):
        r = capi.Run(p, prec)
        r.set_q(q0)
        r.fix_dt(600.0)
        runs.append(r)
    marks = sorted({m for m in (10, 100, 1000) if m < nsteps} | {nsteps})
    points = sorted(set(marks) | set(range(sample, nsteps + 1, sample)))
    ke, ww = [[], []], [[], []]
    out = {"steps": nsteps}
    done = 0
    for pt in points:
        for r in runs:
            k = 0
            while k < pt - done:
                k += r.step(pt - done - k).steps_taken
        done = pt
        if pt % sample == 0 and pt > nsteps // 2:
            for i, r in enumerate(runs):
                b = r.budget()
                ke[i].append(b["ke"])
                ww[i].append(b["wind_work"])
        if pt in marks:
            (psi64, q64), (psi32, q32) = runs[0].get(), runs[1].get()
            out[f"rel_l2_q_{pt}"] = float(np.linalg.norm(q32 - q64) / np.linalg.norm(q64))
            out[f"rel_l2_psi_{pt}"] = float(np.linalg.norm(psi32 - psi64) / np.linalg.norm(psi64))
    for r in runs:
        r.close()
    for name, series in (("mean_ke", ke), ("mean_wind_work", ww)):
        m64, m32 = float(np.mean(series[0])), float(np.mean(series[1]))
        out[name] = {"fp64": m64, "fp32c": m32, "rel_diff": abs(m32 - m64) / abs(m64) if m64 else None}
    out["mean_window"] = f"steps {nsteps // 2 + sample}..{nsteps}, every {sample} steps"
    return out


def run_variants(args, capi, configs, torch, max_over_ranks, world):
    """Step rate of the doubly periodic basin (both precisions) and the cost
    of the forcing add-ons (stochastic ring forcing, 4-D forcing) at the
    workload's size, device-timed like the main line."""
    import numpy as np
    K = args.variant_steps
    base = workload(args.nx, args.nl)

    def rate(params, precision, records=None):
        run = capi.Run(params, precision)
        if records is not None:
            run.set_forcing_records(records)
        run.set_q(configs.noise_ic(params, 2100))
        run.fix_dt(600.0)
        run.step(3)
        stream = torch.cuda.ExternalStream(run.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        info = run.step(K)
        e1.record(stream)
        e1.synchronize()
        assert info.steps_taken == K
        ms = max_over_ranks(e0.elapsed_time(e1)) / K
        run.close()
        return {"ms_per_step": ms, "value": world * lgp_of(params) / (ms / 1e3), "unit": "lgp-steps/s"}

    per = dict(base, bc_fac=-1.0)
    out = {"steps": K, "periodic_fp64": rate(per, 0), "periodic_fp32c": rate(per, 1)}
    # stochastic ring forcing at k_f = 2 pi * 40 / Lx (a ring of radius 40
    # wavenumbers), sigma_f = 1e-12
    st = dict(per, k_f=2 * np.pi * 40 / base["Lx"], sigma_f=1e-12)
    out["periodic_stochastic_fp64"] = rate(st, 0)
    # 4-D forcing, 4 records interpolated in time
    f4 = dict(base, dt_forc=3600.0, dt_forc_period=4 * 3600.0)
    shape = (4,) + tuple(configs.noise_ic(base, 1).shape)
    rec = np.random.Generator(np.random.PCG64(7)).normal(0.0, 1e-12, size=shape)
    out["forcing4d_fp64"] = rate(f4, 0, rec)
    return out


def run_ensemble(args, capi, configs, torch, barrier, max_over_ranks, world):
    """The batched form: uneven members (grids 128^2..1024^2, 2..10 layers,
    random wind amplitude, distinct noise seeds), all FP32-compensated, one
    launch per step stage over all members, replayed as a CUDA graph, the
    work-tile shape (RHS tile height, column-tile width, modes per row-kernel
    block) and then each stage's persistent grid chosen by the autotuner."""
    members = configs.ensemble_members(args.ensemble_members)
    ens = capi.Ensemble([configs.public(p) for p in members], capi.FP32C)
    q0s = [configs.noise_ic(p, p["_seed"]) for p in members]

    def reset():
        for i, (p, q0) in enumerate(zip(members, q0s)):
            ens.set_q(i, q0)
            ens.fix_dt(i, p["dt"])

    reset()
    default_shape = ens.get_shape(0)
    tuned_ms, grids = ens.tune(3)
    shapes = [ens.get_shape(i) for i in range(len(members))]
    reset()
    ens.step(3)
    stream = torch.cuda.ExternalStream(0)
    lgp = sum(configs.lgp(p) for p in members)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    infos = ens.step(args.ensemble_steps, graph=True)
    wall = max_over_ranks(time.perf_counter() - t0)
    assert all(i.steps_taken == args.ensemble_steps for i in infos)
    # a member alone, for the alone-vs-in-the-mix check (bitwise)
    k = max(range(len(members)), key=lambda i: configs.lgp(members[i]))
    psi_mix, q_mix = ens.get(k)
    ens.close()
    run = capi.Run(configs.public(members[k]), capi.FP32C)
    run.set_q(q0s[k])
    run.fix_dt(members[k]["dt"])
    run.step(3 + args.ensemble_steps)
    psi_a, q_a = run.get()
    run.close()
    same = bool((psi_a == psi_mix).all() and (q_a == q_mix).all())
    del stream
    return {"value": world * lgp * args.ensemble_steps / wall, "unit": "lgp-steps/s", "members": len(members),
            "lgp_per_step": lgp, "steps": args.ensemble_steps, "ms_per_step": wall / args.ensemble_steps * 1e3,
            "grids_blocks_per_sm": grids, "tuned_stage_ms": tuned_ms,
            "tile_shape": {"default": default_shape, "tuned_members": shapes,
                           "searched": {"rhs_tile_rows": [16, 32], "col_tile": [8, 4],
                                        "row_group_fwd": [2, 4, 8, 16], "row_group_inv": [2, 3, 4, 5]}},
            "graph": True, "dtype": "f32 (q hi+lo)",
            "largest_member_alone_equals_in_mix": same,
            "timing": "host wall clock around qgw_ensemble_step (graph replays + flush + state read-back)"}


def run_serving(args, capi, configs):
    """The serving form: Poisson arrivals of runs with grids from 256^2 to
    2048^2, 2..20 layers, FP64 or FP32-compensated at 50/50, random wind
    amplitude and noise seed; admission by HBM footprint, continuous
    batching, latency from submission to result."""
    import numpy as np
    import threading
    rng = np.random.Generator(np.random.PCG64(5000))
    reqs = []
    t = 0.0
    for k in range(args.serve_requests):
        t += rng.exponential(1.0 / args.serve_rate)
        NX = int(rng.choice([256, 512, 1024, 2048]))
        nl = int(rng.integers(2, 21))
        tau = float(rng.uniform(0.04, 0.12))
        prec = int(rng.integers(0, 2))
        steps = int(rng.integers(500, 5001)) // max(1, args.serve_step_scale)
        p = configs.basin_params(NX, nl, tau_nm2=tau, dt=600.0, n_hyper=4, nu_hyper=1e9)
        reqs.append((t, p, prec, max(1, steps), 6000 + k))
    pool = capi.Pool(budget_bytes=0, steps_per_tick=16)
    ids = [None] * len(reqs)
    t0 = time.perf_counter()

    def submitter():
        for k, (ta, p, prec, steps, seed) in enumerate(reqs):
            q0 = configs.noise_ic(p, seed)
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids[k] = pool.submit(p, q0, prec, steps)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    lat, work = [], 0.0
    for k, rid in enumerate(ids):
        st = pool.poll(rid, wait_ms=600000)
        assert st == 0, st
        _, _, _, l3 = pool.fetch(rid)
        lat.append(l3[2])
        work += configs.lgp(reqs[k][1]) * reqs[k][3]
    makespan = time.perf_counter() - t0
    stats = pool.stats()
    pool.close()
    lat = np.array(lat)
    n = len(reqs)
    return {"requests": n, "arrival_rate_per_s": args.serve_rate,
            "steps": f"U[500, 5000] / {args.serve_step_scale}", "grids": "{256,512,1024,2048}^2",
            "layers": "U{2..20}", "precision": "FP64 / FP32c 50/50",
            "scaling_vs_stated_load": f"{n} of 2000 requests, step counts divided by {args.serve_step_scale} "
                                      f"(the stated load, ~20 req/s x ~15 M lgp x 2750 steps, exceeds any "
                                      f"single GPU's rate, so the queue grows either way)",
            "throughput": work / makespan, "unit": "lgp-steps/s", "makespan_s": makespan,
            "arrival_window_s": reqs[-1][0],
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "p99_rank": f"{int(np.ceil(0.99 * n))} of {n} sorted latencies",
            "max_resident": stats["max_resident"], "admitted": stats["admitted"], "ticks": stats["ticks"]}


def run_reference(args):
    p = workload(args.nx, args.nl)
    lgp = lgp_of(p)
    workers = os.cpu_count() or 1
    pool = cpu_pool(args.nx, args.nl, workers)
    value, wall = cpu_measure(pool, workers, lgp, args.steps, args.warmup)
    pool.close()
    pool.join()
    cpu = {"value": value, "unit": "lgp-steps/s", "cores": workers, "kind": "port",
           "sample": f"{workers} concurrent full-size runs ({args.nx}^2 x {args.nl}), one model step each "
                     f"per bench step, {args.steps} timed + {args.warmup} warm-up bench steps; the C "
                     f"restatement of the reference step (oracle/qgw_port.c), O(n log n) DST"}
    return {
        "impl": "reference",
        "metric": "layer-gridpoint-steps/s at 1024^2 x 10 layers (plain FP64 step)",
        "value": value, "unit": "lgp-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"closed double-gyre basin NX=NY={args.nx}, nl={args.nl}, biharmonic 1e9, "
                               f"dt=600 s", "NX": args.nx, "nl": args.nl, "lgp_per_step": lgp,
                   "parallelism": f"{workers} independent CPU replicas"},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "lgp-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0
    # CPU baseline first, before any CUDA context exists (spawned workers)
    args._cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        p = workload(args.nx, args.nl)
        workers = os.cpu_count() or 1
        pool = cpu_pool(args.nx, args.nl, workers)
        v, wall = cpu_measure(pool, workers, lgp_of(p), steps=2, warmup=1)
        # one core: one run stepping alone (the reference's serial build)
        v1, wall1 = cpu_measure(pool, 1, lgp_of(p), steps=2, warmup=0)
        pool.close()
        pool.join()
        args._cpu = {"value": v, "unit": "lgp-steps/s", "cores": workers, "kind": "port",
                     "sample": f"{workers} concurrent full-size runs, 1 warm-up + 2 timed model steps each "
                               f"({wall:.1f} s); oracle/qgw_port.c, the C restatement of the reference step",
                     "one_core": {"value": v1, "unit": "lgp-steps/s", "cores": 1,
                                  "sample": f"one full-size run alone, 2 timed model steps ({wall1:.1f} s)"}}
    if world > 1:
        import torch
        torch.distributed.init_process_group(backend="nccl", init_method="env://")
    out = run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
