#!/usr/bin/env python3
"""Benchmark of the periodic FE stiffness operator on one GB300.

Default workload (one "step" = one operator application f = K u):
3D hexahedral periodic grid 128 x 128 x 128, cubic cells h = 1/128,
mu = 1.0, nu = 0.25, FP64, u (3 components per node) ~ N(0, 1) from seed 1
with the mean removed per component.  Metric: operator GDoF/s (DoF = 3 x
128^3 per application) with the HBM roofline fraction of the dominant
kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload operator|operator_f32|cg|serve|aniso]

Multi-GPU (torchrun): every rank runs an independent replica ("replicas
only": the operator does not shard across GPUs here); value = DoF processed
by all ranks / max-over-ranks time.

--impl reference times the reference's CPU path for the same workload (the
oracle restatement of compute_Ku, tests/test_bri17.cpp:56-107, with
numpy/scipy FFTs in place of FFTW) on all host cores, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

METRIC = "operator GDoF/s (% HBM peak); CG solves/s at 1e-8 vs FP64; p50/p99 latency"
L2_BYTES = 129 * 1024 * 1024
WORKLOAD_128 = dict(shape=(128, 128, 128), L=(1.0, 1.0, 1.0), mu=1.0, nu=0.25, seed=1)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.path = os.path.join("/tmp", f"bri17_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for name, val in zip(names, p[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def aggregate_replicas(ms_local: float, units_per_step: int, steps: int, device=None):
    """Whole-job throughput of independent replicas: every rank processed
    `units_per_step * steps` units; the job time is the max over ranks.
    Returns (value in G units/s, max ms).  Works on any torch.distributed
    backend (a CPU tensor for gloo, a CUDA tensor for nccl)."""
    import torch
    import torch.distributed as dist
    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t_max = ms_local
    if ws > 1:
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    return ws * units_per_step * steps / (t_max * 1e-3) / 1e9, t_max


def make_u(shape, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((len(shape),) + tuple(shape))
    u -= u.reshape(len(shape), -1).mean(axis=1).reshape((len(shape),) + (1,) * len(shape))
    return u.astype(dtype)


def fp64_peak_live(torch):
    """FP64 throughput of cuBLAS DGEMM on this GPU (TFLOP/s), measured live
    as the FP64 compute roofline denominator."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def traffic_from_profiles(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/traffic.json), scaled as recorded there; None if absent."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            d = json.load(f)
        return d[workload][kernel]["dram_bytes_per_launch"]
    except Exception:
        return None


def traffic_source(kernel: str, workload: str):
    """Where roofline.traffic comes from: the ncu capture recorded in
    profiles/traffic.json (not measured by this run)."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            d = json.load(f)
        return "recorded in profiles/traffic.json: " + d[workload][kernel]["source"]
    except Exception:
        return None


def pass_bytes(geom_dim, dof, cspec, comps, scalar):
    """Algorithmic bytes per launch of each pass: every pass reads its input
    array once and writes its output array once."""
    csz = 2 * scalar
    spec = comps * cspec * csz
    field = dof * scalar
    return {"rows_r2c": field + spec, "axis_c2c_fwd": 2 * spec, "axis0_fused": 2 * spec,
            "axis_c2c_inv": 2 * spec, "rows_c2r": spec + field}


def fused_flops(shape, comps):
    """Conventional flop count of one axis0_fused launch: 5 n log2 n per
    complex transform (forward + inverse per component per line) plus ~56
    flops per mode for K(k) and the 3x3 product."""
    import math
    n0 = shape[0]
    lines = int(np.prod(shape[1:-1])) * (shape[-1] // 2 + 1) if len(shape) == 3 else shape[-1] // 2 + 1
    per_line = 2 * comps * 5 * n0 * math.log2(n0) + 56 * n0
    return lines * per_line


# ---------------------------------------------------------------------------


def cpu_reference_apply_time(workload, threads: int, reps: int, warmup: int = 1):
    """Time the oracle restatement of compute_Ku on the host: C2C FFTs
    (numpy pocketfft single-threaded, or scipy.fft with `threads` workers)
    plus the per-mode loop in C with `threads` OpenMP threads.  `warmup`
    untimed applications come first."""
    from oracle import oracle as O
    shape = workload["shape"]
    grid = O.Grid(shape, workload["L"])
    h = O.Hooke(workload["mu"], workload["nu"], grid)
    u = make_u(shape, workload["seed"])
    O.set_num_threads(threads)
    axes = tuple(range(1, len(shape) + 1))
    fft_mod = None
    if threads > 1:
        try:
            import scipy.fft as sf
            fft_mod = sf
        except Exception:
            fft_mod = None

    def apply():
        uc = u.astype(np.complex128)
        if fft_mod is not None:
            uhat = fft_mod.fftn(uc, axes=axes, workers=threads)
        else:
            uhat = np.fft.fftn(uc, axes=axes)
        kuhat = h._modal_loop(O.lib().oracle_stiffness_modal_apply, uhat, grid.dim)
        if fft_mod is not None:
            ku = fft_mod.ifftn(kuhat, axes=axes, norm="forward", workers=threads)
        else:
            ku = np.fft.ifftn(kuhat, axes=axes, norm="forward")
        ku *= grid.cell_volume / grid.size
        return ku.real

    for _ in range(max(1, warmup)):
        apply()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        apply()
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args):
    ws, rank, local = dist_env()
    if ws > 1 and rank != 0:
        return 0
    if args.workload not in ("operator", "operator_f32"):
        print(json.dumps({"impl": "reference", "unavailable":
                          f"--workload {args.workload}: the reference has no CG solver or "
                          "request server (its eigenstress solve is the per-mode direct "
                          "one); its CPU operator path is timed by --workload operator"}))
        return 0
    w = dict(WORKLOAD_128)
    if args.shape:
        w["shape"] = tuple(int(n) for n in args.shape.split("x"))
        w["L"] = (1.0,) * len(w["shape"])
    dof = len(w["shape"]) * int(np.prod(w["shape"]))
    threads = os.cpu_count() or 1
    # Warm-up then K timed steps; each step = one full application.
    times = cpu_reference_apply_time(w, threads, max(1, args.steps), args.warmup)
    total = sum(times)
    value = dof * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GDoF/s",
        "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(w, args.gpus),
        "cpu_baseline": {"value": value, "unit": "GDoF/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full {'x'.join(map(str, w['shape']))} FP64 "
                                   "applications (C2C scipy.fft + OpenMP per-mode loop; "
                                   "the reference computes in FP64 only)"},
        "e2e": {"value": value, "unit": "GDoF/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def float_pair_line(hooke, us, fs, nrot, args, dof, stream, u_host, f_host, hbm_peak):
    """The same workload through the float-pair operator of the FP64 handle
    (hi + lo floats on the FP32 pipe, FP64 fields in memory): device time
    over K applications, end to end through the host entry point, and the
    relative difference from the FP64 operator's output."""
    import ctypes as C

    import torch
    from bri17_gb300 import _lib
    L = _lib.load()
    ref = hooke.apply_stiffness(us[0])
    try:
        hooke.set_float_pair(True)
    except Exception:
        return None
    for i in range(args.warmup):
        hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    diff = float((hooke.apply_stiffness(us[0]) - ref).norm() / ref.norm())
    # Per-pass device times (events between the passes).
    L.bri17_op_set_pass_timing(hooke.handle, 1)
    for i in range(args.steps):
        hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
    torch.cuda.synchronize()
    pms = (C.c_double * 16)()
    pn = (C.c_int64 * 16)()
    npass = C.c_int()
    L.bri17_op_pass_times(hooke.handle, pms, pn, 16, C.byref(npass))
    L.bri17_op_set_pass_timing(hooke.handle, 0)
    passes = {L.bri17_pass_name(i).decode(): round(pms[i] / pn[i], 5)
              for i in range(min(16, npass.value)) if pn[i] > 0}
    sp = C.c_void_p(stream.cuda_stream)
    for _ in range(max(1, args.warmup)):
        L.bri17_apply_stiffness_host(hooke.handle, C.c_void_p(u_host.data_ptr()),
                                     C.c_void_p(f_host.data_ptr()), sp)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.bri17_apply_stiffness_host(hooke.handle, C.c_void_p(u_host.data_ptr()),
                                     C.c_void_p(f_host.data_ptr()), sp)
    e2e_s = time.perf_counter() - t0
    form = hooke.fused_form
    hooke.set_float_pair(False)
    return {"value": dof / (ms * 1e-3) / 1e9, "unit": "GDoF/s", "ms_per_step": ms,
            "dtype": "f32 pairs (48-bit significands), f64 fields",
            "rel_diff_vs_f64_operator": diff,
            "operator_hbm_frac": 16 * dof / (ms * 1e-3) / 1e9 / hbm_peak,
            "e2e": {"value": dof * args.steps / e2e_s / 1e9, "unit": "GDoF/s"},
            "axis0_form": form, "pass_ms": passes}


def config_of(w, ngpus, precision="f64"):
    shape = w["shape"]
    return {"workload": f"operator f = K u, periodic grid "
                        f"{'x'.join(map(str, shape))}, h=1/{shape[0]}, "
                        f"mu={w['mu']} nu={w['nu']}, {precision.upper()}, u~N(0,1) seed "
                        f"{w['seed']} mean-free",
            "grid": list(shape), "dof_per_step": len(shape) * int(np.prod(shape)),
            "parallelism": f"replicas x{ngpus}",
            "l2": "inputs rotate over buffer sets larger than L2"}


def run_operator(args, precision="f64"):
    import torch

    from bri17_gb300 import CartesianGrid, Hooke, _lib
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = dict(WORKLOAD_128)
    if args.shape:
        w["shape"] = tuple(int(n) for n in args.shape.split("x"))
        w["L"] = (1.0,) * len(w["shape"])
    shape = w["shape"]
    dim = len(shape)
    dof = dim * int(np.prod(shape))
    hooke = Hooke(w["mu"], w["nu"], CartesianGrid(shape, w["L"]), precision=precision)
    tdt = torch.float64 if precision == "f64" else torch.float32
    scalar = 8 if precision == "f64" else 4
    u0 = torch.from_numpy(make_u(shape, w["seed"])).to(device="cuda", dtype=tdt)
    per_set = 2 * dof * scalar
    nrot = max(2, -(-3 * L2_BYTES // per_set))
    us = [u0.clone() for _ in range(nrot)]
    fs = [torch.empty_like(u0) for _ in range(nrot)]
    stream = torch.cuda.current_stream()
    L = _lib.load()
    for i in range(args.warmup):
        hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
    torch.cuda.synchronize()
    # Official timed region: K applications back to back, CUDA events on the
    # launching stream, nothing between the launches (the passes overlap
    # through programmatic dependent launch).
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # Blocks of exactly K applications, each bracketed by device
    # synchronisation (and a barrier under torchrun), repeated until
    # --min-timed-s has passed; the median block is reported, so that the
    # clock samples cover the whole of a long timed region.
    blocks = []
    t_region = time.perf_counter()
    while True:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
        e1.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        blocks.append(e0.elapsed_time(e1))
        if time.perf_counter() - t_region >= args.min_timed_s or len(blocks) >= 10000:
            break
        if ws > 1:
            torch.distributed.barrier()
    clocks = sampler.stop()
    ms_total = statistics.median(blocks)
    value, t_max = aggregate_replicas(ms_total, dof, args.steps, device="cuda")
    # Per-kernel durations: the same K applications again with the library
    # recording CUDA events around every pass launch (events between the
    # launches also serialise the passes, so this loop is slower).
    import ctypes
    L.bri17_op_set_pass_timing(hooke.handle, 1)
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for i in range(args.steps):
        hooke.apply_stiffness(us[i % nrot], out=fs[i % nrot])
    e3.record(stream)
    torch.cuda.synchronize()
    ms_with_events = e2.elapsed_time(e3) / max(1, args.steps)
    pms = (ctypes.c_double * 16)()
    pn = (ctypes.c_int64 * 16)()
    npass = ctypes.c_int()
    L.bri17_op_pass_times(hooke.handle, pms, pn, 16, ctypes.byref(npass))
    L.bri17_op_set_pass_timing(hooke.handle, 0)
    passes = {L.bri17_pass_name(i).decode(): {"ms_total": pms[i], "launches": pn[i]}
              for i in range(min(16, npass.value)) if pn[i] > 0}
    # Correctness of the timed output (first set) against a fresh apply.
    check = hooke.apply_stiffness(us[0])
    assert torch.equal(check, fs[0]) or args.steps == 0

    # End to end through the host-buffer C-ABI entry point (pinned memory).
    u_host = us[0].cpu().pin_memory()
    f_host = torch.empty_like(u_host).pin_memory()
    import ctypes as C
    sp = C.c_void_p(stream.cuda_stream)
    for _ in range(max(1, args.warmup)):
        _lib.check(L.bri17_apply_stiffness_host(hooke.handle, C.c_void_p(u_host.data_ptr()),
                                                C.c_void_p(f_host.data_ptr()), sp), "host")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.bri17_apply_stiffness_host(hooke.handle, C.c_void_p(u_host.data_ptr()),
                                     C.c_void_p(f_host.data_ptr()), sp)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": dof * args.steps / e2e_s / 1e9, "unit": "GDoF/s",
           "h2d_bytes_per_step": dof * scalar, "d2h_bytes_per_step": dof * scalar,
           "host_path": ("staged copies pipelined per component"
                         if os.environ.get("BRI17_HOST_PATH") == "staged" else
                         "page-locked buffers read and written in place by the first and "
                         "last passes over the host link")}
    # Breakdown: the copies alone (same pinned buffers, one stream).
    dev = torch.empty_like(us[0])
    c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    for _ in range(3):
        c0.record()
        dev.copy_(u_host, non_blocking=True)
        c1.record()
        f_host.copy_(dev, non_blocking=True)
        c2.record()
        c2.synchronize()
    e2e["breakdown_ms"] = {"step": 1e3 * e2e_s / max(1, args.steps),
                           "h2d_alone": c0.elapsed_time(c1), "d2h_alone": c1.elapsed_time(c2),
                           "apply_device": t_max / max(1, args.steps)}

    hbm_peak, peak_kind = peaks()
    cspec = int(np.prod(shape[:-1])) * (shape[-1] // 2 + 1)
    pb = pass_bytes(dim, dof, cspec, dim, scalar)
    dom = max(passes, key=lambda k: passes[k]["ms_total"]) if passes else None
    roof = None
    extra = {}
    if dom:
        avg_ms = passes[dom]["ms_total"] / passes[dom]["launches"]
        ach = pb[dom] / (avg_ms * 1e-3) / 1e9
        # Captured traffic exists for the 128^3 workload only (null otherwise).
        wl = f"{precision}_128cubed" if tuple(shape) == (128, 128, 128) else None
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm_peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": ach / hbm_peak,
                "traffic": traffic_from_profiles(dom, wl),
                "traffic_source": traffic_source(dom, wl),
                "algorithmic_bytes_per_launch": pb[dom], "avg_launch_ms": avg_ms}
        if dom == "axis0_fused":
            flops = fused_flops(shape, dim)
            if precision == "f64":
                p64 = fp64_peak_live(torch)
                extra["fp64_roofline"] = {
                    "kernel": dom, "achieved_tflops": flops / (avg_ms * 1e-3) / 1e12,
                    "peak_tflops": p64, "peak_kind": "cuBLAS DGEMM measured live",
                    "frac": flops / (avg_ms * 1e-3) / 1e12 / p64,
                    "flops_per_launch": flops, "flop_model": "5 n log2 n per complex "
                    "transform + 56 per mode"}
        extra["operator_hbm_frac"] = 2 * dof * scalar / (ms_total / args.steps * 1e-3) / 1e9 / hbm_peak
    if precision == "f64" and ws == 1:
        fp = float_pair_line(hooke, us, fs, nrot, args, dof, stream, u_host, f_host, hbm_peak)
        if fp is not None:
            extra["f64_float_pair"] = fp
    line = {
        "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": precision, "data": "synthetic", "config": config_of(w, ws, precision),
        "roofline": roof, "e2e": e2e, "gpu_launches": sum(p["launches"] for p in passes.values()),
        "gpu_launches_note": "launches per timed region (5 passes x K applications)",
        "clocks": clocks, "timed_blocks": {"blocks": len(blocks), "steps_per_block": args.steps,
                                           "reported": "median block",
                                           "min_ms": min(blocks), "max_ms": max(blocks)},
        "passes": passes, "ms_per_step_with_pass_events": ms_with_events,
        **extra,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        times = cpu_reference_apply_time(w, 1, 2)
        line["cpu_baseline"] = {
            "value": dof * len(times) / sum(times) / 1e9, "unit": "GDoF/s", "cores": 1,
            "kind": "port", "sample": f"{len(times)} full 128^3 applications, 1 thread, "
                                      "C2C numpy FFT + per-mode loop (reference-faithful)"}
    if rank == 0 and ws == 1 and precision == "f64" and not args.shape:
        # The solver and serving configurations, measured in the same run.
        for key, fn in solver_workloads(args):
            t0 = time.perf_counter()
            line[key] = fn()
            line[key]["wall_s"] = time.perf_counter() - t0
            torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# CG workloads (256^3 eigenstress solve; anisotropic 512x512x128).

WORKLOAD_CG = dict(shape=(256, 256, 256), L=(1.0, 1.0, 1.0), mu=1.0, nu=0.3, seed=2)
WORKLOAD_ANISO = dict(shape=(512, 512, 128), L=(1.0, 1.0, 0.125), mu=1.0, nu=0.35, seed=4)


def tau_normal(shape, seed):
    return np.random.default_rng(seed).standard_normal((6,) + tuple(shape))


def tau_inclusions(shape, L, seed):
    """Two z-through columns (centres (0.25, 0.25, Lz/2) and (0.75, 0.75,
    Lz/2), periodic minimum-image distance, radius 0.2): all six Mandel
    components 1 inside, 0 outside, plus N(0, 0.01^2) noise."""
    rng = np.random.default_rng(seed)
    ax = [(np.arange(n) + 0.5) * (Li / n) for n, Li in zip(shape, L)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    inside = np.zeros(shape, dtype=bool)
    for c in ((0.25, 0.25, L[2] / 2), (0.75, 0.75, L[2] / 2)):
        d2 = 0.0
        for coord, cc, Li in zip((X, Y, Z), c, L):
            dd = np.abs(coord - cc)
            dd = np.minimum(dd, Li - dd)
            d2 = d2 + dd * dd
        inside |= d2 <= 0.2 ** 2
    tau = rng.normal(0.0, 0.01, size=(6,) + tuple(shape))
    tau += inside[None].astype(np.float64)
    return tau


def oracle_solution(w, tau, threads):
    """The FP64 oracle's exact solution of the eigenstress problem: the
    per-mode direct solve of include/bri17/bri17.hpp:308-341 over the half
    spectrum, with `threads` FFT and per-mode threads."""
    from oracle import oracle as O
    O.set_num_threads(threads)
    h = O.Hooke(w["mu"], w["nu"], O.Grid(w["shape"], w["L"]))
    return O.eigenstress_solve_half(h, tau, workers=threads)


def solve_reps(args, mode):
    """Timed solves per mode of the CG workloads: --cg-reps when given, else
    3 (mixed) and 1 (plain FP64, the slow one); median reported."""
    if args.cg_reps:
        return args.cg_reps
    return 1 if mode == "plain" else 3


def timed_solves(hooke, b, mode, tol, reps):
    """`reps` solves of K x = b from x = 0, each bracketed by device
    synchronisation; returns (median seconds, last x, last info)."""
    import torch
    times = []
    x, info = None, None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, info = hooke.cg_solve(b, tol=tol, mode=mode, max_iterations=400000,
                                 raise_on_failure=False)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return statistics.median(times), x, info


def cg_object(args, w, tau_fn, label, acc_tol=None):
    """One CG workload: FP64 CG and mixed-precision CG (FP32 operator, FP64
    reliable updates) solving K x = b(tau) at relative residual 1e-8, each
    solution's relative l2 error against the FP64 oracle (the modal direct
    solve), and -- when acc_tol is given -- both again at the residual
    tolerance acc_tol that brings the oracle error to 1e-8 or below."""
    import torch

    from bri17_gb300 import CartesianGrid, Hooke
    shape = w["shape"]
    dof = 3 * int(np.prod(shape))
    tau_np = tau_fn()
    hooke = Hooke(w["mu"], w["nu"], CartesianGrid(shape, w["L"]))
    tau = torch.from_numpy(tau_np).cuda()
    b = hooke.eigenstress_rhs(tau)
    del tau
    torch.cuda.synchronize()
    x_ref = None
    oracle_s = None
    if not args.no_oracle:
        t0 = time.perf_counter()
        x_ref = oracle_solution(w, tau_np, os.cpu_count() or 1)
        oracle_s = time.perf_counter() - t0
        nref = float(np.linalg.norm(x_ref))
    del tau_np

    def err_of(x):
        if x_ref is None:
            return None
        return float(np.linalg.norm(x.cpu().numpy() - x_ref) / nref)

    tols = [("tol_1e-8", 1e-8)]
    if acc_tol is not None:
        tols.append(("error_1e-8", acc_tol))
    out = {}
    sampler = ClockSampler(0)
    sampler.start()
    for mode in ("mixed", "plain"):
        # Warm-up: a short solve captures the graphs and builds the FP32 twin.
        hooke.cg_solve(b, tol=1e-2, mode=mode, raise_on_failure=False)
        for key, tol in tols:
            reps = solve_reps(args, mode) if key == "tol_1e-8" else min(2, solve_reps(args, mode))
            sec, x, info = timed_solves(hooke, b, mode, tol, reps)
            out.setdefault(key, {})["mixed" if mode == "mixed" else "fp64"] = {
                "solves_per_s": 1.0 / sec, "seconds_per_solve": sec, "timed_solves": reps,
                "iterations": info["iterations"], "outer_iterations": info["outer_iterations"],
                "rel_residual": info["rel_residual"], "status": info["status_text"],
                "error_vs_fp64_oracle": err_of(x)}
            del x
    # The FP64-accurate plain solver on float pairs (operator in hi + lo
    # floats on the FP32 pipe, FP64 vectors), reported beside the FP64-pipe
    # solver; the speed-up of the mixed solver stays against the FP64 pipe.
    try:
        hooke.set_float_pair(True)
    except Exception:
        pass
    else:
        hooke.cg_solve(b, tol=1e-2, mode="plain", raise_on_failure=False)
        for key, tol in tols:
            sec, x, info = timed_solves(hooke, b, "plain", tol, 1)
            out[key]["fp64_float_pair"] = {
                "solves_per_s": 1.0 / sec, "seconds_per_solve": sec, "timed_solves": 1,
                "iterations": info["iterations"], "rel_residual": info["rel_residual"],
                "status": info["status_text"], "error_vs_fp64_oracle": err_of(x),
                "method": "plain CG, operator in float pairs (48-bit significands on the "
                          "FP32 pipe), FP64 vectors"}
            del x
        hooke.set_float_pair(False)
    clocks = sampler.stop()
    for key, tol in tols:
        o = out[key]
        o["tol"] = tol
        o["mixed_over_fp64_speedup"] = o["mixed"]["solves_per_s"] / o["fp64"]["solves_per_s"]
    res = {"workload": label, "grid": list(shape), "dof": dof, "mu": w["mu"], "nu": w["nu"],
           "seed": w["seed"], "unit": "solves/s",
           "mixed_method": "FP32 CG on the FP32 operator with FP64 reliable updates (x += d, "
                           "r = b - K x and the zero-mean projection in FP64 each time the "
                           "FP32 residual has dropped 10x; search direction kept)",
           "fp64_method": "plain CG, FP64 operator and vectors",
           "at_tol_1e-8": out["tol_1e-8"], "oracle": "modal direct solve in FP64 "
           "(include/bri17/bri17.hpp:308-341) on the host, half spectrum",
           "oracle_seconds": oracle_s, "clocks": clocks}
    if acc_tol is not None:
        res["at_error_1e-8"] = out["error_1e-8"]
        res["at_error_1e-8"]["note"] = ("residual tolerance chosen so that the solution's error "
                                        "against the FP64 oracle is at most 1e-8")
    return res


def run_cg(args, w, tau_fn, label, acc_tol=None):
    import torch
    torch.cuda.set_device(0)
    obj = cg_object(args, w, tau_fn, label, acc_tol)
    top = obj["at_error_1e-8"] if acc_tol is not None else obj["at_tol_1e-8"]
    line = {
        "metric": METRIC, "value": top["mixed"]["solves_per_s"], "unit": "solves/s",
        "n_gpus": 1, "steps": top["mixed"]["timed_solves"], "warmup": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 inner / f64 outer", "data": "synthetic",
        "config": {"workload": label, "grid": obj["grid"], "dof": obj["dof"],
                   "tol": top["tol"]},
        "cg": obj, "clocks": obj["clocks"],
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# Serving workload: 512 requests, Poisson arrivals (mean 5 ms), cubic sides
# from {32, 48, 64, 96, 128}, mu ~ U[0.5, 2], nu ~ U[0.1, 0.45],
# tau ~ N(0, 1), tol 1e-8, seed 3.

def serve_requests(n, seed):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(0.005, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    sides = rng.choice([32, 48, 64, 96, 128], size=n)
    mus = rng.uniform(0.5, 2.0, size=n)
    nus = rng.uniform(0.1, 0.45, size=n)
    return [dict(i=i, t=float(arrivals[i]), side=int(sides[i]), mu=float(mus[i]),
                 nu=float(nus[i]), seed=seed * 100003 + i) for i in range(n)]


def make_tau(req):
    s = req["side"]
    return np.random.default_rng(req["seed"]).standard_normal((6, s, s, s))


def serve_object(args):
    """The serving stream (512 requests by default) through the
    continuous-batching server (mixed precision, default policy, and again
    with size priority), then the same arrivals served one at a time by the
    plain FP64 GPU solver; p50/p99 latency (arrival to result on the host)
    and solves/s for each, plus a sample of served solutions checked
    against the FP64 oracle and against the one-at-a-time FP64 solution."""
    import torch

    from bri17_gb300 import CartesianGrid, Hooke
    from bri17_gb300.server import Server
    from oracle import oracle as O
    nreq = args.requests
    reqs = serve_requests(nreq, 3)
    # Every request's tau is generated before the timed region (16 GB of FP64
    # for 512 requests; a generator thread alone produces them slower than
    # the arrival rate, which would throttle the stream).  numpy releases the
    # GIL while filling, so a thread pool spreads the work over the cores.
    # They are generated into page-locked buffers (a server's receive
    # buffers), which the server borrows without a copy.
    from concurrent.futures import ThreadPoolExecutor

    def make_pinned(r):
        t = torch.empty((6,) + (r["side"],) * 3, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = make_tau(r)
        return t
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        taus = list(ex.map(make_pinned, reqs))
    # Requests whose served solution is checked: the first two of each size.
    check_ids = []
    for sz in (32, 48, 64, 96, 128):
        check_ids += [r["i"] for r in reqs if r["side"] == sz][:2]
    kept = {}

    def latency_stats(lat, makespan, sides):
        return {"solves_per_s": len(lat) / makespan, "makespan_s": makespan,
                "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)),
                "p50_latency_s_per_size": {
                    str(sz): float(np.percentile([l for l, s in zip(lat, sides) if s == sz], 50))
                    for sz in (32, 48, 64, 96, 128)}}

    def stream(size_priority, taus, keep):
        """One pass of the request stream through a fresh server; taus are
        consumed (dropped once submitted)."""
        srv = Server(memory_budget_bytes=args.memory_gb << 30, slots_per_bucket=args.slots,
                     size_priority=size_priority)
        # Warm the buckets (graph capture, first-touch) with one tiny solve per size.
        for s in (32, 48, 64, 96, 128):
            srv.submit((s, s, s), (1, 1, 1), 1.0, 0.3, np.zeros((6, s, s, s)), tol=1e-8)
        srv.run_until_idle()
        sampler = ClockSampler(0)
        sampler.start()
        t_start = srv.clock()
        submitted, done = 0, {}
        meta = {}
        host_s = {"submit": 0.0, "step": 0.0, "steps": 0}
        while len(done) < nreq:
            now = srv.clock() - t_start
            while submitted < nreq:
                r, tau = reqs[submitted], taus[submitted]
                if r["t"] > now:
                    break
                s = r["side"]
                h0 = time.perf_counter()
                rid = srv.submit((s, s, s), (1, 1, 1), r["mu"], r["nu"], tau, tol=1e-8)
                host_s["submit"] += time.perf_counter() - h0
                meta[rid] = r
                taus[submitted] = None
                submitted += 1
            if srv.pending:
                h0 = time.perf_counter()
                srv.step()
                host_s["step"] += time.perf_counter() - h0
                host_s["steps"] += 1
                for res in srv.poll():
                    x = srv.result(res["id"])
                    if res["id"] in meta:
                        done[res["id"]] = res
                        if keep and meta[res["id"]]["i"] in check_ids:
                            kept[meta[res["id"]]["i"]] = np.array(x)
            else:
                time.sleep(0.0005)
        makespan = max(d["finish_time_s"] for d in done.values()) - t_start
        clocks = sampler.stop()
        ids = list(done)
        lat = [done[i]["finish_time_s"] - t_start - meta[i]["t"] for i in ids]
        ok = sum(1 for d in done.values() if d["status"] == 0)
        srv.close()
        stats = latency_stats(lat, makespan, [meta[i]["side"] for i in ids])
        stats.update({"succeeded": ok, "host_time_s": host_s,
                      "iterations_mean": float(np.mean([done[i]["iterations"] for i in ids]))})
        return stats, clocks

    # The later passes re-read the same page-locked inputs (borrowed, unchanged).
    taus_prio = list(taus) if args.serve_priority_run else None
    taus_base = list(taus)
    main_stats, clocks = stream(False, taus, True)
    prio_stats = stream(True, taus_prio, False)[0] if taus_prio is not None else None

    # One at a time in FP64 over the same arrivals: a single FIFO server that
    # takes the next request once the previous one's solution is on the host.
    hookes = {}
    for s in (32, 48, 64, 96, 128):
        hookes[s] = Hooke(1.0, 0.3, CartesianGrid((s, s, s), (1, 1, 1)))
        hookes[s].cg_solve(hookes[s].eigenstress_rhs(
            torch.zeros((6, s, s, s), dtype=torch.float64, device="cuda")), tol=1e-8)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    t_start = time.perf_counter()
    lat_b, sides_b, iters_b, ok_b = [], [], [], 0
    solo = {}
    for r, tau in zip(reqs, taus_base):
        now = time.perf_counter() - t_start
        if r["t"] > now:
            time.sleep(r["t"] - now)
        h = hookes[r["side"]]
        h.set_material(r["mu"], r["nu"])
        b = h.eigenstress_rhs(tau.cuda(non_blocking=True))
        x, info = h.cg_solve(b, tol=1e-8, mode="plain", raise_on_failure=False)
        xh = x.cpu()
        lat_b.append(time.perf_counter() - t_start - r["t"])
        sides_b.append(r["side"])
        iters_b.append(info["iterations"])
        ok_b += info["status"] == 0
        if r["i"] in check_ids:
            solo[r["i"]] = xh.numpy()
    base_makespan = time.perf_counter() - t_start
    base_clocks = sampler.stop()
    base = latency_stats(lat_b, base_makespan, sides_b)
    base.update({"succeeded": ok_b, "iterations_mean": float(np.mean(iters_b)),
                 "method": "served over the same arrival times, one request at a time: "
                           "upload, right-hand side, plain FP64 CG to 1e-8, download",
                 "clocks": base_clocks})
    del taus_base

    # Served solutions against the FP64 oracle and against the solo FP64 solve.
    checks = []
    threads = os.cpu_count() or 1
    for i in check_ids:
        r = reqs[i]
        s = r["side"]
        w = dict(shape=(s, s, s), L=(1.0, 1.0, 1.0), mu=r["mu"], nu=r["nu"])
        x_ref = oracle_solution(w, make_tau(r), threads)
        nref = np.linalg.norm(x_ref)
        xs = kept[i].reshape(x_ref.shape)
        checks.append({"request": i, "side": s,
                       "error_vs_fp64_oracle": float(np.linalg.norm(xs - x_ref) / nref),
                       "solo_fp64_error_vs_oracle":
                           float(np.linalg.norm(solo[i].reshape(x_ref.shape) - x_ref) / nref),
                       "diff_vs_solo_fp64": float(np.linalg.norm(xs - solo[i].reshape(
                           x_ref.shape)) / nref)})
    return {"workload": "serving stream: 512 eigenstress CG solves, Poisson arrivals mean "
                        "5 ms, cubic sides {32,48,64,96,128}, mu~U[0.5,2], nu~U[0.1,0.45], "
                        "tau~N(0,1), tol 1e-8, seed 3",
            "requests": nreq, "unit": "solves/s",
            "slots_per_bucket": args.slots, "memory_budget_gb": args.memory_gb,
            "batched_mixed": main_stats, "batched_mixed_size_priority": prio_stats,
            "one_at_a_time_fp64": base,
            "batched_over_one_at_a_time": main_stats["solves_per_s"] / base["solves_per_s"],
            "served_vs_oracle_sample": checks,
            "served_vs_oracle_max_error": max(c["error_vs_fp64_oracle"] for c in checks),
            "note": "offered load (200/s) exceeds capacity: latency includes queueing; "
                    "latency is arrival to result on the host",
            "clocks": clocks}


def run_serve(args):
    import torch
    torch.cuda.set_device(0)
    obj = serve_object(args)
    line = {
        "metric": METRIC, "value": obj["batched_mixed"]["solves_per_s"], "unit": "solves/s",
        "n_gpus": 1, "steps": obj["requests"], "warmup": 5, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic", "config": {"workload": obj["workload"]}, "serve": obj,
        "clocks": obj["clocks"],
    }
    print(json.dumps(line))
    return 0


ACC_TOL_256 = 1e-11  # residual tolerance that brings the 256^3 oracle error to <= 1e-8


def solver_workloads(args):
    """(key, thunk) of the solver and serving objects of the default run:
    the 256^3 eigenstress CG, the anisotropic 512x512x128 CG and the
    serving stream."""
    out = []
    names = set(args.with_workloads.split(",")) if args.with_workloads else set()
    if "cg" in names:
        out.append(("cg_256", lambda: cg_object(
            args, WORKLOAD_CG, lambda: tau_normal(WORKLOAD_CG["shape"], 2),
            "3D 256^3 eigenstress CG, mu=1 nu=0.3, tau~N(0,1) seed 2", ACC_TOL_256)))
    if "aniso" in names:
        w = WORKLOAD_ANISO
        out.append(("aniso", lambda: cg_object(
            args, w, lambda: tau_inclusions(w["shape"], w["L"], 4),
            "3D 512x512x128, h=(1/512,1/512,1/1024), mu=1 nu=0.35, two-column inclusion "
            "eigenstress + N(0,0.01) noise, seed 4")))
    if "serve" in names:
        out.append(("serve", lambda: serve_object(args)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--no-serve-priority-run", dest="serve_priority_run",
                    action="store_false",
                    help="--workload serve: skip the second pass with size priorities")
    ap.add_argument("--cg-reps", type=int, default=0,
                    help="timed solves per mode for --workload cg / aniso "
                         "(default 3 mixed, 1 plain)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="operator",
                    choices=["operator", "operator_f32", "cg", "aniso", "serve"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shape", default="",
                    help="operator workloads: grid other than 128x128x128 (e.g. 256x256x256)")
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--slots", type=int, default=64)
    ap.add_argument("--memory-gb", type=int, default=48)
    ap.add_argument("--min-timed-s", type=float, default=3.0,
                    help="operator workloads: repeat the K-step timed block until this "
                         "many seconds have passed (median block reported)")
    ap.add_argument("--with-workloads", default="cg,aniso,serve",
                    help="--workload operator at the default grid on one GPU: solver and "
                         "serving configurations measured in the same run and reported as "
                         "objects of its line (comma list of cg, aniso, serve; '' for none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "operator_f32":
        return run_operator(args, precision="f32")
    if args.workload == "cg":
        return run_cg(args, WORKLOAD_CG, lambda: tau_normal(WORKLOAD_CG["shape"], 2),
                      "3D 256^3 eigenstress CG, mu=1 nu=0.3, tau~N(0,1) seed 2", ACC_TOL_256)
    if args.workload == "aniso":
        w = WORKLOAD_ANISO
        return run_cg(args, w, lambda: tau_inclusions(w["shape"], w["L"], 4),
                      "3D 512x512x128, h=(1/512,1/512,1/1024), mu=1 nu=0.35, two-column "
                      "inclusion eigenstress + N(0,0.01) noise, seed 4")
    if args.workload == "serve":
        return run_serve(args)
    return run_operator(args)


if __name__ == "__main__":
    sys.exit(main())
