#!/usr/bin/env python
"""DOF-updates/s per RK stage of the DGSEM hot path on GB300: mixed precision with
the learned shock indicator against the plain FP64 path, at matched L2 error.

Default workload (--workload khi2d): 2D compressible Euler Kelvin-Helmholtz
instability on a periodic [-1,1]^2 TreeMesh with 512^2 elements (level 9),
polydeg 3 (4,194,304 DOFs per field), VolumeIntegralShockCapturingHG with the
Hennemann-Gassner indicator on density*pressure (alpha_max 0.002, alpha_min
1e-4, smoothing), flux_ranocha volume flux, flux_lax_friedrichs surface and
subcell flux, CarpenterKennedy2N54 with StepsizeCallback(cfl = 1.3).

* Setup (untimed): the learned indicator (MLP 16-64-64-1, BF16 weights) is
  trained on the GPU by the library's own kernels, on (modal coefficients,
  HG indicator) pairs harvested every 10 steps from the KHI run at 256^2 and a
  Gaussian blast at 128^2; it is then deployed with HG as fallback and judge.
* Accuracy (untimed): mixed+learned, mixed+HG and FP64+HG at 512^2 from t = 0
  to t = 0.5, each compared in L2 of density with a 1024^2 run (mixed + HG),
  sampled on a 1024^2 grid of points.
* Throughput: from the t = 0.5 states, W warm-up steps, then K CK2N54 steps
  (CUDA graphs) timed with CUDA events for mixed+learned (`value`), mixed+HG
  and FP64+HG.  A "step" is 5 RK stages; DOF-updates/s per RK stage =
  ndofs x 5 x K / time.
* `roofline`: the mixed HG element kernel timed alone per stage after an L2
  flush (algorithmic bytes per launch / event time); the learned indicator
  kernel beside it.
* `e2e`: the same steps through the C ABI with the state uploaded from and
  downloaded to pinned host memory every step.
* `cpu_baseline`: the oracle (CPU FP64 restatement of Trixi's rhs! + 2N
  stage) on the same mesh, all host threads.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
    python bench.py --workload mms3d      # 3D manufactured solution 32^3, flux differencing
    python bench.py --workload curved2d   # curvilinear StructuredMesh 512^2 (one GPU)

`--impl reference` times the oracle on all host cores instead, on the same
workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "trixi.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "DOF-updates/s per RK stage"
L2_BYTES = 126 * 2 ** 20

# 3D manufactured solution (--workload mms3d)
LEVEL, POLYDEG, CFL, T_END = 5, 3, 0.6, 1.0
WORKLOAD = "3D Euler MMS, periodic [0,2]^3 TreeMesh 32^3 elements, polydeg 3, " \
           "FluxDifferencing(flux_ranocha), flux_lax_friedrichs, CK2N54 CFL 0.6"
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "stage_kernel_3d_mms_32cubed_mixed.json")

# Kelvin-Helmholtz instability with the learned indicator (--workload khi2d)
KHI_LEVEL, KHI_REF_LEVEL, KHI_CFL, KHI_T_ACC, KHI_SAMPLE = 9, 10, 1.3, 0.5, 1024
KHI_WORKLOAD = ("2D Euler Kelvin-Helmholtz instability, periodic [-1,1]^2 TreeMesh 512^2 elements, "
                "polydeg 3, ShockCapturingHG on density*pressure (alpha_max 0.002, alpha_min 1e-4, "
                "smoothing), flux_ranocha volume, flux_lax_friedrichs surface/FV, CK2N54 CFL 1.3; "
                "learned indicator MLP 16-64-64-1 (BF16 weights) with HG fallback; L2(rho) at "
                "t = 0.5 against a 1024^2 run; throughput timed from the t = 0.5 states")
KHI_PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "stage_kernel_2d_khi_512sq_mixed.json")


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def read_traffic(path):
    try:
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


def read_profile(path, key):
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def fma_peaks(dev):
    """Measured FP32 and FP64 FMA rates of this GPU (library microbenchmark), with
    the SM clock sampled meanwhile."""
    import ctypes

    from trixi_gb300 import _lib
    lib = _lib.load()
    sampler = ClockSampler(dev)
    out = {}
    for name, fp64 in (("fp32", 0), ("fp64", 1)):
        best = 0.0
        for _ in range(3):
            v = ctypes.c_double()
            _lib.check(lib.tg_fma_peak(fp64, ctypes.byref(v)))
            best = max(best, v.value)
        out[name + "_tflops"] = best / 1e12
    out["clocks"] = sampler.stop()
    return out


def compute_record(flops_per_launch, ms, peaks):
    """FP32 arithmetic rate of a kernel: flops per launch (from its committed ncu
    capture: 2 FFMA + FADD + FMUL thread instructions) over the live event time."""
    if not flops_per_launch or not peaks:
        return None
    achieved = flops_per_launch / (ms * 1e-3) / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": peaks["fp32_tflops"],
            "unit": "TFLOP/s", "frac": achieved / peaks["fp32_tflops"],
            "flops_per_launch": flops_per_launch, "peak_source": "measured (tg_fma_peak)"}


def make_semi(precision: str, epb: int = 0):
    import trixi_gb300 as T
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEM(polydeg=POLYDEG, surface_flux=T.flux_lax_friedrichs,
                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=LEVEL)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver,
                                          source_terms=T.source_terms_convergence_test,
                                          precision=precision, elements_per_block=epb)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(gpu_index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        self.lines = []
        if self.proc:
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def max_over_ranks(value: float, world: int) -> float:
    """The largest of every rank's `value` (timings: the slowest replica sets the
    whole-job time).  NCCL reduces on the device, gloo on the host."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ndofs: int, ms_per_step: float, world: int) -> float:
    """DOF-updates/s per RK stage of all replicas: each of `world` ranks advances
    its own copy of the workload (ndofs per field, 5 stages per step)."""
    return world * ndofs * 5 / (ms_per_step * 1e-3)


def timed_steps(ctx, steps, cfl, t, sampler_dev=None):
    """K back-to-back step graphs timed with CUDA events on the context stream;
    returns (ms per step, reached t, clocks sampled meanwhile or None)."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.synchronize()
    sampler = ClockSampler(sampler_dev) if sampler_dev is not None else None
    with torch.cuda.stream(stream):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
    t, n = ctx.step(steps, cfl, math.inf, t)
    with torch.cuda.stream(stream):
        ev1.record(stream)
    ev1.synchronize()
    clocks = sampler.stop() if sampler else None
    if n != steps:
        raise RuntimeError(f"{n} of {steps} steps taken")
    return ev0.elapsed_time(ev1) / steps, t, clocks


def timed_stage_parts(ctx, cfl, reps, flush):
    """Each pass of a stage timed alone after an L2 flush (CUDA events on the
    context stream): (stage, indicator ms, element-kernel ms) per repetition,
    cycling over the 5 stages of a step (the state advances as in a step)."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    dt = cfl * ctx.max_dt()
    out = []
    for rep in range(reps):
        s = rep % 5
        with torch.cuda.stream(stream):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
        ctx.rk_stage_part(s, 0.0, dt, 1)
        with torch.cuda.stream(stream):
            e[1].record(stream)
            flush.zero_()
            e2 = torch.cuda.Event(enable_timing=True)
            e2.record(stream)
        ctx.rk_stage_part(s, 0.0, dt, 2)
        with torch.cuda.stream(stream):
            e[2].record(stream)
        e[2].synchronize()
        out.append((s, e[0].elapsed_time(e[1]), e2.elapsed_time(e[2])))
    return out


def khi_semi(level, precision, epb=0):
    from trixi_gb300 import configs as C
    return C.khi_semi(level, precision, epb)


def khi_rho_samples(semi, u, npts=KHI_SAMPLE):
    from trixi_gb300 import configs as C
    return C.sample2d(semi, u, npts)


def e2e_steps(ctx, semi, steps, warmup, cfl, world, flush):
    """The step through the C ABI with host buffers: every step's input state
    copied from page-locked host memory and its result copied back to
    page-locked host memory, the copies overlapping the stepping on the
    context's copy streams (tg_prefetch_state, tg_load_prefetched,
    tg_fetch_state: step k + 1's input arrives and step k's result leaves while
    the device computes), the steps enqueued without waiting (tg_step_enqueue)
    and the clock read once at the end (tg_clock_read)."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    u_host = torch.from_numpy(ctx.download().reshape(-1)).pin_memory()
    outs = [torch.empty_like(u_host).pin_memory() for _ in range(2)]

    def run(n):
        ctx.prefetch(0, u_host.data_ptr())
        for k in range(n):
            ctx.load_prefetched(k % 2)
            if k + 1 < n:
                ctx.prefetch((k + 1) % 2, u_host.data_ptr())
            ctx.step_enqueue(1, cfl, math.inf, 0.0)  # tg_step without the host wait
            ctx.fetch(k % 2, outs[k % 2].data_ptr())
        ctx.transfer_join()
        t, steps, _ = ctx.clock_read()
        if steps != 1:
            raise RuntimeError(f"e2e: {steps} steps taken after the last load, 1 enqueued")

    run(max(warmup, 1))
    ctx.synchronize()
    with torch.cuda.stream(stream):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
    run(steps)
    with torch.cuda.stream(stream):
        e1.record(stream)  # after the join: every copy to the host has landed
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    nbytes = semi.nvalues * 8
    # the host link's own speed for these buffers (DMA copies of the same pinned
    # arrays, as the copy streams make them): with the copies overlapping the
    # stepping, the slower direction bounds a step from below
    dev_buf = torch.empty(u_host.numel(), dtype=torch.float64, device="cuda")
    link = {}
    for name, dst, src in (("h2d", dev_buf, u_host), ("d2h", outs[0], dev_buf)):
        times = []
        for r in range(4):
            with torch.cuda.stream(stream):
                a0 = torch.cuda.Event(enable_timing=True)
                a1 = torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                dst.copy_(src, non_blocking=True)
                a1.record(stream)
            a1.synchronize()
            if r:
                times.append(a0.elapsed_time(a1))
        link[name] = nbytes / (statistics.mean(times) * 1e-3) / 1e9
    del dev_buf
    return {"value": whole_job_rate(semi.ndofs, max_over_ranks(ms, world), world),
            "unit": "DOF-updates/s", "ms_per_step": ms,
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
            "host_link_gbs": {k: round(v, 1) for k, v in link.items()},
            "transfer_floor_ms": max(nbytes / (link["h2d"] * 1e9) * 1e3,
                                     nbytes / (link["d2h"] * 1e9) * 1e3),
            "overlap": "input and result copies on separate copy streams, overlapping the steps"}


def khi_cpu_rate(threads: int, max_seconds: float, level: int = KHI_LEVEL):
    """Oracle (CPU FP64 restatement of Trixi's rhs! + 2N stage) on the KHI mesh
    with HG shock capturing: DOF-updates/s per RK stage over whole CK2N54
    steps run for about `max_seconds` (at least one step)."""
    from oracle import oracle as O
    O.set_threads(threads)
    orc = O.Oracle(2, 3, level, [-1.0, -1.0], [1.0, 1.0],
                   volume_integral=O.VI_SHOCKCAPTURING_HG, volume_flux=O.FLUX_RANOCHA,
                   surface_flux=O.FLUX_LAX_FRIEDRICHS, alpha_max=0.002, alpha_min=0.0001,
                   alpha_smooth=True)
    u = orc.initial_condition(O.IC_KELVIN_HELMHOLTZ, None, 0.0)
    u_tmp = np.zeros_like(u)
    dt = KHI_CFL * orc.max_dt(u)
    stages, t0 = 0, time.perf_counter()
    while True:
        orc.rk_stage(u, u_tmp, stages % 5, 0.0, dt)
        stages += 1
        if stages % 5 == 0 and time.perf_counter() - t0 > max_seconds:
            break
    el = time.perf_counter() - t0
    return orc.ndofs * stages / el, stages, el, orc.ndofs


def khi_arm(args, rank: int, world: int):
    import torch

    from trixi_gb300 import configs as C
    from trixi_gb300.learned import ShockIndicatorMLP

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    setup_t0 = time.perf_counter()
    net = ShockIndicatorMLP(2, 3, seed=3)
    train = C.harvest_and_train(net)
    train_secs = time.perf_counter() - setup_t0

    # ---- accuracy (untimed): t = 0 -> 0.5, learned and FP64 at 512^2, 1024^2 reference
    semi_ml = khi_semi(KHI_LEVEL, "mixed", args.epb)
    semi_hg = khi_semi(KHI_LEVEL, "mixed", args.epb)
    semi_64 = khi_semi(KHI_LEVEL, "fp64")
    u0 = semi_ml.compute_coefficients(0.0)
    ctx_ml, ctx_hg, ctx_64 = semi_ml.device_context, semi_hg.device_context, semi_64.device_context
    net.deploy(semi_ml, band=0.01)
    acc = {}
    t_state = {}
    arms = (("mixed_learned", semi_ml, ctx_ml), ("mixed_hg", semi_hg, ctx_hg),
            ("fp64_hg", semi_64, ctx_64))
    for name, semi, ctx in arms:
        ctx.upload(u0)
        t0 = time.perf_counter()
        t, n = ctx.step(10 ** 7, KHI_CFL, KHI_T_ACC, 0.0)
        ctx.synchronize()
        acc[name] = {"t": t, "steps": n, "secs": time.perf_counter() - t0}
        t_state[name] = t
        if ctx.status() != 0:
            raise RuntimeError(f"{name}: device status word flagged a non-physical state")
    if not args.no_accuracy and rank == 0:
        ref = khi_semi(KHI_REF_LEVEL, "mixed")
        rc = ref.device_context
        rc.upload(ref.compute_coefficients(0.0))
        t, n = rc.step(10 ** 7, KHI_CFL, KHI_T_ACC, 0.0)
        truth = khi_rho_samples(ref, rc.download())
        acc["reference"] = {"scheme": "mixed + HG, 1024^2 elements", "t": t, "steps": n}
        del rc, ref
        for name, semi, ctx in arms:
            d = khi_rho_samples(semi, ctx.download()) - truth
            acc[name]["l2_rho"] = float(np.sqrt(np.mean(d * d)))
            acc[name]["linf_rho"] = float(np.max(np.abs(d)))
        acc["l2_ratio_learned_over_fp64"] = acc["mixed_learned"]["l2_rho"] / acc["fp64_hg"]["l2_rho"]
        acc["l2_ratio_learned_over_hg"] = acc["mixed_learned"]["l2_rho"] / acc["mixed_hg"]["l2_rho"]
        acc["sample_grid"] = f"{KHI_SAMPLE}^2 points (cell centres)"
    # the network against HG on the t = 0.5 state: alpha MAE, fallbacks, positivity
    ctx_ml.alpha()
    pred, hg, flag, counts = net.last(semi_ml.nelements)
    thr = 0.5 * 10 ** (-1.8 * 4 ** 0.25)
    s_par = math.log((1 - 0.0001) / 0.0001)
    a_net = C._clip_alpha(1 / (1 + np.exp(-s_par / thr * (np.maximum(pred, 0) ** 2 - thr))),
                          0.0001, 0.002)
    a_hg = C._clip_alpha(hg, 0.0001, 0.002)
    learned = {"train": train, "setup_secs": train_secs,
               "alpha_mae_network_vs_hg": float(np.mean(np.abs(a_net - a_hg))),
               "band_fallback_fraction": float(np.mean(flag == 1)),
               "positivity_fallbacks_total": int(counts[2]),
               "elements_with_alpha_on_hg": int(np.sum(a_hg > 0))}

    # ---- throughput: W + K steps from the t = 0.5 states ------------------------
    if world > 1:
        torch.distributed.barrier()
    res = {}
    for name, semi, ctx in arms:
        t = t_state[name]
        steps = args.steps if name != "fp64_hg" else max(3, min(args.steps, args.fp64_steps))
        t, _ = ctx.step(args.warmup, KHI_CFL, math.inf, t)
        ms, t, clocks = timed_steps(ctx, steps, KHI_CFL, t,
                                    dev if (name == "mixed_learned" and rank == 0) else None)
        ms = max_over_ranks(ms, world)
        res[name] = dict(ms_per_step=ms, steps=steps, value=whole_job_rate(semi.ndofs, ms, world),
                         clocks=clocks)
        if ctx.status() != 0:
            raise RuntimeError(f"{name}: device status word flagged a non-physical state")
    if world > 1:
        torch.distributed.barrier()

    # ---- roofline: the element kernel and the learned indicator, each alone ------
    parts = timed_stage_parts(ctx_ml, KHI_CFL, max(10, args.steps), flush)
    E, ndofs = semi_ml.nelements, semi_ml.ndofs
    # per launch: u (4 float-float values per node) read and written, u_tmp
    # (FP32) written and, after stage 0, read, rho*p of the new state written
    # (FP32, the next indicator's input); per element its raw blending factor,
    # the 4 face neighbours' ids and raw factors (the kernel applies the
    # smoothing) and the inverse Jacobian
    def elem_bytes(stage):
        return ndofs * (2 * 32 + (16 if stage == 0 else 32) + 4) + E * (4 + 16 + 16 + 4)
    el_ms = statistics.mean(p[2] for p in parts)
    el_bytes = statistics.mean(elem_bytes(p[0]) for p in parts)
    ind_ms = statistics.mean(p[1] for p in parts)
    # the indicator pass: rho*p of every node read (FP32), alpha_raw written
    # (the element kernel smooths it)
    ind_bytes = ndofs * 4 + E * 4
    peaks = read_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    roof = {"bound": "hbm", "achieved": el_bytes / (el_ms * 1e-3) / 1e9, "peak": peak,
            "unit": "GB/s", "traffic": read_traffic(KHI_PROFILE_TRAFFIC),
            "kernel": "mixed_element_kernel<2,4,HG,flux_ranocha,flux_lax_friedrichs>",
            "stage_ms": el_ms, "algorithmic_bytes": el_bytes,
            "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
            "indicator": {"kernel": "learned indicator (modes of rho*p, MLP, HG fallback)",
                          "ms": ind_ms, "algorithmic_bytes": ind_bytes,
                          "achieved": ind_bytes / (ind_ms * 1e-3) / 1e9}}
    roof["frac"] = roof["achieved"] / peak
    roof["indicator"]["frac"] = roof["indicator"]["achieved"] / peak
    fpeaks = fma_peaks(dev) if rank == 0 else None
    roof["compute"] = compute_record(read_profile(KHI_PROFILE_TRAFFIC, "fp32_flops_per_launch"),
                                     el_ms, fpeaks)
    roof["fma_peaks"] = fpeaks

    e2e = None if args.no_e2e else e2e_steps(ctx_ml, semi_ml, args.steps, args.warmup, KHI_CFL,
                                              world, flush)
    ShockIndicatorMLP.undeploy(semi_ml)
    return dict(res=res, acc=acc if not args.no_accuracy else None, learned=learned, roof=roof,
                e2e=e2e, ndofs=ndofs, nelements=E)


def mms_arm(args, rank: int, world: int):
    import torch

    import trixi_gb300 as T

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    results = {}
    semis = {}
    for prec in ("mixed", "fp64"):
        semi = make_semi(prec, args.epb)
        semis[prec] = semi
        ctx = semi.device_context
        stream = torch.cuda.ExternalStream(ctx.stream())
        u0 = semi.compute_coefficients(0.0)
        ctx.upload(u0)
        steps = args.steps if prec == "mixed" else max(3, min(args.steps, args.fp64_steps))
        t, _n = ctx.step(args.warmup, CFL, math.inf, 0.0)
        ctx.synchronize()
        if world > 1:
            torch.distributed.barrier()
        sampler = ClockSampler(dev) if (prec == "mixed" and rank == 0) else None
        # K back-to-back step graphs; the state and stage buffers (2 x 84 MB FP64
        # + u_tmp) are larger than L2, so every step streams them from HBM.
        with torch.cuda.stream(stream):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
        t, n = ctx.step(steps, CFL, math.inf, t)
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        assert n == steps
        times = [ev0.elapsed_time(ev1)]
        ctx.synchronize()
        clocks = sampler.stop() if sampler else None
        if world > 1:
            torch.distributed.barrier()
        tot = max_over_ranks(sum(times), world)
        ms_step = tot / steps
        results[prec] = dict(ms_per_step=ms_step, steps=steps,
                             value=whole_job_rate(semi.ndofs, ms_step, world), clocks=clocks)
        if ctx.status() != 0:
            raise RuntimeError(f"{prec}: device status word flagged a non-physical state")

    # ---- roofline of the stage kernel (mixed): events around single stages ----
    semi = semis["mixed"]
    ctx = semi.device_context
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.upload(semi.compute_coefficients(0.0))
    dt = 0.6 * ctx.max_dt()
    for s in range(5):
        ctx.rk_stage(s, 0.0, dt)
    st = []
    for rep in range(max(10, args.steps)):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        ctx.rk_stage(rep % 5, 0.0, dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        st.append(e0.elapsed_time(e1))
    stage_ms = statistics.mean(st)
    alg_bytes = semi.ndofs * (2 * 8 + 2 * 4) * semi.equations.nvariables  # u r/w FP64, u_tmp r/w FP32
    achieved = alg_bytes / (stage_ms * 1e-3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        with open(PROFILE_TRAFFIC) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        pass

    # ---- e2e through the C ABI with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        ctx.upload(semi.compute_coefficients(0.0))
        e2e = e2e_steps(ctx, semi, args.steps, args.warmup, CFL, world, flush)

    # ---- accuracy at t_end (untimed): L2 density error of both paths ----
    acc = None
    if not args.no_accuracy:
        acc = {}
        for prec, semi_p in semis.items():
            c = semi_p.device_context
            c.upload(semi_p.compute_coefficients(0.0))
            tt, n = c.step(10 ** 7, CFL, T_END, 0.0)
            l2, linf = T.calc_error_norms(None, tt, semi_p)  # on the device
            acc[prec] = {"l2_rho": float(l2[0]), "linf_rho": float(linf[0]), "t": tt, "steps": n}
    return results, dict(stage_ms=stage_ms, achieved=achieved, peak=peak, alg_bytes=alg_bytes,
                         traffic=traffic, peak_src="measured" if "hbm_gbs" in peaks else "fallback"), \
        e2e, acc, semis["mixed"]


# ---------------------------------------------------------------------------
# Curvilinear 2D workload (--workload curved2d): StructuredMesh of the waving
# flag (examples/structured_2d_dgsem/elixir_euler_source_terms_waving_flag.jl)
# at 512^2 elements, polydeg 3, weak form, LLF (max_abs_speed_naive),
# source_terms_convergence_test, CFL 0.8.
CURVED_CELLS, CURVED_CFL, CURVED_T_END = 512, 0.8, 0.25
CURVED_WORKLOAD = ("2D Euler MMS on the waving-flag StructuredMesh (transfinite map), 512^2 "
                   "elements, polydeg 3, weak form, LLF naive, CK2N54 CFL 0.8")


def _waving_flag_faces():
    return (lambda s: (-1.0, s - 1.0), lambda s: (1.0, s + 1.0),
            lambda s: (s, -1.0 + np.sin(0.5 * np.pi * s)),
            lambda s: (s, 1.0 + np.sin(0.5 * np.pi * s)))


def make_curved_semi(precision: str, cells: int = CURVED_CELLS):
    import trixi_gb300 as T
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.FluxLaxFriedrichs(T.max_abs_speed_naive))
    mesh = T.StructuredMesh((cells, cells), faces=_waving_flag_faces())
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver,
                                          source_terms=T.source_terms_convergence_test,
                                          precision=precision)


def curved_cpu_rate(threads: int, nsteps: int, max_seconds: float):
    """Oracle (CPU FP64 restatement of Trixi's curvilinear rhs! + 2N54) on the
    curved workload's mesh: DOF-updates/s per RK stage."""
    from oracle import oracle as O
    O.set_threads(threads)
    semi = make_curved_semi("fp64")
    orc = O.CurvedOracle(3, semi.node_coordinates, semi.mesh.neighbors(), 1.4, O.VI_WEAK,
                         O.FLUX_CENTRAL, O.FLUX_LAX_FRIEDRICHS_NAIVE, O.SRC_CONVERGENCE_TEST)
    u = orc.initial_condition(O.IC_CONVERGENCE_TEST, 0.0)
    t0 = time.perf_counter()
    done = 0
    while done < nsteps:
        u, _t, k = orc.solve(u, 0.0, 10.0, CURVED_CFL, max_steps=1)
        done += k
        if time.perf_counter() - t0 > max_seconds:
            break
    el = time.perf_counter() - t0
    return semi.ndofs * 5 * done / el, done, el


def curved_arm(args):
    import torch

    import trixi_gb300 as T

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    res, semis = {}, {}
    clocks = None
    for prec in ("mixed", "fp64"):
        semi = make_curved_semi(prec)
        semis[prec] = semi
        ctx = semi.device_context
        stream = torch.cuda.ExternalStream(ctx.stream())
        ctx.upload(semi.compute_coefficients(0.0))
        steps = args.steps if prec == "mixed" else max(3, min(args.steps, args.fp64_steps))
        t, _ = ctx.step(args.warmup, CURVED_CFL, math.inf, 0.0)
        ctx.synchronize()
        sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if prec == "mixed" else None
        with torch.cuda.stream(stream):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
        t, n = ctx.step(steps, CURVED_CFL, math.inf, t)
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        if sampler:
            clocks = sampler.stop()
        res[prec] = dict(ms_per_step=ms, steps=n, value=whole_job_rate(semi.ndofs, ms, 1))
        if ctx.status() != 0:
            raise RuntimeError(f"{prec}: device status word flagged a non-physical state")
    # roofline of the mixed curvilinear stage kernel, single stages after an L2 flush
    semi = semis["mixed"]
    ctx = semi.device_context
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.upload(semi.compute_coefficients(0.0))
    dt = CURVED_CFL * ctx.max_dt()
    for s in range(5):
        ctx.rk_stage(s, 0.0, dt)
    st = []
    for rep in range(max(10, args.steps)):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        ctx.rk_stage(rep % 5, 0.0, dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        st.append(e0.elapsed_time(e1))
    stage_ms = statistics.mean(st)
    # per node and stage: u (4 float-float) read + write, u_tmp (4 FP32) read +
    # write, contravariant vectors (float4) + inverse Jacobian (FP32) + source
    # phase (float4) read
    alg_bytes = semi.ndofs * (4 * 8 * 2 + 4 * 4 * 2 + 16 + 4 + 16)
    achieved = alg_bytes / (stage_ms * 1e-3) / 1e9
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        peaks = {}
    peak = peaks.get("hbm_gbs", 6800.0)
    acc = None
    if not args.no_accuracy:
        acc = {}
        for prec, sp in semis.items():
            c = sp.device_context
            c.upload(sp.compute_coefficients(0.0))
            tt, n = c.step(10 ** 7, CURVED_CFL, CURVED_T_END, 0.0)
            l2, linf = T.calc_error_norms(c.download(), tt, sp)
            acc[prec] = {"l2_rho": float(l2[0]), "linf_rho": float(linf[0]), "t": tt, "steps": n}
        # at the elixir's own size and t_end (16^2, t = 2), where the scheme's
        # error (~3e-5) is far above the mixed path's FP32 rounding floor
        # (~1e-9 relative at t = 0.25 on 512^2, where FP64's error is ~2e-11)
        for prec in ("mixed", "fp64"):
            sp = make_curved_semi(prec, 16)
            c = sp.device_context
            c.upload(sp.compute_coefficients(0.0))
            tt, n = c.step(10 ** 7, CURVED_CFL, 2.0, 0.0)
            l2, linf = T.calc_error_norms(c.download(), tt, sp)
            acc[prec + "_16x16_t2"] = {"l2_rho": float(l2[0]), "linf_rho": float(linf[0]),
                                       "t": tt, "steps": n}
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        (rate, done, el), flags = cpu_baseline(curved_cpu_rate, threads, 2, 20.0)
        cpu = {"value": rate, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
               "sample": f"{done} CK2N54 steps of the full 512^2 curved mesh, FP64, {threads} "
                         f"threads, {flags} (C++ restatement of Trixi's curvilinear rhs!, not "
                         f"Trixi)"}
    line = {
        "metric": METRIC, "value": res["mixed"]["value"], "unit": "DOF-updates/s", "n_gpus": 1,
        "steps": res["mixed"]["steps"], "warmup": args.warmup,
        "ms_per_step": res["mixed"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (analytic manufactured solution)",
        "config": {"workload": CURVED_WORKLOAD, "ndofs_per_field": semi.ndofs,
                   "precision": "mixed", "parallelism": "single GPU",
                   "l2_policy": "inputs larger than L2 (2 x 134 MB state + 67 MB u_tmp per step); "
                                "stage-kernel roofline timed after a 256 MB L2 flush"},
        "fp64": {"value": res["fp64"]["value"], "ms_per_step": res["fp64"]["ms_per_step"],
                 "steps": res["fp64"]["steps"], "dtype": "f64"},
        "mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
        "accuracy": acc,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "curved_kernel_mixed<4,weak>", "stage_ms": stage_ms,
                     "algorithmic_bytes": alg_bytes,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
        "cpu_baseline": cpu, "e2e": None, "clocks": clocks,
        # per step: clock prologue, 5 element kernels, clock epilogue; per timed
        # tg_step call: the clock set-up and two clock reads
        "gpu_launches": 7 * res["mixed"]["steps"] + 3,
    }
    print(json.dumps(line))


def cpu_oracle_rate(threads: int, nsteps: int, max_seconds: float):
    """Oracle (CPU FP64 restatement of Trixi's rhs! + 2N54) DOF-updates/s per RK stage."""
    from oracle import oracle as O
    O.set_threads(threads)
    orc = O.Oracle(3, POLYDEG, LEVEL, [0.0] * 3, [2.0] * 3, volume_integral=O.VI_FLUXDIFF,
                   volume_flux=O.FLUX_RANOCHA, surface_flux=O.FLUX_LAX_FRIEDRICHS,
                   source=O.SRC_CONVERGENCE_TEST)
    u = orc.initial_condition(O.IC_CONVERGENCE_TEST, None, 0.0)
    u_tmp = np.zeros_like(u)
    dt = CFL * orc.max_dt(u)
    done, t0 = 0, time.perf_counter()
    while done < nsteps:
        for s in range(5):
            orc.rk_stage(u, u_tmp, s, 0.0, dt)
        done += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    el = time.perf_counter() - t0
    return orc.ndofs * 5 * done / el, done, el, orc.ndofs


def reference_arm(args, rank: int, world: int):
    """The reference's CPU path on the machine's host cores: the oracle (a C++
    restatement of Trixi's FP64 rhs! + 2N stage; Julia and Trixi are not
    installed) on the selected workload, all host threads, rank 0 only."""
    if rank != 0:
        return
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    flags = O.select_build("native")
    budget = float(os.environ.get("TG_REFERENCE_SECONDS", "60"))
    if args.workload == "mms3d":
        if args.warmup > 0:
            cpu_oracle_rate(threads, 1, 0.0)
        rate, done, el, ndofs = cpu_oracle_rate(threads, args.steps, budget)
        workload, stages = WORKLOAD, 5 * done
        sample = f"{done} CK2N54 steps of the full 32^3 mesh"
        data = "synthetic (analytic manufactured solution)"
    elif args.workload == "curved2d":
        rate, done, el = curved_cpu_rate(threads, args.steps, budget)
        ndofs, workload, stages = CURVED_CELLS ** 2 * 16, CURVED_WORKLOAD, 5 * done
        sample = f"{done} CK2N54 steps of the full 512^2 curved mesh"
        data = "synthetic (analytic manufactured solution)"
    else:
        rate, stages, el, ndofs = khi_cpu_rate(threads, budget)
        done, workload = stages // 5, KHI_WORKLOAD
        sample = f"{stages} RK stages of the full 512^2 KHI mesh from t = 0 (HG indicator)"
        data = "synthetic (analytic initial condition)"
    line = {"metric": METRIC, "value": rate, "unit": "DOF-updates/s", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": el / max(done, 1e-9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": data, "impl": "reference",
            "config": {"workload": workload, "ndofs_per_field": ndofs, "precision": "fp64"},
            "cpu_baseline": {"value": rate, "unit": "DOF-updates/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{sample}, FP64, {threads} threads, {flags} "
                                       f"(C++ restatement of Trixi's CPU rhs!, not Trixi)"},
            "e2e": {"value": rate, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline(fn, *a):
    """Runs an oracle rate function with the native build of the oracle."""
    from oracle import oracle as O
    flags = O.select_build("native")
    return fn(*a), flags


def khi_line(args, rank, world):
    out = khi_arm(args, rank, world)
    mms = None
    if not args.no_mms3d:
        import copy
        a2 = copy.copy(args)
        a2.no_e2e, a2.steps = True, min(args.steps, 20)
        results, roof, _e2e, acc, semi3 = mms_arm(a2, rank, world)
        mms = {"workload": WORKLOAD, "ndofs_per_field": semi3.ndofs,
               "value": results["mixed"]["value"], "fp64": results["fp64"]["value"],
               "mixed_over_fp64": results["mixed"]["value"] / results["fp64"]["value"],
               "ms_per_step": results["mixed"]["ms_per_step"], "accuracy": acc,
               "roofline": {"achieved": roof["achieved"], "peak": roof["peak"],
                            "frac": roof["achieved"] / roof["peak"], "stage_ms": roof["stage_ms"],
                            "algorithmic_bytes": roof["alg_bytes"], "traffic": roof["traffic"],
                            "kernel": "mixed_element_pipe_kernel<3,4,FD,flux_ranocha,"
                                      "flux_lax_friedrichs,EPB=2>"}}
    if rank != 0:
        return
    res = out["res"]
    ml, hg, f64 = res["mixed_learned"], res["mixed_hg"], res["fp64_hg"]
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        (rate, stages, el, _), flags = cpu_baseline(khi_cpu_rate, threads, 15.0)
        cpu = {"value": rate, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
               "sample": f"{stages} RK stages of the full 512^2 KHI mesh (HG indicator), FP64, "
                         f"{threads} threads, {flags} (C++ restatement of Trixi's CPU rhs!, "
                         f"not Trixi)"}
    line = {
        "metric": METRIC, "value": ml["value"], "unit": "DOF-updates/s", "n_gpus": world,
        "steps": ml["steps"], "warmup": args.warmup, "ms_per_step": ml["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic initial condition; training pairs harvested from the "
                "method's own runs)",
        "config": {"workload": KHI_WORKLOAD, "ndofs_per_field": out["ndofs"],
                   "nelements": out["nelements"], "precision": "mixed",
                   "arithmetic": "FP32 flux, volume and surface arithmetic; state stored as "
                                 "float-float (hi, lo) FP32 pairs (~48-bit significand), FP32 "
                                 "2N register; FP64 for integrals and the step clock",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2_policy": "inputs larger than L2: per step 2 x 134 MB float-float state "
                                "+ 67 MB u_tmp vs 126 MB L2; kernel rooflines timed after a "
                                "256 MB L2 flush"},
        "mixed_hg": {"value": hg["value"], "ms_per_step": hg["ms_per_step"]},
        "fp64": {"value": f64["value"], "ms_per_step": f64["ms_per_step"],
                 "steps": f64["steps"], "dtype": "f64", "indicator": "HG"},
        "mixed_over_fp64": ml["value"] / f64["value"],
        "learned_over_hg": ml["value"] / hg["value"],
        "accuracy": out["acc"],
        "learned": out["learned"],
        "roofline": out["roof"],
        "cpu_baseline": cpu,
        "e2e": out["e2e"],
        "clocks": ml["clocks"],
        # per step: clock prologue, 5 x (indicator, element kernel: the element
        # kernel applies the smoothing itself), clock epilogue; per timed tg_step
        # call: the clock set-up and two clock reads
        "gpu_launches": 12 * ml["steps"] + 3,
        "mms3d": mms,
    }
    print(json.dumps(line))


def mms_line(args, rank, world):
    results, roof, e2e, acc, semi = mms_arm(args, rank, world)
    if rank != 0:
        return
    mixed, fp64 = results["mixed"], results["fp64"]
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        (rate, done, el, _), flags = cpu_baseline(cpu_oracle_rate, threads, 2, 20.0)
        cpu = {"value": rate, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
               "sample": f"{done} CK2N54 steps of the full 32^3 mesh, FP64, {threads} threads, "
                         f"{flags} (C++ restatement of Trixi's CPU rhs!, not Trixi)"}
    line = {
        "metric": METRIC, "value": mixed["value"], "unit": "DOF-updates/s", "n_gpus": world,
        "steps": mixed["steps"], "warmup": args.warmup, "ms_per_step": mixed["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic manufactured solution)",
        "config": {"workload": WORKLOAD, "ndofs_per_field": semi.ndofs, "precision": "mixed",
                   "arithmetic": "FP32 flux arithmetic; float-float state; FP32 2N register",
                   "elements_per_block": semi.device_context.elements_per_block(),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2_policy": "inputs larger than L2: per step 2 x 84 MB FP64 state + 42 MB "
                                "FP32 u_tmp vs 126 MB L2; stage-kernel roofline timed after a "
                                "256 MB L2 flush"},
        "fp64": {"value": fp64["value"], "ms_per_step": fp64["ms_per_step"],
                 "steps": fp64["steps"], "dtype": "f64"},
        "mixed_over_fp64": mixed["value"] / fp64["value"],
        "accuracy": acc,
        "roofline": {"bound": "hbm", "achieved": roof["achieved"], "peak": roof["peak"],
                     "unit": "GB/s", "frac": roof["achieved"] / roof["peak"],
                     "traffic": roof["traffic"],
                     "kernel": "mixed_element_pipe_kernel<3,4,FD,flux_ranocha,flux_lax_friedrichs,EPB=2>",
                     "stage_ms": roof["stage_ms"], "algorithmic_bytes": roof["alg_bytes"],
                     "peak_source": roof["peak_src"]},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": mixed["clocks"],
        # per step: clock prologue, 5 element kernels, clock epilogue; per timed
        # tg_step call: the clock set-up and two clock reads
        "gpu_launches": 7 * mixed["steps"] + 3,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--epb", type=int, default=0, help="elements per block (0: library default)")
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mms3d", action="store_true",
                    help="khi2d: leave out the 3D manufactured-solution figures")
    ap.add_argument("--workload", default="khi2d", choices=["khi2d", "mms3d", "curved2d"],
                    help="khi2d: KHI 512^2 with the learned indicator (headline); mms3d: 3D "
                         "manufactured solution 32^3; curved2d: curvilinear StructuredMesh")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        torch.distributed.init_process_group(
            "nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload == "curved2d":
        if rank == 0:
            curved_arm(args)
        return
    if args.workload == "mms3d":
        mms_line(args, rank, world)
        return
    khi_line(args, rank, world)


if __name__ == "__main__":
    main()
