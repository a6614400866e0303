"""Benchmark: DOF-stage updates/s of the adaptive sparse-grid DG right-hand side with fused
SSP-RK3 stage updates, on the 3D adaptive Burgers workload (u_t + div(u^2/2 (1,1,1)) = 0,
u0 = 0.5 + 0.25 sin(2 pi (x+y+z)), Alpert k=2, Lagrange degree-3 flux interpolation, LxF,
refine 1e-5 / coarsen 1e-6, start level 3, max level 8, CFL 0.1, to T = 0.05).

One bench step = one whole run to T = 0.05 (36 adaptive time steps: predictor, refine, SSP-RK3,
coarsen), timed on the device from the first to the last time step.  The headline `value` is the
plain FP64 path; the metric itself (mixed precision + learned adaptivity against plain FP64 at
matched L2 error) is `burgers3d_adaptive.metric`.  The 6D linear advection stage, the sparse 3D
Burgers steps, the batched solves and the adaptive wave equation are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference runs the reference's own CPU loop (AdaM-DG built from its sources, all host
threads), one adaptive time step per bench step.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "adaptive-multiresolution-dg_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DIM, NMAX, K = 6, 8, 2
COEF = [1.0] * DIM
CFL = 0.1
# DRAM bytes of one mixed stage launch of the 6D N=8 workload, per kernel variant, from ncu
# (dram__bytes_read.sum + dram__bytes_write.sum; variant 0 was not captured)
NCU_TRAFFIC_BYTES = {1: (720.902 + 241.610) * 1e6, 2: (441.076 + 236.082) * 1e6}
# DRAM bytes of one FP64 right-hand side of the 3D adaptive Burgers workload on its final grid
# (1,004 elements), summed over its 11 kernels, ncu with a cold L2 before every kernel
NCU_TRAFFIC_RHS_CONFIG3 = 24.704512e6
METRIC = "DOF-stage updates/s at matched L2 error: plain FP64 vs mixed+learned-adapt"
WORKLOAD = "6D linear advection, sparse grid N=8, Alpert k=2, SSP-RK3 (34,455,456 DOF)"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if len(s) >= 7 and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) >= 7 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 7 for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def element_keys(g) -> np.ndarray:
    """Packed 1D orders of the grid's elements (nmax bits per dimension), one int64 per element."""
    lv, sp = g.elements()
    o = np.where(lv == 0, 0, (1 << np.maximum(lv - 1, 0)) + (sp - 1) // 2).astype(np.int64)
    key = np.zeros(len(o), np.int64)
    for d in range(o.shape[1]):
        key = (key << g.nmax) | o[:, d]
    return key


def horizon_labels(keys_steps, dec_steps, horizon):
    """Classifier labels for a learned step over `horizon` steps: 0 (refine) where the plain
    criterion refines the element at this step or one of the next horizon - 1, else 2 (coarsen)
    where it removes the element at this step, else 1 (keep)."""
    out = []
    for s in range(len(keys_steps)):
        refined = np.concatenate([keys_steps[j][dec_steps[j] == 1]
                                  for j in range(s, min(len(keys_steps), s + horizon))])
        lab = np.where(np.isin(keys_steps[s], refined), 0, np.where(dec_steps[s] == 2, 2, 1))
        out.append(lab.astype(np.int32))
    return out


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The largest of every rank's value (a timed region is as long as its slowest replica)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dt_for():
    dx = 1.0 / (1 << NMAX)
    return CFL * dx / sum(abs(c) for c in COEF)


def exact_l2(g, t):
    return g.l2_error_separable(lambda x, d: math.sin(2 * math.pi * (x - COEF[d] * t)), 0.5 ** (0.5 * DIM))


def fp64_peak_tflops(torch):
    """Measured FP64 FMA throughput of this GPU (torch float64 GEMM, best of 5)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def bench_linear6d(ctx, stream, args, world):
    """6D N=8 linear advection (34,455,456 DOF): device-timed RK3 steps in both modes, the stage
    kernel's roofline, and the end-to-end serving call with host buffers."""
    import torch

    import amdg
    g = amdg.Grid(ctx, DIM, NMAX, K)
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    u0 = g.coefficients().reshape(-1).copy()
    op = amdg.LinearOperator(g, COEF)
    dt = dt_for()
    dof = g.dof

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed_device(prec):
        g.set_coefficients(u0)
        op.rk3_steps(dt, args.warmup, prec)
        g.set_coefficients(u0)
        barrier()
        l0 = ctx.launch_count()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        op.rk3_steps(dt, args.steps, prec)
        e.record(stream)
        barrier()
        launches = ctx.launch_count() - l0
        sec = max_over_ranks(s.elapsed_time(e) / 1e3, world)
        err = exact_l2(g, args.steps * dt)
        return sec, launches, err

    def timed_kernel(prec, reps=6):
        """Average duration of one fused stage launch (dominant kernel), CUDA events on its stream."""
        g.set_coefficients(u0)
        op.rk3_steps(dt, 1, prec)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        op.rk3_steps(dt, reps, prec)
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e) / 1e3 / (3 * reps)

    sec64, launches64, err64 = timed_device(amdg.FP64)
    sec32, launches32, err32 = timed_device(amdg.MIXED)
    k64 = timed_kernel(amdg.FP64)
    k32 = timed_kernel(amdg.MIXED)
    # the tensor-core variant (3xTF32 mma.sync on the bulk-copy ring) forced, beside the autotuner's pick
    chosen = op.tuning()[0][1]
    op.set_variant(amdg.MIXED, 3)
    k_mma = timed_kernel(amdg.MIXED)
    sec_mma, _, err_mma = timed_device(amdg.MIXED)
    op.set_variant(amdg.MIXED, chosen)
    # end to end: every step is a request whose state comes from pinned host memory and whose
    # result goes back to it; amdg_rk3ssp_serve_host overlaps the copies of neighbouring requests
    ins = [torch.empty(dof, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    outs = [torch.empty(dof, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    for a in ins:
        a[:] = u0
    req_in = [ins[r % 2] for r in range(args.steps)]
    req_out = [outs[r % 2] for r in range(args.steps)]
    op.serve_host(req_in[:2], req_out[:2], dt, 1, amdg.MIXED)  # warm-up
    barrier()
    t0 = time.perf_counter()
    op.serve_host(req_in, req_out, dt, 1, amdg.MIXED)
    barrier()
    e2e_sec = time.perf_counter() - t0
    g.set_coefficients(u0)
    op.rk3_steps(dt, 1, amdg.MIXED)
    ctx.synchronize()
    serve_ok = bool(np.array_equal(outs[(args.steps - 1) % 2], g.coefficients().reshape(-1)))
    pairs, flops = op.pairs, op.flops_per_apply
    E = g.num_elements
    bytes_per_launch = 24.0 * dof + 8.0 * pairs + 4.0 * (E * DIM + 1)
    pk, pk_kind = peaks()
    fp64_peak = fp64_peak_tflops(torch)
    units = 3.0 * dof * args.steps * world
    ach32 = bytes_per_launch / k32 / 1e9
    ach64 = bytes_per_launch / k64 / 1e9
    out = {
        "workload": WORKLOAD, "elements": E, "dof": dof, "dt": dt,
        "mixed": {"value": units / sec32, "ms_per_step": sec32 / args.steps * 1e3, "launches": launches32,
                  "l2_error_vs_exact": err32,
                  "dtype": "f32 operator apply; f64 state, stage vectors as f32 (hi, lo) pairs"},
        "plain_fp64": {"value": units / sec64, "ms_per_step": sec64 / args.steps * 1e3, "kernel_ms": k64 * 1e3,
                       "l2_error_vs_exact": err64, "launches": launches64,
                       "fp64_tflops": flops / k64 / 1e12, "fp64_peak_tflops_measured": fp64_peak,
                       "fp64_frac": flops / k64 / 1e12 / fp64_peak, "hbm_frac": ach64 / pk["hbm_gbs"]},
        "roofline_mixed": {"bound": "hbm", "achieved": ach32, "peak": pk["hbm_gbs"], "unit": "GB/s",
                           "frac": ach32 / pk["hbm_gbs"], "traffic": NCU_TRAFFIC_BYTES.get(op.tuning()[0][1]),
                           "peak_kind": pk_kind, "kernel_ms": k32 * 1e3,
                           "algorithmic_bytes_per_launch": bytes_per_launch, "fp32_tflops": flops / k32 / 1e12},
        "e2e_mixed": {"value": units / e2e_sec if world == 1 else None, "unit": "DOF-stage updates/s",
                      "h2d_bytes_per_step": 8 * dof, "d2h_bytes_per_step": 8 * dof,
                      "call": "amdg_rk3ssp_serve_host (mixed), one RK3 step per request, pinned host buffers",
                      "result_matches_device_step": serve_ok},
        "tensor_core_variant": {"kernel": "linear_mma_kernel<6,3> (3xTF32 mma.sync m16n8k8, FP32 accumulation)",
                                "kernel_ms": k_mma * 1e3, "hbm_frac": bytes_per_launch / k_mma / 1e9 / pk["hbm_gbs"],
                                "ms_per_step": sec_mma / args.steps * 1e3, "l2_error_vs_exact": err_mma,
                                "speed_vs_chosen_variant": k32 / k_mma},
        "autotune": {"variants": {"fp64": op.tuning()[0][0], "mixed": op.tuning()[0][1]},
                     "stage_ms": {"fp64": op.tuning()[1][0], "mixed": op.tuning()[1][1]},
                     "bulk_copy_config": {"chosen": op.copy_config()[0],
                                          "stage_ms_by_config": op.copy_config()[1]}},
    }
    out["_cpu"] = (g, u0, op)
    return out


def bench_linear_small(ctx, stream, args):
    """Config 1 at its stated length (2D linear advection, c = (1, 1), u0 = sin(2 pi (x+y)),
    sparse N = 7, 576 elements, 2561 SSP-RK3 steps of 1/2561 to T = 1) and the 4D part of config 2
    (4D N = 8, 850,176 DOF, c = 1, u0 = prod sin(2 pi x_d), to T = 0.1): whole runs timed with CUDA
    events in FP64 and mixed precision, L2 error against the exact translated solution (split
    formula), and for config 1 the reference's own assembled-matrix loop on the host (one thread:
    the Eigen SpMV path has no OpenMP)."""
    import torch

    import amdg
    import amdg_oracle as O
    out = {}

    def run(g, op, u0, dt, steps, prec):
        g.set_coefficients(u0)
        op.rk3_steps(dt, min(steps, 20), prec)  # warm-up
        g.set_coefficients(u0)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        op.rk3_steps(dt, steps, prec)
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e) / 1e3

    # config 1
    g = amdg.Grid(ctx, 2, 7, 2)
    g.init_separable(O.sin_sum_terms(2))
    u0 = g.coefficients().reshape(-1).copy()
    op = amdg.LinearOperator(g, [1.0, 1.0])
    steps, dt = 2561, 1.0 / 2561
    c1 = {"workload": "2D linear advection, sparse grid N=7 (576 elements, 5,184 DOF), k=2, upwind, SSP-RK3, "
                      "2561 steps to T = 1"}
    for name, prec in (("fp64", amdg.FP64), ("mixed", amdg.MIXED)):
        sec = run(g, op, u0, dt, steps, prec)
        err = g.l2_error_separable_sum([lambda x, d, f=f: f(x - 1.0, d) for f in O.sin_sum_terms(2)], 0.5 ** 0.5)
        c1[name] = {"value": 3.0 * g.dof * steps / sec, "ms_per_run": sec * 1e3, "l2_error_vs_exact_T1": err}
    op.close()
    g.close()
    if ensure_ref_harness():
        res = subprocess.run([REF_HARNESS, "linear", "2", "7", "2", "1", "sin_sum", "assembled", str(steps), repr(dt),
                              "1.0", "1.0"], capture_output=True, text=True, check=True,
                             env=dict(os.environ, OMP_NUM_THREADS="1"))
        f = [ln.split() for ln in res.stdout.splitlines() if ln.startswith("TIME")][0]
        kv = dict(x.split("=") for x in f[1:])
        ref = float(kv["dof_stage"]) / float(kv["evolve_s"])
        c1["reference_cpu"] = {"value": ref, "unit": "DOF-stage updates/s", "cores": 1, "kind": "reference",
                               "sample": f"the whole run (AdaM-DG's assembled HyperbolicAlpt + RK3SSP::step_rk, "
                                         f"{float(kv['evolve_s']):.2f} s of evolution)"}
        c1["fp64_vs_reference_cpu"] = c1["fp64"]["value"] / ref
    out["linear2d_config1_T1"] = c1
    # the 4D part of config 2
    g = amdg.Grid(ctx, 4, 8, 2)
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    u0 = g.coefficients().reshape(-1).copy()
    op = amdg.LinearOperator(g, [1.0] * 4)
    dt = CFL * (1.0 / 256) / 4.0
    steps = int(round(0.1 / dt))
    c2 = {"workload": f"4D linear advection, sparse grid N=8 (10,496 elements, 850,176 DOF), k=2, SSP-RK3, "
                      f"{steps} steps to T = 0.1"}
    for name, prec in (("fp64", amdg.FP64), ("mixed", amdg.MIXED)):
        sec = run(g, op, u0, dt, steps, prec)
        err = g.l2_error_separable(lambda x, d, t=steps * dt: math.sin(2 * math.pi * (x - t)), 0.5 ** 2)
        c2[name] = {"value": 3.0 * g.dof * steps / sec, "ms_per_step": sec / steps * 1e3, "l2_error_vs_exact": err}
    op.close()
    g.close()
    out["linear4d_n8_T01"] = c2
    return out


def run_ours(args):
    import torch

    import amdg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = amdg.Context(local)
    # a non-default stream shared by torch (events) and the library (kernels)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- headline: 3D adaptive Burgers to T = 0.05, plain FP64 --------------------------------
    cfg = Config3(ctx, stream)
    for _ in range(args.warmup):
        cfg.run(amdg.FP64)
    barrier()
    runs = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            runs.append(cfg.run(amdg.FP64))
    clocks = clk.summary()
    sec = max_over_ranks(sum(r["sec"] for r in runs), world)
    stage_dof = sum(r["stage_dof_updates"] for r in runs)
    units = stage_dof * world
    value = units / sec
    plain = cfg.run(amdg.FP64, keep=True)
    g, op = plain.pop("_grid"), plain.pop("_op")
    op.close()
    g.close()
    plain["sec"] = sec / args.steps
    plain["value"] = stage_dof / sec
    # end to end through the C-ABI: the state is copied in from pinned host memory at the start of
    # every run and the final state copied out to it (H2D, 36 adaptive steps, D2H)
    hin = torch.empty(1 << 20, dtype=torch.float64, pin_memory=True).numpy()
    hout = torch.empty(1 << 20, dtype=torch.float64, pin_memory=True).numpy()
    cfg.run(amdg.FP64, host_io=(hin, hout))
    barrier()
    e2e = [cfg.run(amdg.FP64, host_io=(hin, hout)) for _ in range(args.steps)]
    e2e_sec = max_over_ranks(sum(r["sec"] for r in e2e), world)
    # dominant work: one FP64 right-hand side on the final grid (CUDA events), against the
    # per-DOF-stage traffic of the Lagrange path (233 B: state, point values, surplus passes)
    rhs_sec, rhs_dof, rhs_E, rhs_flops = config3_rhs_timing(cfg, amdg.FP64)
    rhs32_sec, _, _, _ = config3_rhs_timing(cfg, amdg.MIXED)
    pk, pk_kind = peaks()
    fp64_peak = fp64_peak_tflops(torch)
    ach = 233.0 * rhs_dof / rhs_sec / 1e9
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "DOF-stage updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": sec / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: IC 0.5 + 0.25 sin(2 pi (x+y+z)) projected onto the adaptive grid",
        "config": {"workload": WORKLOAD3, **{k: v for k, v in CONFIG3.items() if k != "tau"},
                   "step": "one run to T = 0.05: 36 adaptive time steps (forward-Euler predictor, refine, "
                           "SSP-RK3, coarsen); DOF-stage updates = 3 x DOF after refinement per time step",
                   "elements_init": 832, "elements_final": runs[-1]["elements_final"],
                   "time_steps_per_run": runs[-1]["steps"],
                   "l2_flush": "a 512 MB buffer written before every timed run (the state is L2-resident)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "l2_error_vs_exact_l1_l2_linf": plain["error_vs_exact_l1_l2_linf"],
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": NCU_TRAFFIC_RHS_CONFIG3, "peak_kind": pk_kind,
                     "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum summed over the 11 kernels of one "
                                     "FP64 right-hand side on this grid, ncu with its default cache flush before "
                                     "every kernel (cold L2); in the run the working set stays in L2 "
                                     "(profiles/rhs_burgers3d_config3.md)",
                     "kernel": "one FP64 right-hand side (point values, surplus passes, transforms, reduction) "
                               f"on the final grid ({rhs_E} elements, {rhs_dof} DOF)",
                     "kernel_ms": rhs_sec * 1e3, "algorithmic_bytes_per_launch": 233.0 * rhs_dof,
                     "algorithmic_flops": rhs_flops, "fp64_tflops": rhs_flops / rhs_sec / 1e12,
                     "fp64_peak_tflops_measured": fp64_peak, "fp64_frac": rhs_flops / rhs_sec / 1e12 / fp64_peak,
                     "mixed_rhs_ms": rhs32_sec * 1e3,
                     "note": "L2-resident working set: the FP64 pipe binds, not HBM (fp64_frac against the "
                             "measured float64 GEMM rate)"},
        "e2e": {"value": units / e2e_sec, "unit": "DOF-stage updates/s",
                "h2d_bytes_per_step": 8 * 22464, "d2h_bytes_per_step": 8 * e2e[-1]["dof_final"],
                "call": "amdg_grid_set_coefficients from pinned host memory, 36 amdg_burgers_adaptive_step calls, "
                        "amdg_grid_get_coefficients into pinned host memory"},
        "gpu_launches": sum(r["launches"] for r in runs),
        "host_phase_ms_per_run": runs[-1]["host_phase_ms"],
        "clocks": clocks,
    }
    if args.learn_runs > 0:
        line["burgers3d_adaptive"] = bench_config3_arms(cfg, args, plain)
        m = line["burgers3d_adaptive"]["metric"]
        line["metric_at_matched_error"] = {k: v for k, v in m.items()
                                           if k != "network_gain_vs_criterion_same_horizon_and_eps"}
    line.update(bench_linear_small(ctx, stream, args))
    lin = bench_linear6d(ctx, stream, args, world)
    lin_cpu = lin.pop("_cpu")
    line["linear6d"] = lin
    line["burgers3d"] = bench_burgers(ctx, stream, args)
    if args.batch_solves > 0:
        line["batched"] = bench_batched(ctx, stream, args)
    if args.wave_learn_runs > 0:
        line["wave2d_adaptive"] = bench_wave_adaptive(ctx, stream, args)
    if args.herm_runs > 0:
        line["burgers2d_hermite_adaptive"] = bench_herm_adaptive(ctx, stream, args)
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline_config3(args)
        line["linear6d"]["cpu_baseline"] = cpu_baseline(*lin_cpu[:2], budget_s=args.cpu_seconds)
    lin_cpu[2].close()
    lin_cpu[0].close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def bench_burgers(ctx, stream, args):
    """3D inviscid Burgers, 0.5 + 0.25 sin(2 pi (x+y+z)), sparse grid N=8 (no
    adaptivity), Lagrange degree-3 flux interpolation, LxF alpha = 1.1 max|u|,
    SSP-RK3, dt = CFL 0.1 / (max|u| sum_d 2^N): DOF-stage updates/s in both modes."""
    import torch

    import amdg
    import amdg_oracle as O
    dim, N = 3, 8
    g = amdg.Grid(ctx, dim, N, 2)
    g.init_separable(O.burgers_ic_terms(dim))
    u0 = g.coefficients().reshape(-1).copy()
    umax = 0.75
    op = amdg.BurgersOperator(g, 1.1 * umax)
    dt = CFL / (umax * dim * (1 << N))
    out = {"workload": "3D Burgers, sparse grid N=8 (4096 elements, 110,592 DOF), Lagrange m=3, LxF, SSP-RK3",
           "dof": g.dof}
    for name, prec in (("fp64", amdg.FP64), ("mixed", amdg.MIXED)):
        g.set_coefficients(u0)
        op.rk3_steps(dt, args.warmup, prec)
        g.set_coefficients(u0)
        torch.cuda.synchronize()
        l0 = ctx.launch_count()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        op.rk3_steps(dt, args.steps, prec)
        e.record(stream)
        torch.cuda.synchronize()
        sec = s.elapsed_time(e) / 1e3
        out[name] = {"value": 3.0 * g.dof * args.steps / sec, "ms_per_step": sec / args.steps * 1e3,
                     "launches_per_step": (ctx.launch_count() - l0) / args.steps}
    ref = g.coefficients().reshape(-1).copy()
    g.set_coefficients(u0)
    op.rk3_steps(dt, args.steps, amdg.FP64)
    ctx.synchronize()
    u64 = g.coefficients().reshape(-1)
    g.set_coefficients(u0)
    op.rk3_steps(dt, args.steps, amdg.MIXED)
    ctx.synchronize()
    u32 = g.coefficients().reshape(-1)
    out["mixed_vs_fp64_rel_l2"] = float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64))
    del ref
    op.close()
    g.close()
    return out


HERM2D = {"n_init": 3, "nmax": 8, "eps": 1e-5, "eta": 1e-6, "alpha": 1.2, "cfl": 0.2, "T": 0.03}


def ref_herm_steps(nsteps: int, threads: int):
    """The reference's adaptive 2D Hermite Burgers loop (02_hyperbolic_05_burgers_adapt.cpp), timing
    mode: per time step the wall seconds and the DOF its RK stages advanced."""
    c = HERM2D
    cmd = [REF_HARNESS, "burgers_herm_adapt", str(c["n_init"]), str(c["nmax"]), repr(c["eps"]), repr(c["eta"]),
           repr(c["alpha"]), repr(c["cfl"]), str(nsteps), "time", repr(c["T"])]
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    res = subprocess.run(cmd, env=env, capture_output=True, text=True, check=True)
    return [(float(f[2]), int(f[3])) for f in (ln.split() for ln in res.stdout.splitlines()) if f and f[0] == "TSTEP"]


def bench_herm_adaptive(ctx, stream, args):
    """2D adaptive Burgers with the flux interpolated by cubic Hermite interpolation: the loop of
    example/02_hyperbolic_05_burgers_adapt.cpp without artificial viscosity (u0 = sin(2 pi (x+y)),
    start level 3, max level 8, refine 1e-5, coarsen 1e-6, LxF 1.2, CFL 0.2 with wave speed 1,
    to T = 0.03, 34 steps).  DOF-stage updates/s of whole runs (CUDA events, initialisation
    excluded) in FP64 and mixed precision, beside the reference's own loop on the host cores."""
    import torch

    import amdg
    import amdg_oracle as O
    c = HERM2D
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def one(prec):
        g = amdg.Grid(ctx, 2, c["nmax"], 2, level_init=c["n_init"])
        g.init_separable_adaptive(O.sin_sum_terms(2), c["eps"])
        op = amdg.BurgersOperator(g, c["alpha"], hermite=True)
        ctx.synchronize()
        flush.fill_(1)
        torch.cuda.synchronize()
        sd0, _ = op.counters()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t, steps = 0.0, 0
        while t < c["T"] - 1e-12:
            lv = g.max_mesh_level()
            dt_full = c["cfl"] / sum(2.0 ** int(m) for m in lv)
            cfl = c["cfl"] if t + dt_full <= c["T"] else c["cfl"] * (c["T"] - t) / dt_full
            t += op.adaptive_step(cfl, 1.0, c["eps"], c["eta"], prec)
            steps += 1
        ev1.record(stream)
        ev1.synchronize()
        sd1, _ = op.counters()
        res = {"sec": ev0.elapsed_time(ev1) / 1e3, "stage_dof_updates": sd1 - sd0, "steps": steps,
               "elements_final": g.num_elements, "u": g.coefficients().reshape(-1).copy()}
        op.close()
        g.close()
        return res

    out = {"workload": "2D adaptive Burgers, cubic Hermite flux interpolation (HermInterpolation + "
                       "HyperbolicSameFluxHermRHS), u0 = sin(2 pi (x+y)), start level 3, max level 8, refine 1e-5, "
                       "coarsen 1e-6, LxF alpha 1.2, CFL 0.2, to T = 0.03"}
    finals = {}
    for name, prec in (("fp64", amdg.FP64), ("mixed", amdg.MIXED)):
        for _ in range(max(1, args.warmup)):
            one(prec)
        runs = [one(prec) for _ in range(args.herm_runs)]
        sec = sum(r["sec"] for r in runs)
        out[name] = {"value": sum(r["stage_dof_updates"] for r in runs) / sec, "ms_per_run": sec / len(runs) * 1e3,
                     "steps": runs[-1]["steps"], "elements_final": runs[-1]["elements_final"]}
        finals[name] = runs[-1]["u"]
    if finals["fp64"].shape == finals["mixed"].shape:
        out["mixed_vs_fp64_rel_l2"] = float(np.linalg.norm(finals["mixed"] - finals["fp64"]) /
                                            np.linalg.norm(finals["fp64"]))
    out["mixed_speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    if ensure_ref_harness():
        cores = os.cpu_count() or 1
        steps = ref_herm_steps(args.cpu_steps + 2, cores)
        sec = sum(x[0] for x in steps)
        ref = sum(3.0 * x[1] for x in steps) / sec
        out["reference_cpu"] = {"value": ref, "unit": "DOF-stage updates/s", "cores": cores, "kind": "reference",
                                "sample": f"the first {len(steps)} time steps of the same run (AdaM-DG built from its "
                                          f"sources on this host, {cores} OpenMP threads), {sec:.1f} s"}
        out["fp64_vs_reference_cpu"] = out["fp64"]["value"] / ref
    return out


def wave_ic_terms(dim, a, b, c):
    """a + b sin(2 pi (sum_d x_d + c)) as separable terms."""
    import amdg_oracle as O
    terms = [lambda x, d, a=a: a if d == 0 else 1.0]
    for f in O.sin_sum_terms(dim, shift=-c):
        terms.append(lambda x, d, f=f, b=b: (b if d == 0 else 1.0) * f(x, d))
    return terms


CONFIG3 = {"dim": 3, "nmax": 8, "level_init": 3, "eps": 1e-5, "eta": 1e-6, "T": 0.05, "umax": 0.75, "alpha": 0.825,
           "cfl": 0.1, "tau": 0.8}
WORKLOAD3 = ("3D adaptive Burgers u_t + div(u^2/2 (1,1,1)) = 0 on the periodic unit cube, u0 = 0.5 + 0.25 "
             "sin(2 pi (x+y+z)), Alpert k=2, Lagrange degree-3 flux interpolation, LxF alpha 0.825, SSP-RK3, CFL 0.1, "
             "refine 1e-5, coarsen 1e-6, start level 3, max level 8, to T = 0.05")


class Config3:
    """Runs of the 3D adaptive Burgers workload to T = 0.05 (the reference's adaptive loop:
    predictor, refine, SSP-RK3, coarsen; or the learned / criterion pre-adaptation over a
    horizon).  A run's timed region is the evolution loop only (initialisation and error
    evaluation excluded), bracketed by CUDA events on the library's stream after an L2 flush."""

    def __init__(self, ctx, stream):
        import torch
        self.ctx, self.stream, self.torch = ctx, stream, torch
        self.flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def make(self):
        import amdg
        import amdg_oracle as O
        c = CONFIG3
        g = amdg.Grid(self.ctx, c["dim"], c["nmax"], 2, level_init=c["level_init"])
        g.init_separable_adaptive(O.burgers_ic_terms(c["dim"]), c["eps"])
        return g, amdg.BurgersOperator(g, c["alpha"])

    def run(self, prec, mlp=None, horizon=0, keep=False, host_io=None, t_end=None, eps=None):
        """horizon 0: the plain adaptive step; horizon >= 1: one pre-adaptation (classifier `mlp`, or
        the criterion alone when mlp is None) then `horizon` steps.  host_io = (pinned input,
        pinned output): the state is copied in from host memory at the start of the timed region
        and out at its end (the end-to-end form)."""
        torch, ctx, c = self.torch, self.ctx, dict(CONFIG3)
        g, op = self.make()  # the initial grid is the workload's (refine 1e-5)
        if eps is not None:  # the adaptivity of the run itself
            c["eps"], c["eta"] = eps, eps / 10.0
        t_end = c["T"] if t_end is None else t_end
        if host_io is not None:
            host_io[0][:g.dof] = g.coefficients().reshape(-1)
        ctx.synchronize()
        self.flush_buf.fill_(1)
        torch.cuda.synchronize()
        sd0, rhs0 = op.counters()
        l0 = ctx.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ctx.profile(True)
        ev0.record(self.stream)
        w0 = time.perf_counter()
        if host_io is not None:
            g.set_coefficients(host_io[0][:g.dof])
        t, steps, cls = 0.0, 0, np.zeros(3, np.int64)
        while t < t_end - 1e-12:
            if horizon >= 1:
                dt, n, st = op.adaptive_steps_learned(mlp, c["cfl"], c["umax"], c["eps"], c["eta"],
                                                      c["tau"] if mlp is not None else 2.0, horizon, t_end - t, prec)
                cls += st[:3]
                t += dt
                steps += n
                continue
            lv = g.max_mesh_level()
            dt_full = c["cfl"] / sum(c["umax"] * 2.0 ** int(m) for m in lv)
            cfl = c["cfl"] if t + dt_full <= t_end else c["cfl"] * (t_end - t) / dt_full
            t += op.adaptive_step(cfl, c["umax"], c["eps"], c["eta"], prec)
            steps += 1
        if host_io is not None:
            g.coefficients(out=host_io[1])
        ev1.record(self.stream)
        ev1.synchronize()
        wall = time.perf_counter() - w0
        prof = ctx.profile_read()
        ctx.profile(False)
        sd1, rhs1 = op.counters()
        res = {"sec": ev0.elapsed_time(ev1) / 1e3, "wall_s": wall, "steps": steps, "t_end": t,
               "stage_dof_updates": sd1 - sd0, "rhs_evaluations": rhs1 - rhs0, "launches": ctx.launch_count() - l0,
               "elements_final": g.num_elements, "dof_final": g.dof,
               "host_phase_ms": {k: round(v[0] * 1e3, 3) for k, v in prof.items() if v[1]}}
        if horizon >= 1:
            res["pre_adaptation"] = {"net_refine": int(cls[0]), "unsure": int(cls[1]), "missed_refinements": int(cls[2])}
        if keep:
            res["error_vs_exact_l1_l2_linf"] = [float(v) for v in g.error_burgers(t, gauss_points=2)]
            res["_grid"], res["_op"] = g, op
        else:
            op.close()
            g.close()
        return res


def config3_rhs_timing(cfg, prec, reps=20):
    """Average device time of one right-hand side on the final grid of a plain run (CUDA events)."""
    import torch
    r = cfg.run(prec, keep=True)
    g, op = r["_grid"], r["_op"]
    du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(cfg.stream)
    for _ in range(reps):
        op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    ev1.record(cfg.stream)
    ev1.synchronize()
    sec = ev0.elapsed_time(ev1) / 1e3 / reps
    dof, E = g.dof, g.num_elements
    flops, pairs = op.work()
    op.close()
    g.close()
    return sec, dof, E, flops


def train_config3_classifier(cfg, args, horizon, eps):
    """The classifier of a learned arm, trained on the decisions of plain FP64 runs (refine eps,
    coarsen eps/10) of other seeded waves a + b sin(2 pi (x+y+z+c)) (horizon labels: refine where
    the criterion refines the element within the next `horizon` steps)."""
    import torch

    import amdg
    c = CONFIG3
    dim = c["dim"]
    F = 27 * (1 + 2 * dim)
    ctx = cfg.ctx
    t0 = time.perf_counter()
    rng = np.random.default_rng(1)
    feats, labs = [], []
    for _ in range(args.learn_runs):
        a, b, cc = rng.uniform(0.4, 0.6), rng.uniform(0.15, 0.3), rng.uniform(0.0, 1.0)
        g = amdg.Grid(ctx, dim, c["nmax"], 2, level_init=c["level_init"])
        g.init_separable_adaptive(wave_ic_terms(dim, a, b, cc), c["eps"])
        op = amdg.BurgersOperator(g, 1.1 * (a + b))
        keys_steps, dec_steps = [], []
        for _s in range(args.learn_steps):
            buf = torch.empty(g.num_elements * F, dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            op.features_device(g.device_ptr(), buf.data_ptr())
            ctx.synchronize()
            feats.append(buf.cpu().numpy().reshape(-1, F))
            keys_steps.append(element_keys(g))
            _dt, dec = op.adaptive_step_ex(c["cfl"], a + b, eps, eps / 10.0)
            dec_steps.append(np.asarray(dec))
        labs.extend(horizon_labels(keys_steps, dec_steps, horizon))
        op.close()
        g.close()
    x, y = np.concatenate(feats), np.concatenate(labs)
    collect_s = time.perf_counter() - t0
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    torch.cuda.synchronize()
    mlp = amdg.MLP(ctx, F, 64, 3, 3, seed=11)
    t0 = time.perf_counter()
    loss = mlp.train_device(dx.data_ptr(), dy.data_ptr(), len(y), epochs=args.learn_epochs, batch=256, lr=2e-3,
                            seed=12)
    info = {"runs": args.learn_runs, "steps_per_run": args.learn_steps, "horizon": horizon, "refine_eps": eps,
            "samples": int(len(y)), "class_counts": [int((y == i).sum()) for i in range(3)],
            "epochs": args.learn_epochs, "final_loss": loss, "collect_s": collect_s,
            "train_s": time.perf_counter() - t0}
    return mlp, info


def bench_config3_arms(cfg, args, plain):
    """The metric itself: wall time to T of mixed precision with learned adaptivity against the plain
    FP64 path at matched error (final L2 error against the exact solution within 10 % of the plain
    path's).  Arms with a pre-adaptation over a horizon (classifier, or the surplus criterion alone:
    what the network itself gains) run at refine thresholds eps = s x 1e-5 (coarsen eps/10), the
    classifier trained at the same eps.  Per horizon: the scales of --eps-scales, then up to
    --eps-bisect bisection steps on s between the two neighbouring scales whose learned-arm error
    ratios bracket 1 (when none of them matched).  A learned arm counts for the metric only at
    matched error; the network's own gain is the best matched criterion-only arm's time over the
    best matched learned arm's (both over all horizons and scales tried)."""
    import amdg
    out = {"plain_fp64": plain}
    ref_err = plain["error_vs_exact_l1_l2_linf"][1]

    def measure(prec, net, h, eps):
        t_short = 4 * CONFIG3["cfl"] / (CONFIG3["umax"] * 3 * 32)
        try:
            cfg.run(prec, mlp=net, horizon=h, t_end=t_short, eps=eps)  # warm-up
            runs = [cfg.run(prec, mlp=net, horizon=h, keep=(i == 0), eps=eps) for i in range(args.arm_runs)]
        except amdg.AmdgError as ex:  # e.g. a solution that blew up on a pre-adapted grid
            return {"failed": str(ex), "horizon": h, "refine_eps": eps, "matched_error": False}
        r = runs[0]
        g, op = r.pop("_grid"), r.pop("_op")
        op.close()
        g.close()
        secs = sorted(x["sec"] for x in runs)
        r["sec"] = secs[len(secs) // 2]
        r["sec_runs"] = secs
        r["value"] = r["stage_dof_updates"] / r["sec"]
        r["horizon"], r["refine_eps"] = h, eps
        r["error_ratio_vs_plain_fp64"] = r["error_vs_exact_l1_l2_linf"][1] / ref_err
        r["wall_speedup_vs_plain_fp64"] = plain["sec"] / r["sec"]
        r["dof_stage_speedup_vs_plain_fp64"] = r["value"] / plain["value"]
        r["matched_error"] = bool(0.9 <= r["error_ratio_vs_plain_fp64"] <= 1.1)
        return r

    out["mixed_plain"] = measure(amdg.MIXED, None, 0, None)
    trainings = []

    def arms_at(h, scale):
        eps = 1e-5 * scale
        mlp, info = train_config3_classifier(cfg, args, h, eps)
        trainings.append(info)
        out[f"mixed_learned_h{h}_s{scale:g}"] = lr = measure(amdg.MIXED, mlp, h, eps)
        out[f"mixed_criterion_h{h}_s{scale:g}"] = measure(amdg.MIXED, None, h, eps)
        mlp.close()
        return lr.get("error_ratio_vs_plain_fp64", float("inf")), lr["matched_error"]

    for h in args.arm_horizons:
        tried = sorted((s, arms_at(h, s)) for s in args.eps_scales)
        if any(m for _, (_, m) in tried):
            continue
        lo = hi = None
        for (s0, (r0, _)), (s1, (r1, _)) in zip(tried, tried[1:]):
            if r0 < 1.0 < r1:
                lo, hi = s0, s1
                break
        for _ in range(args.eps_bisect if lo is not None else 0):
            mid = round(0.5 * (lo + hi), 4)
            ratio, matched = arms_at(h, mid)
            if matched:
                break
            lo, hi = (mid, hi) if ratio < 1.0 else (lo, mid)
    out["training"] = trainings

    def best(prefix):
        keys = [k for k in out if k.startswith(prefix) and out[k]["matched_error"]]
        return max(keys, key=lambda k: out[k]["wall_speedup_vs_plain_fp64"]) if keys else None

    bl, bc = best("mixed_learned"), best("mixed_criterion")
    gain = {}
    for k in out:
        if k.startswith("mixed_learned"):
            crit = k.replace("learned", "criterion")
            if "sec" in out[k] and "sec" in out[crit]:
                gain[k] = out[crit]["sec"] / out[k]["sec"]
    out["metric"] = {
        "definition": "wall time to T = 0.05 of the plain FP64 path over that of mixed precision + learned "
                      "adaptivity, counting only arms whose final L2 error vs exact is within 10 % of the plain "
                      "path's; the north-star target is 5x",
        "best_matched_arm": bl,
        "wall_speedup": out[bl]["wall_speedup_vs_plain_fp64"] if bl else None,
        "dof_stage_speedup": out[bl]["dof_stage_speedup_vs_plain_fp64"] if bl else None,
        "error_ratio": out[bl]["error_ratio_vs_plain_fp64"] if bl else None,
        "best_matched_criterion_only_arm": bc,
        "criterion_only_wall_speedup": out[bc]["wall_speedup_vs_plain_fp64"] if bc else None,
        "network_gain_at_matched_error": (out[bc]["sec"] / out[bl]["sec"]) if (bl and bc) else None,
        "network_gain_vs_criterion_same_horizon_and_eps": gain,
    }
    return out


def bench_wave_adaptive(ctx, stream, args):
    """2D wave equation u_tt = div(c^2 grad u), c = 1 + 0.5 sin(2 pi x) sin(2 pi y), Gaussian bump
    exp(-200 |x - (0.3, 0.4)|^2) at rest, adaptive (refine 1e-5, coarsen 1e-6, max level 9, start
    level 3), IPDG sigma = 10, RK4ODE2nd, CFL 0.1, to T = --wave-time: the plain FP64 path
    (EulerODE2nd predictor, refine, RK4, coarsen) against mixed precision with the learned
    refine/coarsen classifier, trained on the plain criterion's decisions in 20 seeded runs (bump
    centre in [0.25, 0.75]^2, width parameter in [100, 300]).  No exact solution: each final
    solution is compared, on a 128^2 cell-centre mesh, with a plain FP64 run at max level 10 and
    the same thresholds."""
    import torch

    import amdg
    import amdg_oracle as O
    dim, nmax, level_init, eps, eta, sigma, T, tau, speed = 2, 9, 3, 1e-5, 1e-6, 10.0, args.wave_time, 0.8, 1.0
    F = 2 * 9 * (1 + 2 * dim)  # features of u and of u_t
    H = args.wave_learn_horizon
    out = {"workload": f"2D wave u_tt = div(c^2 grad u), c = 1 + 0.5 sin(2 pi x) sin(2 pi y), Gaussian bump at "
                       f"rest, adaptive (refine 1e-5, coarsen 1e-6, max level 9, start level 3), Alpert k=2, "
                       f"Lagrange degree 4 (msh_case 2 nodes), IPDG sigma 10, RK4ODE2nd, CFL 0.1, to T = {T}"}
    t0 = time.perf_counter()
    rng = np.random.default_rng(2)
    feats, labs = [], []
    for _ in range(args.wave_learn_runs):
        centre = tuple(rng.uniform(0.25, 0.75, 2))
        width = rng.uniform(100.0, 300.0)
        g = amdg.Grid(ctx, dim, nmax, 2, level_init=level_init)
        g.init_separable_adaptive(O.wave_ic_terms(dim, centre, width), eps)
        op = amdg.WaveOperator(g, sigma)
        keys_steps, dec_steps = [], []
        for _s in range(args.wave_learn_steps):
            buf = torch.empty(g.num_elements * F, dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            op.features_device(g.device_ptr(), buf.data_ptr())
            ctx.synchronize()
            feats.append(buf.cpu().numpy().reshape(-1, F))
            keys_steps.append(element_keys(g))
            _dt, dec = op.adaptive_step_ex(CFL, speed, eps, eta)
            dec_steps.append(np.asarray(dec))
        labs.extend(horizon_labels(keys_steps, dec_steps, args.wave_learn_horizon))
        op.close()
        g.close()
    x, y = np.concatenate(feats), np.concatenate(labs)
    collected = int(len(y))
    # the grids fill up, so the runs give millions of samples: keep every sample of the rare
    # classes (refine, coarsen) up to half the cap and fill the rest with "keep" samples
    cap = args.wave_train_samples
    if len(y) > cap:
        pick = np.random.default_rng(3)
        rare = np.flatnonzero(y != 1)
        if len(rare) > cap // 2:
            rare = pick.choice(rare, cap // 2, replace=False)
        keep = pick.choice(np.flatnonzero(y == 1), cap - len(rare), replace=False)
        idx = np.sort(np.concatenate([rare, keep]))
        x, y = x[idx], y[idx]
    collect_s = time.perf_counter() - t0
    dx, dy = torch.from_numpy(np.ascontiguousarray(x)).cuda(), torch.from_numpy(np.ascontiguousarray(y)).cuda()
    torch.cuda.synchronize()
    mlp = amdg.MLP(ctx, F, 64, 3, 3, seed=21)
    t0 = time.perf_counter()
    loss = mlp.train_device(dx.data_ptr(), dy.data_ptr(), len(y), epochs=args.learn_epochs, batch=256, lr=2e-3,
                            seed=22)
    out["training"] = {"runs": args.wave_learn_runs, "steps_per_run": args.wave_learn_steps, "horizon": H,
                       "samples_collected": collected, "samples": int(len(y)),
                       "class_counts": [int((y == i).sum()) for i in range(3)], "epochs": args.learn_epochs,
                       "final_loss": loss, "collect_s": collect_s, "train_s": time.perf_counter() - t0}
    mesh = (np.arange(128) + 0.5) / 128

    def run(learned, prec, t_end, e=eps, et=eta, nm=nmax, horizon=H):
        g = amdg.Grid(ctx, dim, nm, 2, level_init=level_init)
        g.init_separable_adaptive(O.wave_ic_terms(dim), e)
        op = amdg.WaveOperator(g, sigma)
        t, steps, cls = 0.0, 0, np.zeros(3, np.int64)
        ctx.synchronize()
        ctx.profile(True)
        t0 = time.perf_counter()
        while t < t_end - 1e-12:
            if learned:  # one pre-adaptation, then `horizon` steps (the last one landing on t_end)
                dt, n, st = op.adaptive_steps_learned(mlp, CFL, speed, e, et, tau, horizon, t_end - t, prec)
                cls += st[:3]
                t += dt
                steps += n
                continue
            lv = g.max_mesh_level()
            dt_full = CFL / sum(speed * 2.0 ** int(m) for m in lv)
            cfl = CFL if t + dt_full <= t_end else CFL * (t_end - t) / dt_full
            dt = op.adaptive_step(cfl, speed, e, et, prec)
            t += dt
            steps += 1
        ctx.synchronize()
        wall = time.perf_counter() - t0
        prof = ctx.profile_read()
        ctx.profile(False)
        stage_dof, rhs = op.counters()
        res = {"value": stage_dof / wall, "wall_s": wall, "steps": steps, "t_end": t, "stage_dof_updates": stage_dof,
               "rhs_evaluations": rhs, "elements_final": g.num_elements, "dof_final": g.dof,
               "host_phase_ms": {k: round(v[0] * 1e3, 3) for k, v in prof.items() if v[1]}}
        if t_end >= T:
            vals = torch.zeros(len(mesh) ** dim, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            g.eval_tensor_device(mesh, vals.data_ptr())
            ctx.synchronize()
            res["_mesh_values"] = vals.cpu().numpy()
        if learned:
            res["classifier"] = {"net_refine": int(cls[0]), "unsure": int(cls[1]), "missed_refinements": int(cls[2])}
        op.close()
        g.close()
        return res

    ref = None
    if not args.wave_no_level10:
        ref_run = run(False, amdg.FP64, T, eps, eta, 10)
        ref = ref_run.pop("_mesh_values")
        out["fp64_level10_run"] = {"what": "plain FP64 on this GPU (not the reference code), refine 1e-5, coarsen "
                                           "1e-6, max level 10",
                                   "wall_s": ref_run["wall_s"], "steps": ref_run["steps"],
                                   "elements_final": ref_run["elements_final"]}
    # the learned arm at the trained horizon ("mixed_learned") and at horizons 1 and 4
    arms = [("plain_fp64", False, amdg.FP64, 1), ("mixed_learned", True, amdg.MIXED, H)]
    if not args.wave_main_arms:
        arms += [(f"mixed_learned_h{h}", True, amdg.MIXED, h) for h in (1, 4) if h != H]
    arms += [("mixed_plain", False, amdg.MIXED, 1)]
    for name, learned, prec, horizon in arms:
        run(learned, prec, 4 * CFL / (speed * dim * 128), horizon=horizon)  # warm-up: a few steps
        out[name] = run(learned, prec, T, horizon=horizon)
        out[name]["horizon"] = horizon
        v = out[name].pop("_mesh_values")
        if ref is not None:
            out[name]["rel_l2_diff_vs_fp64_level10_run"] = float(np.linalg.norm(v - ref) / np.linalg.norm(ref))
        out[name]["_v"] = v
    base = out["plain_fp64"].pop("_v")
    for name in [a[0] for a in arms[1:]]:
        v = out[name].pop("_v")
        out[name]["rel_l2_diff_vs_plain_fp64"] = float(np.linalg.norm(v - base) / np.linalg.norm(base))
        if ref is not None:
            out[name]["error_ratio_vs_plain_fp64"] = (out[name]["rel_l2_diff_vs_fp64_level10_run"] /
                                                     out["plain_fp64"]["rel_l2_diff_vs_fp64_level10_run"])
        out[name]["speedup_vs_plain_fp64"] = out["plain_fp64"]["wall_s"] / out[name]["wall_s"]
    mlp.close()
    return out


def bench_batched(ctx, stream, args):
    """Batched serving: independent 3D linear advection solves, random velocity
    in [-1,1]^3, 1-4 periodic Gaussian bumps (centres U[0.2,0.8]^3, widths
    U[0.03,0.15]), adaptive grids up to level 8 (uneven sizes), all advanced by
    one graph-captured launch per RK stage; per-solve L2 error against the
    exact translated solution."""
    import torch

    import amdg
    import amdg_oracle as O
    work = O.batched_workload(args.batch_solves, seed=0)
    # each solve's refine threshold log-uniform in [batch_eps_min, batch_eps_max] (seeded): grid sizes
    # from about 10^3 to 10^5 elements
    lo, hi = math.log(args.batch_eps_min), math.log(args.batch_eps_max)
    eps_of = np.exp(np.random.default_rng(7).uniform(lo, hi, len(work)))
    t0 = time.perf_counter()
    grids = []
    for w, eps in zip(work, eps_of):
        g = amdg.Grid(ctx, 3, 8, 2, level_init=2)
        g.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], vectorized=True),
                                  float(eps), vectorized=True)
        grids.append(g)
    init_s = time.perf_counter() - t0
    sizes = [g.num_elements for g in grids]
    dts = []
    for g, w in zip(grids, work):
        lv = g.max_mesh_level()
        dts.append(CFL / sum(abs(v) * 2.0 ** int(m) for v, m in zip(w["velocity"], lv)))
    out = {"workload": f"{len(work)} independent 3D linear advection solves, adaptive N<=8, k=2, seed 0, "
                       f"refine threshold per solve log-uniform in [{args.batch_eps_min:g}, {args.batch_eps_max:g}]",
           "solves": len(work), "elements_min": min(sizes), "elements_max": max(sizes),
           "elements_median": int(np.median(sizes)), "elements_total": sum(sizes), "init_s": init_s}
    for name, prec in (("fp64", amdg.FP64), ("mixed", amdg.MIXED)):
        batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
        batch.set_dt(dts)
        batch.rk3_steps(args.warmup, prec, use_graph=True)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        batch.rk3_steps(args.steps, prec, use_graph=True)
        e.record(stream)
        torch.cuda.synchronize()
        sec = s.elapsed_time(e) / 1e3
        kernel, kernel_ms = batch.tuning()
        pi = 0 if prec == amdg.FP64 else 1
        stage_s = kernel_ms[pi][kernel[pi]] / 1e3
        # algorithmic bytes of one stage: 24 B per DOF (stage input, u^n, output) + 8 B per pair + 8 B per row
        stage_bytes = 24.0 * batch.dof + 8.0 * batch.pairs + 8.0 * (batch.num_elements * 3 + 1)
        pk, pk_kind = peaks()
        out[name] = {"value": 3.0 * batch.dof * args.steps / sec, "ms_per_step": sec / args.steps * 1e3,
                     "dof": batch.dof, "launches_per_step": 3,
                     "stage_kernel": amdg.Batch.kernel_name(kernel[pi]),
                     "stage_ms_by_kernel": {amdg.Batch.kernel_name(c): t for c, t in enumerate(kernel_ms[pi]) if t > 0},
                     "roofline": {"bound": "hbm", "achieved": stage_bytes / stage_s / 1e9, "peak": pk["hbm_gbs"],
                                  "unit": "GB/s", "frac": stage_bytes / stage_s / 1e9 / pk["hbm_gbs"],
                                  "peak_kind": pk_kind, "algorithmic_bytes_per_stage": stage_bytes}}
        errs = []
        nsteps = args.warmup + args.steps
        for i in range(0, len(work), max(1, len(work) // 16)):
            w = work[i]
            batch.store(i)
            shift = [v * dts[i] * nsteps for v in w["velocity"]]
            exact = O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], shift=shift, vectorized=True)
            norm = O.gaussian_bump_norm(w["centers"], w["widths"], w["amplitudes"])
            errs.append(grids[i].l2_error_separable_sum(exact, norm, vectorized=True) / norm)
        out[name]["rel_l2_error_sampled"] = {"median": float(np.median(errs)), "max": float(np.max(errs)),
                                             "solves_sampled": len(errs)}
        batch.close()
        # restore the initial coefficients for the next precision
        for g, w in zip(grids, work):
            g.init_separable(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], vectorized=True),
                             vectorized=True)
    for g in grids:
        g.close()
    if args.batch_adapt_every > 0:
        out["adaptive"] = bench_batched_adaptive(ctx, stream, args, work[:args.batch_adapt_solves])
    out["init_adaptive_intp"] = bench_init_intp(ctx)
    return out


def bench_init_intp(ctx):
    """Adaptive Lagrange-interpolation initialisation (degree 3) of exp(-50 |x - (0.3, 0.4, 0.5)|^2)
    on a 3D grid from the sparse grid of level 3 to level 8, refine 1e-5: wall time of the call
    (point values on the host, surpluses and the final transform on the device)."""
    import amdg
    c = np.array([0.3, 0.4, 0.5])

    def f(x):
        return np.exp(-50.0 * np.sum((x - c) ** 2, axis=1))

    res = {}
    for rep in range(2):  # the first call includes one-time table builds
        g = amdg.Grid(ctx, 3, 8, 2, level_init=3)
        ctx.synchronize()
        t0 = time.perf_counter()
        rounds = g.init_adaptive_intp(f, 1e-5, 3)
        ctx.synchronize()
        res = {"workload": "3D Gaussian bump, level 3 to 8, Lagrange degree 3, refine 1e-5",
               "wall_s": time.perf_counter() - t0, "rounds": rounds, "elements": g.num_elements, "dof": g.dof}
        g.close()
    return res


def grid_features(g) -> np.ndarray:
    """Classifier inputs of every element as the feature kernel computes them: log10(|c| + 1e-20)/20 + 1
    of the element's coefficients, then of its parent and grandparent in each dimension (0 where
    absent)."""
    keys = element_keys(g)
    B, dim, mask = g.block, g.dim, (1 << g.nmax) - 1
    mag = (np.log10(np.abs(g.coefficients().reshape(len(keys), B)) + 1e-20) / 20.0 + 1.0).astype(np.float32)
    srt = np.argsort(keys, kind="stable")
    F = np.zeros((len(keys), B * (1 + 2 * dim)), np.float32)
    F[:, :B] = mag
    for d in range(dim):
        shift = g.nmax * (dim - 1 - d)
        k = keys.copy()
        alive = np.ones(len(keys), bool)
        for gen in range(2):
            o = (k >> shift) & mask
            alive &= o > 0
            k = (k & ~(mask << shift)) | (np.where(o == 1, 0, o // 2) << shift)
            pos = np.minimum(np.searchsorted(keys[srt], k), len(keys) - 1)
            hit = alive & (keys[srt][pos] == k)
            slot = 1 + 2 * d + gen
            F[hit, slot * B:(slot + 1) * B] = mag[srt[pos[hit]]]
    return F


def refine_labels(g, eps) -> np.ndarray:
    """The criterion's choice for every element: 0 (refine) where its block norm exceeds eps, else
    1 (keep).  Coarsening stays on the criterion and refinement only touches leaves, so these
    are the decisions the classifier stands in for."""
    u = g.coefficients().reshape(g.num_elements, g.block)
    return np.where(np.sqrt(np.sum(u * u, axis=1)) > eps, 0, 1).astype(np.int32)


def bench_batched_adaptive(ctx, stream, args, work):
    """The batched solves with adaptivity inside the batch: every A steps each solve's grid is refined
    (surplus criterion, or the classifier with the criterion where it is unsure) and coarsened, and
    the batch rebuilt; "static" keeps the initial grids.  The classifier is trained on the
    criterion's decisions in a separate seeded batch.  Throughput counts the adaptation's time;
    errors against the exact translated bumps."""
    import torch

    import amdg
    import amdg_oracle as O
    A, eps, eta, tau = args.batch_adapt_every, args.batch_eps, args.batch_eps / 10, 0.8
    nsteps = args.batch_adapt_rounds * A

    def make(ws):
        gs = []
        for w in ws:
            g = amdg.Grid(ctx, 3, 8, 2, level_init=2)
            g.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"],
                                                            vectorized=True), eps, vectorized=True)
            gs.append(g)
        return gs

    def dts_of(gs, ws):
        return [CFL / sum(abs(v) * 2.0 ** int(m) for v, m in zip(w["velocity"], g.max_mesh_level()))
                for g, w in zip(gs, ws)]

    # training data: the criterion's decisions on another seeded set of solves
    t0 = time.perf_counter()
    train = O.batched_workload(min(32, len(work)), seed=1)
    gs = make(train)
    batch = amdg.Batch(ctx, gs, [w["velocity"] for w in train])
    feats, labs = [], []
    for _ in range(max(2, args.batch_adapt_rounds - 2)):
        batch.set_dt(dts_of(gs, train))
        batch.rk3_steps(A, amdg.MIXED, use_graph=True)
        for i in range(len(train)):
            batch.store(i)
        feats += [grid_features(g) for g in gs]
        labs += [refine_labels(g, eps) for g in gs]
        batch.adapt(eps, eta)
    batch.close()
    for g in gs:
        g.close()
    x, y = np.concatenate(feats), np.concatenate(labs)
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    torch.cuda.synchronize()
    mlp = amdg.MLP(ctx, x.shape[1], 64, 3, 3, seed=31)
    loss = mlp.train_device(dx.data_ptr(), dy.data_ptr(), len(y), epochs=args.learn_epochs, batch=256, lr=2e-3,
                            seed=32)
    out = {"solves": len(work), "adapt_every_steps": A, "steps": nsteps, "refine_eps": eps, "coarsen_eta": eta, "tau": tau,
           "training": {"solves": len(train), "samples": int(len(y)),
                        "class_counts": [int((y == i).sum()) for i in range(3)], "final_loss": loss,
                        "s": time.perf_counter() - t0}}
    for name, learned in (("static", None), ("criterion", False), ("learned", True)):
        gs = make(work)
        batch = amdg.Batch(ctx, gs, [w["velocity"] for w in work])
        elapsed = np.zeros(len(work))
        dof_stages = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = np.zeros(2, np.int64)
        sizes, adapt_s = [batch.num_elements], 0.0
        ctx.profile(True)
        for _ in range(nsteps // A):
            dts = dts_of(gs, work)
            batch.set_dt(dts)
            batch.rk3_steps(A, amdg.MIXED, use_graph=True)
            dof_stages += 3.0 * batch.dof * A
            elapsed += np.asarray(dts) * A
            if learned is None:
                continue
            t1 = time.perf_counter()
            st = batch.adapt(eps, eta, mlp if learned else None, tau)
            adapt_s += time.perf_counter() - t1
            stats += st[:2]
            sizes.append(int(st[2]))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        prof = ctx.profile_read()
        ctx.profile(False)
        errs = []
        for i in range(0, len(work), max(1, len(work) // 16)):
            w = work[i]
            batch.store(i)
            shift = [v * elapsed[i] for v in w["velocity"]]
            exact = O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], shift=shift, vectorized=True)
            norm = O.gaussian_bump_norm(w["centers"], w["widths"], w["amplitudes"])
            errs.append(gs[i].l2_error_separable_sum(exact, norm, vectorized=True) / norm)
        out[name] = {"value": dof_stages / wall, "wall_s": wall, "adapt_s": adapt_s, "elements_by_adaptation": sizes,
                     "host_phase_ms": {k: round(v[0] * 1e3, 3) for k, v in prof.items() if v[1]},
                     "rel_l2_error_sampled": {"median": float(np.median(errs)), "max": float(np.max(errs))}}
        if learned:
            out[name]["classifier"] = {"net_refine": int(stats[0]), "unsure": int(stats[1])}
        batch.close()
        for g in gs:
            g.close()
    mlp.close()
    return out


def profile_wave_rhs():
    """Profiling case of the wave right-hand side (not a bench line): the 2D adaptive wave grid
    after 40 plain adaptive steps (max level 9, refine 1e-5, coarsen 1e-6; about 20,000
    elements), RHS times in FP64 and mixed, then one FP64 and one mixed right-hand side between
    cudaProfilerStart / cudaProfilerStop, for ncu --profile-from-start off."""
    import torch

    import amdg
    import amdg_oracle as O
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    g = amdg.Grid(ctx, 2, 9, 2, level_init=3)
    g.init_separable_adaptive(O.wave_ic_terms(2), 1e-5)
    op = amdg.WaveOperator(g, 10.0)
    for _ in range(40):
        op.adaptive_step(CFL, 1.0, 1e-5, 1e-6)
    ctx.synchronize()
    du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    for prec in (amdg.FP64, amdg.MIXED):
        op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    ctx.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for prec, name in ((amdg.FP64, "fp64"), (amdg.MIXED, "mixed")):
        s.record(stream)
        for _ in range(20):
            op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
        e.record(stream)
        torch.cuda.synchronize()
        print(json.dumps({"elements": g.num_elements, "dof": g.dof, f"rhs_{name}_ms": s.elapsed_time(e) / 20}),
              flush=True)
    torch.cuda.cudart().cudaProfilerStart()
    op.rhs_device(du.data_ptr(), out.data_ptr(), amdg.FP64)
    op.rhs_device(du.data_ptr(), out.data_ptr(), amdg.MIXED)
    ctx.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    op.close()
    g.close()


def profile_config3():
    """Profiling case (not a bench line): one plain FP64 and one mixed run of the 3D adaptive Burgers
    workload after a warm-up run each, between cudaProfilerStart / cudaProfilerStop, for
    ncu --profile-from-start off."""
    import torch

    import amdg
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    cfg = Config3(ctx, stream)
    for prec in (amdg.FP64, amdg.MIXED):
        cfg.run(prec)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    for prec in (amdg.FP64, amdg.MIXED):
        r = cfg.run(prec)
        print(json.dumps({"prec": int(prec), "ms": r["sec"] * 1e3, "launches": r["launches"]}), flush=True)
    torch.cuda.cudart().cudaProfilerStop()


def profile_herm():
    """Profiling case (not a bench line): one plain FP64 and one mixed run of the 2D adaptive
    Hermite Burgers workload (max level 8 to T = 0.03) after a warm-up run each, between
    cudaProfilerStart / cudaProfilerStop, for ncu --profile-from-start off."""
    import torch

    import amdg
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    import amdg_oracle as O
    c = HERM2D

    def one(prec):
        g = amdg.Grid(ctx, 2, c["nmax"], 2, level_init=c["n_init"])
        g.init_separable_adaptive(O.sin_sum_terms(2), c["eps"])
        op = amdg.BurgersOperator(g, c["alpha"], hermite=True)
        ctx.synchronize()
        l0 = ctx.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t = 0.0
        while t < c["T"] - 1e-12:
            dt_full = c["cfl"] / sum(2.0 ** int(m) for m in g.max_mesh_level())
            cfl = c["cfl"] if t + dt_full <= c["T"] else c["cfl"] * (c["T"] - t) / dt_full
            t += op.adaptive_step(cfl, 1.0, c["eps"], c["eta"], prec)
        ev1.record(stream)
        ev1.synchronize()
        res = {"prec": int(prec), "ms": ev0.elapsed_time(ev1), "launches": ctx.launch_count() - l0,
               "elements_final": g.num_elements}
        op.close()
        g.close()
        return res

    for prec in (amdg.FP64, amdg.MIXED):
        one(prec)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    for prec in (amdg.FP64, amdg.MIXED):
        print(json.dumps(one(prec)), flush=True)
    torch.cuda.cudart().cudaProfilerStop()


def profile_rhs_config3():
    """Profiling case (not a bench line): one FP64 and one mixed right-hand side on the final grid of
    a plain 3D adaptive Burgers run (1,004 elements), each after a warm-up evaluation, between
    cudaProfilerStart / cudaProfilerStop (the dozen kernels of each, for DRAM traffic per RHS)."""
    import torch

    import amdg
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    cfg = Config3(ctx, stream)
    r = cfg.run(amdg.FP64, keep=True)
    g, op = r["_grid"], r["_op"]
    du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
    out = torch.zeros_like(du)
    for prec in (amdg.FP64, amdg.MIXED):
        op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    torch.cuda.cudart().cudaProfilerStart()
    for prec in (amdg.FP64, amdg.MIXED):
        op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({"elements": g.num_elements, "dof": g.dof, "launches": ctx.launch_count() - l0}), flush=True)
    op.close()
    g.close()


def profile_batch():
    """Profiling case (not a bench line): 64 of the batched solves (per-solve refine thresholds
    log-uniform in [1e-8, 1e-5], adaptive N<=8), one mixed SSP-RK3 step with the autotuner's stage
    kernel between cudaProfilerStart / cudaProfilerStop, stage times per candidate first."""
    import torch

    import amdg
    import amdg_oracle as O
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    work = O.batched_workload(64, seed=0)
    eps_of = np.exp(np.random.default_rng(7).uniform(math.log(1e-8), math.log(1e-5), len(work)))
    grids = []
    for w, eps in zip(work, eps_of):
        g = amdg.Grid(ctx, 3, 8, 2, level_init=2)
        g.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], vectorized=True),
                                  float(eps), vectorized=True)
        grids.append(g)
    dts = [CFL / sum(abs(v) * 2.0 ** int(m) for v, m in zip(w["velocity"], g.max_mesh_level()))
           for g, w in zip(grids, work)]
    batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
    batch.set_dt(dts)
    kernel, ms = batch.tuning()
    print(json.dumps({"elements": batch.num_elements, "dof": batch.dof, "pairs": batch.pairs,
                      "mixed_kernel": amdg.Batch.kernel_name(kernel[1]),
                      "stage_ms": {amdg.Batch.kernel_name(c): t for c, t in enumerate(ms[1]) if t > 0}}), flush=True)
    batch.rk3_steps(1, amdg.MIXED, use_graph=False)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    batch.rk3_steps(1, amdg.MIXED, use_graph=False)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    batch.close()
    for g in grids:
        g.close()


def profile_linear6d():
    """Profiling case (not a bench line): one mixed SSP-RK3 step of the 6D N=8 linear workload with
    the tensor-core variant (3 launches of linear_mma_kernel), then one with the bulk-copy FMA
    variant, between cudaProfilerStart / cudaProfilerStop; stage times by CUDA events first."""
    import torch

    import amdg
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    g = amdg.Grid(ctx, DIM, NMAX, K)
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    op = amdg.LinearOperator(g, COEF)
    dt = dt_for()
    op.rk3_steps(dt, 1, amdg.MIXED)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for v in (3, 2):
        op.set_variant(amdg.MIXED, v)
        op.rk3_steps(dt, 1, amdg.MIXED)
        ev0.record(stream)
        op.rk3_steps(dt, 4, amdg.MIXED)
        ev1.record(stream)
        ev1.synchronize()
        print(json.dumps({"variant": v, "stage_ms": ev0.elapsed_time(ev1) / 12, "dof": g.dof}), flush=True)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    for v in (3, 2):
        op.set_variant(amdg.MIXED, v)
        op.rk3_steps(dt, 1, amdg.MIXED)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    op.close()
    g.close()


def profile_rhs3d():
    """Profiling case (not a bench line): the 3D Burgers right-hand side on the sparse grid N=8
    (4096 elements), FP64 and mixed, with each transform-sweep kernel variant (0 thread per output,
    1 thread per column, 2 warp per term and element); times by CUDA events, then one right-hand
    side per (variant, precision) between cudaProfilerStart / Stop."""
    import torch

    import amdg
    import amdg_oracle as O
    torch.cuda.set_device(0)
    ctx = amdg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    g = amdg.Grid(ctx, 3, 8, 2)
    g.init_separable(O.burgers_ic_terms(3))
    op = amdg.BurgersOperator(g, 0.825)
    du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    flops, _ = op.work()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for variant in (0, 1, 2, 3, 4):
        op.set_sweep_variant(variant)
        for prec in (amdg.FP64, amdg.MIXED):
            op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
            ev0.record(stream)
            for _ in range(10):
                op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
            ev1.record(stream)
            ev1.synchronize()
            ms = ev0.elapsed_time(ev1) / 10
            print(json.dumps({"variant": variant, "prec": int(prec), "rhs_ms": ms, "elements": g.num_elements,
                              "flops": flops, "tflops": flops / ms / 1e9}), flush=True)
    torch.cuda.cudart().cudaProfilerStart()
    for variant in (0, 1, 2, 3, 4):
        op.set_sweep_variant(variant)
        for prec in (amdg.FP64, amdg.MIXED):
            op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    op.close()
    g.close()


def cpu_baseline(g, u0, budget_s=15.0):
    """Oracle (port of the reference algorithm) on the host cores: one RHS
    evaluation over a bounded, contiguous sample of elements of the same grid,
    repeated until ~budget_s of CPU time; DOF-stage updates/s."""
    import amdg_oracle as O
    lv, sp = g.elements()
    op = O.LinearOp(DIM, NMAX, K, lv, sp, COEF)
    cores = os.cpu_count() or 1
    u = u0.reshape(g.num_elements, -1)
    n_el = 4096
    e0 = g.num_elements // 2 - n_el // 2
    op.apply_range(u, e0, e0 + 64, cores)  # warm caches
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        op.apply_range(u, e0, e0 + n_el, cores)
        done += n_el
    sec = time.perf_counter() - t0
    op.close()
    return {"value": done * g.block / sec, "unit": "DOF-stage updates/s", "cores": cores, "kind": "port",
            "sample": f"{done} element-RHS evaluations (blocks of {n_el} contiguous elements of the 6D N=8 grid), "
                      f"{sec:.1f} s"}


REF_HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def ensure_ref_harness() -> bool:
    """The reference library's harness (oracle/Makefile: AdaM-DG built from its own sources in
    baseline/_ref): True when it runs on this host, building it first when it is missing or was
    built for another architecture."""
    def runs():
        try:
            return subprocess.run([REF_HARNESS], capture_output=True, timeout=60).returncode == 2
        except (OSError, subprocess.SubprocessError):
            return False
    if os.path.exists(REF_HARNESS) and runs():
        return True
    if not os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "source")):
        return False
    for stale in (REF_HARNESS, os.path.join(ROOT, "oracle", "_ref", "obj")):
        if os.path.isdir(stale):
            import shutil
            shutil.rmtree(stale)
        elif os.path.exists(stale):
            os.remove(stale)
    res = subprocess.run(["make", "-s", f"-j{os.cpu_count() or 1}", "-C", os.path.join(ROOT, "oracle"), "ref"],
                         capture_output=True, text=True)
    return res.returncode == 0 and runs()


def ref_config3_steps(nsteps: int, threads: int):
    """The reference's adaptive loop on the 3D Burgers workload, timing mode: per time step the wall
    seconds (evolution only) and the DOF its RK stages advanced."""
    c = CONFIG3
    cmd = [REF_HARNESS, "burgers_adapt", str(c["dim"]), str(c["level_init"]), str(c["nmax"]), repr(c["eps"]),
           repr(c["eta"]), repr(c["alpha"]), repr(c["cfl"]), repr(c["umax"]), str(nsteps), "time", repr(c["T"])]
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    res = subprocess.run(cmd, env=env, capture_output=True, text=True, check=True)
    return [(float(f[2]), int(f[3])) for f in (ln.split() for ln in res.stdout.splitlines()) if f and f[0] == "TSTEP"]


def cpu_baseline_config3(args):
    """The reference's own CPU loop on the host cores over a bounded sample of the headline
    workload (its first time steps); the oracle port when the reference cannot be built here."""
    cores = os.cpu_count() or 1
    if ensure_ref_harness():
        n = args.cpu_steps
        steps = ref_config3_steps(n, cores)
        sec = sum(x[0] for x in steps)
        return {"value": sum(3.0 * x[1] for x in steps) / sec, "unit": "DOF-stage updates/s", "cores": cores,
                "kind": "reference",
                "sample": f"the first {len(steps)} time steps of the 3D adaptive Burgers run (AdaM-DG built from its "
                          f"sources on this host, {cores} OpenMP threads), {sec:.1f} s of evolution"}
    import amdg_oracle as O
    c = CONFIG3
    t0 = time.perf_counter()
    hist = O.burgers_adaptive_run(c["dim"], c["level_init"], c["nmax"], c["eps"], c["eta"], c["alpha"], c["cfl"],
                                  c["umax"], 2)
    sec = time.perf_counter() - t0
    units = sum(3.0 * len(k) * 27 for k, _, _ in hist[1:])
    return {"value": units / sec, "unit": "DOF-stage updates/s", "cores": cores, "kind": "port",
            "sample": f"initialisation and 2 time steps of the oracle port, {sec:.1f} s"}


def run_reference(args):
    """The reference's own CPU implementation of the headline path (AdaM-DG's adaptive Burgers loop,
    built from its sources on this host) with every host thread; one bench step = one adaptive
    time step of the workload (a bounded sample), the first W of them untimed."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    c = CONFIG3
    if ensure_ref_harness():
        steps = ref_config3_steps(args.warmup + args.steps, cores)
        timed = steps[args.warmup:]
        kind = "reference"
        sample = (f"time steps {args.warmup}..{len(steps) - 1} of the 3D adaptive Burgers run, one per bench step "
                  f"(AdaM-DG built from its sources on this host, {cores} OpenMP threads)")
    else:
        import amdg_oracle as O
        timed = []
        keys, u = O.init_adaptive_separable(c["dim"], c["level_init"], c["nmax"], 2, O.burgers_ic_terms(c["dim"]),
                                            c["eps"])
        for _ in range(min(args.warmup + args.steps, 4)):
            t0 = time.perf_counter()
            hist = O.burgers_adaptive_run(c["dim"], c["level_init"], c["nmax"], c["eps"], c["eta"], c["alpha"],
                                          c["cfl"], c["umax"], 1)
            timed.append((time.perf_counter() - t0, len(hist[-1][0]) * 27))
        kind = "port"
        sample = "initialisation and one time step of the oracle port per bench step"
    sec = sum(x[0] for x in timed)
    value = sum(3.0 * x[1] for x in timed) / sec
    line = {
        "metric": METRIC, "value": value, "unit": "DOF-stage updates/s", "n_gpus": world, "steps": len(timed),
        "warmup": args.warmup, "ms_per_step": sec / len(timed) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: IC 0.5 + 0.25 sin(2 pi (x+y+z)) projected onto the adaptive grid",
        "config": {"workload": WORKLOAD3, **{k: v for k, v in CONFIG3.items() if k != "tau"},
                   "step": "one adaptive time step of the run (predictor, refine, SSP-RK3, coarsen)"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "DOF-stage updates/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "DOF-stage updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-steps", type=int, default=4, help="time steps of the reference loop in cpu_baseline")
    ap.add_argument("--arm-runs", type=int, default=3, help="timed runs per arm of the 3D adaptive Burgers metric")
    ap.add_argument("--arm-horizons", type=int, nargs="+", default=[8, 12],
                    help="horizons of the pre-adapted arms of the 3D adaptive Burgers metric")
    ap.add_argument("--arm-tau", type=float, default=CONFIG3["tau"],
                    help="probability at or above which the classifier's refine decision replaces the criterion's "
                         "in the learned arms of the 3D adaptive Burgers metric")
    ap.add_argument("--eps-scales", type=float, nargs="+", default=[1.5, 2, 2.25, 2.5],
                    help="refine thresholds of the pre-adapted arms, in units of 1e-5")
    ap.add_argument("--eps-bisect", type=int, default=3,
                    help="bisection steps on the refine threshold of a horizon whose scales matched no error")
    ap.add_argument("--batch-solves", type=int, default=256)
    ap.add_argument("--batch-eps", type=float, default=1e-5, help="refine threshold of the adaptive batch")
    ap.add_argument("--batch-eps-min", type=float, default=1e-8, help="smallest per-solve refine threshold")
    ap.add_argument("--batch-eps-max", type=float, default=1e-5, help="largest per-solve refine threshold")
    ap.add_argument("--batch-adapt-every", type=int, default=20,
                    help="steps between adaptations of the batched solves' grids (0: skip that run)")
    ap.add_argument("--batch-adapt-solves", type=int, default=64, help="solves in the adaptive batched run")
    ap.add_argument("--batch-adapt-rounds", type=int, default=10, help="adaptations in the adaptive batched run")
    ap.add_argument("--learn-runs", type=int, default=4, help="plain runs whose decisions train the classifier (0: skip)")
    ap.add_argument("--learn-steps", type=int, default=12)
    ap.add_argument("--learn-horizon", type=int, default=4,
                    help="time steps per learned pre-adaptation in the 3D Burgers runs")
    ap.add_argument("--learn-epochs", type=int, default=30)
    ap.add_argument("--herm-runs", type=int, default=3, help="timed runs of the 2D Hermite Burgers line (0: skip)")
    ap.add_argument("--wave-learn-runs", type=int, default=20, help="plain wave runs that train its classifier (0: skip)")
    ap.add_argument("--wave-learn-steps", type=int, default=30)
    ap.add_argument("--wave-train-samples", type=int, default=300000, help="training samples kept (stratified)")
    ap.add_argument("--wave-learn-horizon", type=int, default=2, help="time steps per learned pre-adaptation (wave)")
    ap.add_argument("--profile", choices=["none", "wave_rhs", "config3", "rhs3d", "linear6d", "batch", "herm",
                                          "rhs_config3"],
                    default="none",
                    help="wave_rhs: run the wave right-hand-side profiling case instead of the bench")
    ap.add_argument("--wave-only", action="store_true",
                    help="run only the 2D adaptive wave line (for a run to the config's T = 0.5) and print it")
    ap.add_argument("--wave-main-arms", action="store_true",
                    help="wave line: plain FP64, mixed + learned at the trained horizon and mixed plain only")
    ap.add_argument("--wave-no-level10", action="store_true",
                    help="skip the max-level-10 FP64 run the wave arms' errors are measured against")
    ap.add_argument("--wave-time", type=float, default=0.05,
                    help="final time of the 2D wave runs (the config's 0.5 takes ~5000 steps on a filling grid)")
    args = ap.parse_args()
    CONFIG3["tau"] = args.arm_tau
    if args.profile == "wave_rhs":
        profile_wave_rhs()
    elif args.profile == "config3":
        profile_config3()
    elif args.profile == "linear6d":
        profile_linear6d()
    elif args.profile == "batch":
        profile_batch()
    elif args.profile == "herm":
        profile_herm()
    elif args.profile == "rhs_config3":
        profile_rhs_config3()
    elif args.profile == "rhs3d":
        profile_rhs3d()
    elif args.wave_only:
        import torch

        import amdg
        torch.cuda.set_device(0)
        ctx = amdg.Context(0)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx.set_stream(stream.cuda_stream)
        print(json.dumps({"wave2d_adaptive": bench_wave_adaptive(ctx, stream, args)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
