"""Collision-step throughput on one GB300 (cells*steps/s): surrogate+fallback vs plain.

Workload: 20^3 velocity lattice on [-5,5]^3 cut to the sphere R=4.8 (3648
nodes), a batch of spatial cells of seeded mixtures of 1-4 Maxwellians
(Dirichlet(1) weights, u ~ N(0, I), T ~ U[0.5, 2]); one step = loss nu +
gain I + FP64 conservation projection + relaxation (Courant dt).  The plain
step computes the gain with the context's gain path (collision matrices on
the tensor cores with the BF16 hi/lo split, FP32-equivalent, by default); the
surrogate step takes the gain from the
learned network for every cell whose estimated error is within --tol and
from the plain path for the others (gd_surrogate_gain).  The network is
trained before the timed region on pairs the plain path generates.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` times K surrogate+fallback steps with
f resident in HBM (CUDA events on the launching stream, L2 flushed between
steps), `plain` the same for the plain step; `e2e` times the surrogate steps
through the C ABI with the distribution copied host->device before and
device->host after every step; `accuracy` compares the step's projected Q with
the FP32 pair kernel's on the same cells, per cell, and (from the CPU-baseline
leg, where the oracle runs) with the oracle's FP64 path on the first cells;
`roofline` covers the plain gain kernel (tensor pipe for the collision
matrices, measured FP32 FMA peak for the SIMT pair kernels); `cpu_baseline`
times the oracle's OpenMP FP32 host path on a bounded sample.  Under torchrun each rank runs its own batch (weak scaling, no
collective on the data path) and the time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cells*steps/s at 20^3 grid: surrogate+fallback vs plain on GB300, rel-L2<=1e-3"
UNIT = "cell-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_BF16_TFLOPS = 1900.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--grid", type=int, default=20)
    p.add_argument("--radius", type=float, default=4.8)
    p.add_argument("--cells", type=int, default=4096)
    p.add_argument("--courant", type=float, default=0.5)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="target length of the bounded CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--ref-cells", type=int, default=128,
                   help="reference arm: whole cells of the workload evaluated per step on the host")
    p.add_argument("--gain", choices=["pair", "pair_tc", "bf16", "bf16x3"], default="bf16x3",
                   help="gain algorithm of the timed step (FP32 pair-product kernel, pair products with the "
                        "contraction on the tensor cores, or tensor-core collision matrices)")
    p.add_argument("--alternatives", default="pair,pair_tc,bf16",
                   help="comma list of other gain paths to time after the main run ('' for none)")
    p.add_argument("--no-surrogate", action="store_true", help="time the plain step only")
    p.add_argument("--settle", type=float, default=3.0, help="seconds of untimed plain steps before timing")
    p.add_argument("--tol", type=float, default=1e-3, help="surrogate acceptance tolerance (relative L2 of Q)")
    p.add_argument("--pairs", type=int, default=65536, help="surrogate training pairs")
    p.add_argument("--train-steps", type=int, default=6000)
    p.add_argument("--fp64-cells", type=int, default=32,
                   help="cells of the timed batch checked against the oracle's FP64 path (in the CPU-baseline leg)")
    p.add_argument("--kernels", action="store_true",
                   help="time the step's loss, projection and relaxation kernels one by one against their "
                        "rooflines (one JSON line) instead of the step")
    p.add_argument("--once", action="store_true",
                   help="with --kernels: launch each kernel once, untimed (the command an ncu capture runs)")
    return p.parse_args()


GAIN_PATHS = {"pair": 0, "bf16": 1, "bf16x3": 2, "pair_tc": 3}


def workload(args, ncells):
    kind = "plain collision step" if args.no_surrogate else \
        f"surrogate+fallback collision step (tol {args.tol:g})"
    return {"workload": f"{kind}, {args.grid}^3 lattice [-5,5]^3 cut to R={args.radius}",
            "gain": args.gain,
            "cells": ncells, "dt_mode": f"courant {args.courant} (dt = courant / max nu, as relax_f)",
            "inputs": "seeded mixtures of 1-4 Maxwellians: Dirichlet(1) weights, u~N(0,I), T~U[0.5,2]",
            "l2": "256 MiB buffer written between timed steps (inside the timed region)"}


def peaks(gd, device):
    """Roofline denominators: the BF16 tensor peak from MEASURED_PEAKS.json
    (cuBLAS burst, else the fallback), and the FP32 / FP64 FMA throughput
    measured in this run by the library's own microbenchmark (gd_fma_peak)."""
    try:
        with open(PEAKS_FILE) as fh:
            d = json.load(fh)
        out = {"bf16": float(d["bf16_tflops"]), "bf16_source": "measured bf16 dense burst (MEASURED_PEAKS.json)"}
    except Exception:
        out = {"bf16": FALLBACK_BF16_TFLOPS, "bf16_source": "fallback bf16 dense"}
    out["fp32"] = gd.fma_peak(device, 32) / 1e12
    out["fp64"] = gd.fma_peak(device, 64) / 1e12
    out["fma_source"] = "FFMA/DFMA throughput measured in this run (gd_fma_peak)"
    return out


class Clocks:
    """nvidia-smi sampler running while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def host_oracle(args):
    """The oracle for the bench grid and its grid lists (built by the oracle
    itself, so a host-only run never loads the GPU library)."""
    from oracle.pyoracle import Oracle
    o = Oracle(args.grid, R=args.radius)
    return o, {"u": o.u, "v": o.v, "w": o.w, "ui": o.ui, "vi": o.vi, "wi": o.wi}


def host_step(o, f):
    """One collision evaluation of the oracle's FP32 OpenMP host path (loss +
    gain + FP64 projection) on compact [n_pnt][cells]; returns seconds."""
    fb = o.to_box(f)
    t0 = time.perf_counter()
    nu = o.loss_f32(fb)
    gain = o.gain_f32(fb)
    o.project(f, nu, gain)
    return time.perf_counter() - t0


def host_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def workload_cells(args, grid, ncells):
    """The first ncells cells of the bench workload (its seed and its full
    batch of args.cells draws, so the sample is a prefix of the timed cells)."""
    from gpu_determ_gb300 import inputs
    f = inputs.dirichlet_mixtures(grid, max(args.cells, ncells), seed=args.seed + 17)
    return np.ascontiguousarray(f[:, :ncells])


def fp64_q(o, f):
    """The oracle's FP64 loss and gain and an FP64 conservation projection
    (collision_integral.cu:217-526, solved per cell) of compact f [n][cells]."""
    fb = o.to_box(f)
    nu, g = o.loss_f64(fb), o.gain_f64(fb)
    f = f.astype(np.float64)
    phi = o.phi()
    fnu = f * nu
    A = np.einsum("nk,nl,nc->ckl", phi, phi, fnu)
    B = np.einsum("nk,nc->ck", phi, g - fnu)
    X = np.linalg.solve(A, B[..., None])[..., 0]
    return g - fnu * (1.0 + phi @ X.T)


def cpu_baseline(args, seconds, checks=None):
    """The oracle's FP32 OpenMP host path on a bounded sample of whole cells
    of the workload, grown until one evaluation takes about `seconds`.  With
    checks (name -> the GPU's projected Q of the workload's first k cells),
    the oracle also serves as the checker: its FP64 path on those k cells,
    untimed, and the per-cell relative L2 of each Q against it."""
    o, grid = host_oracle(args)
    f_all = workload_cells(args, grid, 2048)
    host_step(o, f_all[:, :1])  # thread pool and page warm-up
    nc, t = 2, host_step(o, f_all[:, :2])
    while t < 0.6 * seconds and nc < 2048:  # grow the sample to the target length
        nc = min(2048, max(nc * 2, int(nc * seconds / max(t, 1e-3))))
        t = host_step(o, f_all[:, :nc])
    out = {"value": nc / t, "unit": UNIT, "cores": host_threads(), "kind": "port",
           "sample": f"{nc} cell(s) x 1 step, all {o.n_pnt} nodes, {t:.1f} s"}
    if checks:
        k = next(iter(checks.values())).shape[1]
        q64 = fp64_q(o, f_all[:, :k])
        out["fp64_check"] = {}
        for name, q in checks.items():
            e = np.linalg.norm(q - q64, axis=0) / np.linalg.norm(q64, axis=0)
            out["fp64_check"][name] = {"cell_rel_l2_median": float(np.median(e)),
                                       "cell_rel_l2_p99": float(np.quantile(e, 0.99)),
                                       "cell_rel_l2_max": float(e.max()),
                                       "batch_rel_l2": float(np.linalg.norm(q - q64) / np.linalg.norm(q64))}
    return out


def run_reference(args):
    """The reference arm: the oracle's host path (the reference has no CPU
    implementation of its own) timed on all host cores, each step one
    collision evaluation of the same --ref-cells whole cells of the workload,
    whatever --steps is; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    o, grid = host_oracle(args)
    nc = max(1, args.ref_cells)
    f = workload_cells(args, grid, nc)
    for _ in range(max(args.warmup, 1)):
        host_step(o, f[:, :2])  # warm-up of the thread pool and pages, on two cells
    times = [host_step(o, f) for _ in range(max(1, args.steps))]
    total = sum(times)
    v = nc * len(times) / total
    info = {"value": v, "unit": UNIT, "cores": host_threads(), "kind": "port",
            "sample": f"{nc} cell(s) of the workload per step x {len(times)} steps, all {o.n_pnt} nodes, "
                      f"{total:.1f} s"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": dict(workload(args, args.cells), gain="oracle FP32 OpenMP host path",
                                                sample_cells=nc),
            "cpu_baseline": info,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import gpu_determ_gb300 as gd
    from gpu_determ_gb300 import inputs

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    spec = gd.GridSpec(args.grid, R=args.radius)
    ctx = gd.Context(spec, device=local)
    ctx.set_gain_path(GAIN_PATHS[args.gain])
    n = ctx.n_pnt
    nc = args.cells
    grid = spec.fill()
    f_host = inputs.dirichlet_mixtures(grid, nc, seed=args.seed + 17 + rank)
    f0 = torch.from_numpy(f_host).cuda()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from gpu_determ_gb300.sharding import max_over_ranks as _max

    def max_over_ranks(ms):
        return _max(ms, device="cuda")

    def plain_step(fb):
        ctx.step(fb, nc, nc, gd.DT_COURANT, args.courant, stream=stream)

    model = None
    nu = torch.empty_like(f0)
    gain = torch.empty_like(f0)
    fallbacks = []
    if not args.no_surrogate:
        from gpu_determ_gb300 import surrogate as sg
        t0 = time.perf_counter()
        model = sg.fit(ctx, grid, pairs=args.pairs, steps=args.train_steps, max_cells=nc, seed=args.seed)
        fit_s = time.perf_counter() - t0
        tol_arg = model.tol_arg(args.tol)

        def sur_step(fb):
            fallbacks.append(model.surrogate.gain(fb, nc, nc, tol_arg, nu, gain, stream=stream))
            ctx.project(fb, nu, gain, nc, nc, nu_corr=nu, stream=stream)
            ctx.relax(fb, nu, gain, nc, nc, gd.DT_COURANT, args.courant, stream=stream)

    def timed(step_fn, host_copies=False):
        """K steps from f0 (device-resident, or copied from/to pinned host
        buffers inside the timed region); returns ms."""
        fb = f0.clone()
        for _ in range(args.warmup):
            step_fn(fb)
        fb.copy_(f0)
        if host_copies:
            pin_in = torch.from_numpy(f_host).pin_memory()
            pin_out = torch.empty_like(pin_in).pin_memory()
        barrier()
        with Clocks(local) as clk:
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            # an NVTX range names the timed steps for a profiler's launch list
            torch.cuda.nvtx.range_push("timed_e2e" if host_copies else "timed")
            ev0.record(stream)
            for _ in range(args.steps):
                flush.fill_(1)
                if host_copies:
                    fb.copy_(pin_in, non_blocking=True)
                step_fn(fb)
                if host_copies:
                    pin_out.copy_(fb, non_blocking=True)
            ev1.record(stream)
            torch.cuda.nvtx.range_pop()
            barrier()
        return max_over_ranks(ev0.elapsed_time(ev1)), clk

    # untimed plain steps for a few seconds first, so the first timed region
    # does not see the GPU's ramp from idle
    fb = f0.clone()
    t_settle = time.perf_counter()
    while time.perf_counter() - t_settle < args.settle:
        plain_step(fb)
        torch.cuda.synchronize()
    del fb
    ms_plain, clk_plain = timed(plain_step)
    plain_value = world * nc * args.steps / (ms_plain / 1000.0)
    main_step = plain_step if model is None else sur_step
    if model is None:
        ms, clk = ms_plain, clk_plain
    else:
        fallbacks.clear()
        ms, clk = timed(sur_step)
        fb_timed = fallbacks[args.warmup:] if len(fallbacks) > args.warmup else fallbacks
    value = world * nc * args.steps / (ms / 1000.0)
    ms_e2e, _ = timed(main_step, host_copies=True)
    e2e = world * nc * args.steps / (ms_e2e / 1000.0)
    nbytes = n * nc * 4

    # dominant kernel: the plain gain (the fallback path)
    peak = peaks(gd, local)
    roof = gain_roofline(args.gain, ctx, f0, nc, stream, flush, peak, max(2, args.steps))

    # accuracy: projected Q of one evaluation on the timed cells against the
    # FP32 pair kernel's (the reference's arithmetic) on the same cells, per
    # cell; and, in the CPU-baseline leg, against the oracle's FP64 path
    ref_ctx = gd.Context(spec, device=local)
    q_ref, _ = projected_q(gd, ref_ctx, f0, nc)
    ref_ctx.close()
    q_plain, _ = projected_q(gd, ctx, f0, nc)

    dtype = {"pair": "f32", "pair_tc": "bf16x3 pair products and weights (FP32 accumulate)",
             "bf16": "bf16 (FP32 accumulate)",
             "bf16x3": "bf16x3 (hi/lo split, FP32 accumulate, at most 256 products per tensor-core accumulation)"
             }[args.gain]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": dtype + ", FP64 projection" + ("" if model is None else "; surrogate bf16 (FP32 accumulate)"),
            "data": "synthetic", "config": workload(args, nc),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "ms_per_step": ms_e2e / args.steps},
            "clocks": clk.summary(), "roofline": roof,
            "peaks": {"bf16_tflops": peak["bf16"], "bf16_source": peak["bf16_source"],
                      "fp32_fma_tflops": peak["fp32"], "fp64_fma_tflops": peak["fp64"],
                      "fma_source": peak["fma_source"]},
            "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": ms_plain / args.steps,
                      "gain": args.gain, "clocks": clk_plain.summary(),
                      "accuracy": cell_stats(gd, ctx, q_plain, q_ref, nc)}}
    n_loss, n_gain = path_launches(args.gain, ctx)
    if model is None:
        # per plain step: loss, gain, projection, max, dt, relaxation
        line["gpu_launches"] = (n_loss + n_gain + 4) * args.steps
        q_main = q_plain
        line["accuracy"] = dict(cell_stats(gd, ctx, q_plain, q_ref, nc), tol=args.tol)
    else:
        # loss, error network 8, selection 1, projection 1, relaxation 3; then
        # either the plain gain in place when every cell falls back, or the
        # network 8 and nu f 1, plus gather 1, plain gain and scatter 1 when some do
        line["gpu_launches"] = sum(n_loss + 13 + (n_gain if k == nc else 9 + (n_gain + 2 if k > 0 else 0))
                                   for k in fb_timed)
        rep, q_main = surrogate_report(args, gd, ctx, model, f0, nc, stream, fit_s, fb_timed, plain_value, q_ref)
        rep["speedup_vs_plain"] = value / plain_value
        line["accuracy"] = next(c for c in rep["tolerance_curve"] if c["tol"] == args.tol)
        line["surrogate"] = rep
    line["accuracy"]["reference"] = "FP32 pair kernel + FP64 projection on the same cells"
    alts = {}
    if rank == 0 and world == 1:
        alts = alternatives(args, ctx, f0, nc, stream, flush, peak, q_ref)
        if alts:
            line["alternatives"] = alts
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        k = min(args.fp64_cells, nc)
        checks = {"timed_path": q_main[:, :k].cpu().numpy(), "plain": q_plain[:, :k].cpu().numpy(),
                  "fp32_pair": q_ref[:, :k].cpu().numpy()}
        line["cpu_baseline"] = cpu_baseline(args, args.cpu_seconds, checks)
        fp64 = line["cpu_baseline"].pop("fp64_check", None)
        if fp64:
            line["accuracy"]["vs_fp64_sample"] = dict(fp64["timed_path"], cells=k)
            line["plain"]["accuracy"]["vs_fp64_sample"] = dict(fp64["plain"], cells=k)
            line["accuracy"]["fp32_pair_vs_fp64_sample"] = dict(fp64["fp32_pair"], cells=k)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def path_launches(name, ctx):
    """Kernel launches of the loss and of the gain on a gain path: the FP32
    loss kernel, or on the tensor-core paths the BF16 conversion of f and one
    tensor-core GEMM; the FP32 gain kernel and its chunk reduction, the
    pair tensor-core kernel between its scale and conversion kernels, or the
    conversion of f and the collision-matrix kernel."""
    if name == "pair":
        return 1, 2
    if name == "pair_tc":
        return 2, 3
    return 2, 2


def cell_stats(gd, ctx, q, q_ref, nc):
    """Per-cell relative L2 of Q against q_ref (median, p99, max), batch
    relative L2, and the conservation of Q (max over cells and moments of
    |sum Q phi_k| / sum |Q phi_k|)."""
    import torch
    from gpu_determ_gb300 import surrogate as sg
    err = torch.empty(nc, dtype=torch.float64, device=q.device)
    gd.cell_rel_l2(q, nc, q_ref, nc, ctx.n_pnt, nc, err)
    e = err.cpu().numpy()
    phi = sg._basis(ctx, q.device)
    mom = (phi @ q).abs() / (phi.abs() @ q.abs()).clamp_min(1e-300)
    return {"batch_rel_l2": float(torch.linalg.norm(q - q_ref) / torch.linalg.norm(q_ref)),
            "cell_rel_l2_median": float(np.median(e)), "cell_rel_l2_p99": float(np.quantile(e, 0.99)),
            "cell_rel_l2_max": float(e.max()), "cells_within_1e-3": float(np.mean(e <= 1e-3)),
            "conservation_max": float(mom.max())}


def projected_q(gd, ctx, f, nc, gain_fn=None):
    """FP64 projected Q of one evaluation on f (plain gain, or gain_fn's)."""
    import torch
    nu = torch.empty_like(f)
    gain = torch.empty_like(f)
    q = torch.zeros(f.shape, dtype=torch.float64, device=f.device)
    nfb = None
    if gain_fn is None:
        ctx.collision(f, nc, nc, nu, gain)
    else:
        nfb = gain_fn(f, nu, gain)
    ctx.project(f, nu, gain, nc, nc, q=q)
    torch.cuda.synchronize()
    return q, nfb


def surrogate_report(args, gd, ctx, model, f0, nc, stream, fit_s, fb_timed, plain_value, q_ref):
    """Accuracy of surrogate+fallback on the timed cells against the FP32 pair
    kernel's projected Q, and the fallback fraction / throughput trade-off
    over looser tolerances.  Returns the report and the projected Q at the
    timed tolerance."""
    import torch
    curve = []
    q_at_tol = None
    for tol in sorted({args.tol, 1e-2, 3e-2, 1e-1, 3e-1, 1.0}):
        ta = model.tol_arg(tol)
        q, nfb = projected_q(gd, ctx, f0, nc, lambda f, nu, g: model.surrogate.gain(f, nc, nc, ta, nu, g))
        if tol == args.tol:
            q_at_tol = q
        # one timed step at this tolerance (gain + projection + relaxation)
        fb = f0.clone()
        nu = torch.empty_like(f0)
        g = torch.empty_like(f0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        model.surrogate.gain(fb, nc, nc, ta, nu, g, stream=stream)
        ctx.project(fb, nu, g, nc, nc, nu_corr=nu, stream=stream)
        ctx.relax(fb, nu, g, nc, nc, gd.DT_COURANT, args.courant, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        v = nc / (e0.elapsed_time(e1) / 1000.0)
        curve.append(dict({"tol": tol, "fallback_fraction": nfb / nc, "value": v, "speedup_vs_plain": v / plain_value},
                          **cell_stats(gd, ctx, q, q_ref, nc)))
    q_sur, _ = projected_q(gd, ctx, f0, nc, lambda f, nu, g: model.surrogate.gain(f, nc, nc, float("inf"), nu, g))
    # the step with no fallback at all: what the network would deliver if its
    # accuracy let every cell through (exact loss, network, projection, relaxation)
    fb = f0.clone()
    nu = torch.empty_like(f0)
    g = torch.empty_like(f0)
    model.surrogate.gain(fb, nc, nc, float("inf"), nu, g, stream=stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    reps = 5
    for _ in range(reps):
        model.surrogate.gain(fb, nc, nc, float("inf"), nu, g, stream=stream)
        ctx.project(fb, nu, g, nc, nc, nu_corr=nu, stream=stream)
        ctx.relax(fb, nu, g, nc, nc, gd.DT_COURANT, args.courant, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    no_fb = nc * reps / (e0.elapsed_time(e1) / 1000.0)
    # what any network fed BF16 inputs can reach: the exact plain operator
    # applied to f rounded to BF16, against the same operator on f
    q_bf16_in, _ = projected_q(gd, ctx, f0.bfloat16().float(), nc)
    q_plain, _ = projected_q(gd, ctx, f0, nc)
    rep = {"tol": args.tol, "fallback_fraction": float(np.mean(fb_timed)) / nc if fb_timed else None,
           "speedup_vs_plain": None, "reference": "FP32 pair kernel + FP64 projection on the same cells",
           "surrogate_only": dict(cell_stats(gd, ctx, q_sur, q_ref, nc), value=no_fb, unit=UNIT,
                                  speedup_vs_plain=no_fb / plain_value),
           "bf16_input_floor": dict(cell_stats(gd, ctx, q_bf16_in, q_plain, nc),
                                    what="plain operator on BF16-rounded f vs on f"),
           "tolerance_curve": curve,
           "training": dict(model.report, fit_total_s=round(fit_s, 1)),
           "network": {"layers": "n->256, 256->512 GELU, 512->512 GELU, 512->256 +residual, 256->n",
                       "params": model.net.info["num_params"],
                       "forward_flop_per_cell": model.net.info["forward_flop_per_cell"]}}
    return rep, q_at_tol


def time_gain(ctx, f0, nc, stream, flush, reps):
    """Average duration of the gain call (CUDA events on the launching
    stream, L2 flushed before each), seconds."""
    import torch
    gain = torch.empty_like(f0)
    for _ in range(2):
        ctx.collision(f0, nc, nc, None, gain, stream=stream)
    torch.cuda.synchronize()
    g_ms = []
    for _ in range(reps):
        flush.fill_(1)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        ctx.collision(f0, nc, nc, None, gain, stream=stream)
        a1.record(stream)
        a1.synchronize()
        g_ms.append(a0.elapsed_time(a1))
    return statistics.mean(g_ms) / 1000.0


def gain_roofline(name, ctx, f0, nc, stream, flush, peak, reps):
    """Throughput of the gain launch against its bounding pipe: the BF16
    tensor peak for the collision-matrix kernel (FLOP of the tiles issued),
    the measured FP32 FMA peak for the SIMT pair-product kernels (algorithmic
    FLOP of the pair-product formulation)."""
    g_avg = time_gain(ctx, f0, nc, stream, flush, reps)
    traffic, traffic_src = None, None
    if name in ("pair", "pair_tc"):
        inf = ctx.info
        flop = nc * (7 * inf["pair_products"] + 2 * inf["contraction_terms"] + inf["scatter_terms"])
        kernel = "gain_pair_kernel (+ chunk reduction)" if name == "pair" else \
            "pair_tc_kernel (tcgen05 contraction, + chunk reduction)"
        work = "7 FLOP per pair product + 2 per nonzero-weight term + 1 per scatter update"
        bound, pk, src = "fp32", peak["fp32"], peak["fma_source"]
    else:
        # stored tiles: the nonzero 256 x 64 tiles of each G_i's block upper
        # triangle; issued: their 256 x 16 slices with a nonzero entry (one MMA
        # K step each; the all-zero slices are skipped)
        inf = ctx._info()
        tiles = inf["cmatrix_tiles"]  # stored (one matrix per orbit of the lattice's reflections)
        # issued over every node; one BF16 pass issues whole tiles (4 K steps each)
        slices = inf["cmatrix_slices"] if name == "bf16x3" else 4 * inf["cmatrix_node_tiles"]
        flop = 2.0 * ((nc + 127) // 128 * 128) * 256 * 16 * slices * (3 if name == "bf16x3" else 1)
        kernel, work = "cmatrix_gain_kernel (tcgen05)", \
            "MACs x 2 of the 128x256x16 MMA K steps issued (nonzero slices of the stored tiles of the block upper triangle of each symmetric G_i; x3 for bf16x3)"
        bound, pk, src = "tensor", peak["bf16"], peak["bf16_source"]
        # DRAM bytes per launch: every node's matrix tiles stream through about
        # once (a representative's tiles once per reflection: the launch runs
        # reflection-major).  An ncu capture of the BF16x3 kernel (CTA pairs) on
        # 14^3 / 4096 cells read and wrote 7.806 GB for 5.820 GB of tiles the
        # nodes stream (ratio 1.341); scaled here by the 20^3 launch's tiles.
        g_bytes = inf["cmatrix_node_tiles"] * 256 * 64 * 2 * (2 if name == "bf16x3" else 1)
        traffic = 1.341 * g_bytes
        traffic_src = "ncu dram__bytes_read+write of a 14^3/4096-cell launch, scaled by the matrix tile bytes the nodes stream"
    ach = flop / g_avg / 1e12
    out = {"bound": bound, "kernel": kernel, "achieved": ach, "peak": pk, "unit": "TFLOP/s",
           "frac": ach / pk, "peak_source": src, "work": work,
           "flop_per_launch": flop, "traffic": traffic, "traffic_source": traffic_src, "launch_ms": g_avg * 1000.0}
    if name not in ("pair", "pair_tc"):
        # the dense bilinear form's count, 2 n^3 + 2 n^2 FLOP per cell: what the
        # launch computes without exploiting the symmetry of G_i and its zero tiles
        n = ctx.n_pnt
        dense = nc * (2.0 * n ** 3 + 2.0 * n ** 2) * (3 if name == "bf16x3" else 1)
        out["dense_equivalent"] = {"flop_per_launch": dense, "tflops": dense / g_avg / 1e12,
                                   "issued_fraction": flop / dense}
    return out


def alternatives(args, ctx, f0, nc, stream, flush, peak, q_ref):
    """Step throughput of the other gain paths on the same workload, with the
    per-cell relative L2 of their projected Q against the FP32 pair kernel's."""
    import torch
    import gpu_determ_gb300 as gd
    names = [a for a in args.alternatives.split(",") if a and a != args.gain]
    if not names:
        return {}
    out = {}
    for name in names:
        try:
            ctx.set_gain_path(GAIN_PATHS[name])
        except gd.GDError as e:
            out[name] = {"unavailable": str(e)}
            continue
        f = f0.clone()
        for _ in range(args.warmup):
            ctx.step(f, nc, nc, gd.DT_COURANT, args.courant, stream=stream)
        f.copy_(f0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            flush.fill_(1)
            ctx.step(f, nc, nc, gd.DT_COURANT, args.courant, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.check()
        ms = e0.elapsed_time(e1)
        q, _ = projected_q(gd, ctx, f0, nc)
        out[name] = {"value": nc * args.steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / args.steps,
                     "accuracy": cell_stats(gd, ctx, q, q_ref, nc),
                     "roofline": gain_roofline(name, ctx, f0, nc, stream, flush, peak, max(2, args.steps))}
    ctx.set_gain_path(GAIN_PATHS[args.gain])
    return out


def run_kernels(args):
    """The step's kernels besides the gain, one by one on the bench workload:
    CUDA events on the launching stream, the 256 MiB L2 flush before each
    launch, best of --steps after --warmup.  Each is set against what bounds
    it: HBM bytes (MEASURED_PEAKS.json), or the FP32 / FP64 FMA or BF16 tensor
    throughput.  GB300's FP64 rate is 1/64 of its FP32 rate, and float <-> double
    conversions issue on the same pipe, so the FP64 projection and relaxation
    are bound by it rather than by HBM."""
    import torch
    import gpu_determ_gb300 as gd
    from gpu_determ_gb300 import inputs

    torch.cuda.set_device(0)
    spec = gd.GridSpec(args.grid, R=args.radius)
    t0 = time.perf_counter()
    ctx = gd.Context(spec)
    torch.cuda.synchronize()
    build_s = {"context": time.perf_counter() - t0}
    n, nc = ctx.n_pnt, args.cells
    f = torch.from_numpy(inputs.dirichlet_mixtures(spec.fill(), nc, seed=args.seed + 17)).cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    nu, gain, nuc = (torch.empty_like(f) for _ in range(3))
    q = torch.empty(f.shape, dtype=torch.float64, device="cuda")
    fr = f.clone()
    tm, dt = torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")
    stream = torch.cuda.current_stream()
    ms = {}

    def run(name, fn):
        fn()
        torch.cuda.synchronize()
        if args.once:
            return
        for _ in range(args.warmup):
            fn()
        best = float("inf")
        for _ in range(max(1, args.steps)):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        ms[name] = best

    run("loss_fp32", lambda: ctx.collision(f, nc, nc, nu, None))
    if args.gain != "pair":
        t0 = time.perf_counter()
        ctx.set_gain_path(GAIN_PATHS[args.gain])
        torch.cuda.synchronize()
        build_s["gain_path"] = time.perf_counter() - t0
        run("loss_tc", lambda: ctx.collision(f, nc, nc, nu, None))
    ctx.collision(f, nc, nc, nu, gain)
    run("project", lambda: ctx.project(f, nu, gain, nc, nc, nuc, q, None))
    run("relax_fixed", lambda: ctx.relax(fr, nuc, gain, nc, nc, gd.DT_FIXED, 1e-4, tm, dt))
    run("relax_courant", lambda: ctx.relax(fr, nuc, gain, nc, nc, gd.DT_COURANT, args.courant, tm, dt))
    ctx.check()
    line = {"mode": "kernels", "once": bool(args.once), "build_s": build_s,
            "config": {"grid": args.grid, "radius": args.radius, "nodes": n, "cells": nc, "gain": args.gain,
                       "l2": "256 MiB buffer written before each timed launch"}}
    if args.once:
        print(json.dumps(line))
        return
    pk = peaks(gd, 0)
    try:
        with open(PEAKS_FILE) as fh:
            hbm, hbm_src = float(json.load(fh)["hbm_gbs"]), "measured copy (MEASURED_PEAKS.json)"
    except Exception:
        hbm, hbm_src = 6800.0, "fallback copy bandwidth"
    cells = float(n) * nc

    def entry(t, flop=None, fpeak=None, nbytes=None, work=""):
        e = {"ms": t, "work": work}
        if flop is not None:
            e.update({"tflops": flop / t / 1e9, "flop_peak_tflops": fpeak, "flop_frac": flop / t / 1e9 / fpeak})
        if nbytes is not None:
            e.update({"gbs": nbytes / t / 1e6, "hbm_peak_gbs": hbm, "hbm_frac": nbytes / t / 1e6 / hbm})
        return e

    k = {}
    k["loss_kernel (FP32)"] = entry(ms["loss_fp32"], flop=2.0 * n * n * nc, fpeak=pk["fp32"],
                                    work="2 n^2 FLOP per cell (one FMA per partner), vs the FP32 FMA peak")
    if "loss_tc" in ms:
        rows, cols, kk = -(-n // 128) * 128, -(-nc // 128) * 128, -(-n // 64) * 64
        k["convert + gemm3_nt_kernel (loss on tensor cores)"] = entry(
            ms["loss_tc"], flop=3 * 2.0 * rows * cols * kk, fpeak=pk["bf16"],
            nbytes=4.0 * n * kk + 4.0 * kk * nc + 4.0 * cells + 4.0 * cells,
            work="3 BF16 MMA products per K step over the padded tiles, vs the BF16 peak; bytes: B and f "
                 "as BF16 hi/lo, f read and nu written in FP32")
    k["project_kernel (FP64)"] = entry(ms["project"], flop=65.0 * cells, fpeak=pk["fp64"], nbytes=24.0 * cells,
                                       work="65 FP64 FLOP per node and cell (53 for the 25 sums, 12 for nu' and "
                                            "Q) and 7 conversions; bytes: f, nu, I read, nu' and FP64 Q written")
    k["relax_kernel (FP64, fixed dt)"] = entry(ms["relax_fixed"], flop=4.0 * cells, fpeak=pk["fp64"],
                                               nbytes=16.0 * cells,
                                               work="f + dt (I - f nu') in FP64: 4 FLOP and 4 conversions; bytes: f, nu', "
                                                    "I read, f written")
    k["max_kernel + dt_kernel (Courant dt)"] = entry(max(ms["relax_courant"] - ms["relax_fixed"], 1e-6),
                                                     nbytes=4.0 * cells, work="nu' read once")
    line.update({"kernels": k, "peaks": {"hbm_gbs": hbm, "hbm_source": hbm_src, "fp32_tflops": pk["fp32"],
                                         "fp64_tflops": pk["fp64"], "bf16_tflops": pk["bf16"],
                                         "fma_source": pk["fma_source"], "bf16_source": pk["bf16_source"]}})
    print(json.dumps(line))


def main():
    args = parse()
    if args.kernels:
        run_kernels(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
