"""Throughput of the plain collision step on one GB300 (cells*steps/s).

Workload: 20^3 velocity lattice on [-5,5]^3 cut to the sphere R=4.8 (3648
nodes), a batch of spatial cells of seeded Maxwellian mixtures; one step =
loss nu + gain I + FP64 conservation projection + relaxation (Courant dt).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` times K steps with f resident in HBM
(CUDA events on the launching stream, L2 flushed between steps); `e2e` times
the same steps through the C ABI with the distribution copied host->device
before and device->host after every step; `roofline` covers the gain kernel;
`cpu_baseline` times the oracle's OpenMP FP32 host path on a bounded sample.
Under torchrun each rank runs its own batch (weak scaling, no collective on
the data path) and the time is the maximum over ranks.
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

METRIC = "cells*steps/s at 20^3 grid (deterministic collision step, Q rel-L2 <= 1e-3)"
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
    p.add_argument("--gain", choices=["pair", "bf16", "bf16x3"], default="bf16",
                   help="gain algorithm of the timed step (FP32 pair-product kernel or tensor-core collision matrices)")
    p.add_argument("--alternatives", default="pair,bf16x3",
                   help="comma list of other gain paths to time after the main run ('' for none)")
    return p.parse_args()


GAIN_PATHS = {"pair": 0, "bf16": 1, "bf16x3": 2}


def workload(args, ncells):
    return {"workload": f"plain collision step, {args.grid}^3 lattice [-5,5]^3 cut to R={args.radius}",
            "gain": args.gain,
            "cells": ncells, "dt_mode": f"courant {args.courant} (dt = courant / max nu, as relax_f)",
            "inputs": "seeded Maxwellian mixtures: 1-3 components, n~LogN(0,0.3), u~N(0,0.7^2), T~U[0.6,1.8]",
            "l2": "256 MiB buffer written between timed steps (inside the timed region)"}


def peaks():
    try:
        with open(PEAKS_FILE) as fh:
            d = json.load(fh)
        return float(d["bf16_tflops"]), "measured"
    except Exception:
        return FALLBACK_BF16_TFLOPS, "fallback"


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


def cpu_baseline(args, seconds):
    """The oracle's FP32 OpenMP host path (loss + gain + FP64 projection) on a
    bounded sample of cells of the same workload."""
    from gpu_determ_gb300 import GridSpec, inputs
    from oracle.pyoracle import Oracle
    o = Oracle(args.grid, R=args.radius)
    grid = GridSpec(args.grid, R=args.radius).fill()
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    def run(nc):
        f = inputs.mixtures(grid, nc, seed=args.seed + 1)
        fb = o.to_box(f)
        t0 = time.perf_counter()
        nu = o.loss_f32(fb)
        gain = o.gain_f32(fb)
        o.project(f, nu, gain)
        return time.perf_counter() - t0

    run(1)  # thread pool and page warm-up
    nc, t = 2, run(2)
    while t < 0.6 * seconds and nc < 2048:  # grow the sample to the target length
        nc = min(2048, max(nc * 2, int(nc * seconds / max(t, 1e-3))))
        t = run(nc)
    return {"value": nc / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{nc} cell(s) x 1 step, all {o.n_pnt} nodes, {t:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vals = []
    info = None
    for _ in range(args.warmup):
        pass  # host code: no warm-up state beyond the first sample
    for _ in range(max(1, args.steps)):
        info = cpu_baseline(args, args.cpu_seconds / max(1, args.steps) * 2)
        vals.append(info["value"])
    v = statistics.median(vals)
    info["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": dict(workload(args, 1), gain="oracle FP32 OpenMP host path"),
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
    f_host = inputs.mixtures(grid, nc, seed=args.seed + rank)
    f0 = torch.from_numpy(f_host).cuda()
    f = f0.clone()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.step(f, nc, nc, gd.DT_COURANT, args.courant, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # device-resident timed region
    f.copy_(f0)
    barrier()
    with Clocks(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            flush.fill_(1)
            step()
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nc * args.steps / (ms / 1000.0)

    # end to end through the C ABI with host buffers (pinned), copies timed
    pinned_in = torch.from_numpy(f_host).pin_memory()
    pinned_out = torch.empty_like(pinned_in).pin_memory()
    fdev = torch.empty_like(f0)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        flush.fill_(1)
        fdev.copy_(pinned_in, non_blocking=True)
        ctx.step(fdev, nc, nc, gd.DT_COURANT, args.courant, stream=stream)
        pinned_out.copy_(fdev, non_blocking=True)
    e1.record(stream)
    barrier()
    ms_e2e = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t.item())
    e2e = world * nc * args.steps / (ms_e2e / 1000.0)
    nbytes = n * nc * 4

    # dominant kernel: the gain
    peak, peak_kind = peaks()
    roof = gain_roofline(args.gain, ctx, f0, nc, stream, flush, peak, peak_kind, max(2, args.steps))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"pair": "f32", "bf16": "bf16 (FP32 accumulate)", "bf16x3": "bf16x3 (FP32 accumulate)"}[args.gain]
            + ", FP64 projection",
            "data": "synthetic", "config": workload(args, nc),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "ms_per_step": ms_e2e / args.steps},
            "gpu_launches": (7 if args.gain == "pair" else 6) * args.steps,
            "clocks": clk.summary(), "roofline": roof}
    alts = {}
    if rank == 0 and world == 1:
        alts = alternatives(args, ctx, f0, nc, stream, flush, peak, peak_kind)
        if alts:
            line["alternatives"] = alts
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def gain_roofline(name, ctx, f0, nc, stream, flush, peak, peak_kind, reps):
    """Average duration of the gain call (CUDA events on the launching stream,
    L2 flushed before each) and its throughput against the BF16 tensor peak:
    algorithmic FLOP of the pair-product formulation for the FP32 kernel,
    dense tile FLOP for the tensor-core collision-matrix kernel."""
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
    g_avg = statistics.mean(g_ms) / 1000.0
    if name == "pair":
        inf = ctx.info
        flop = nc * (7 * inf["pair_products"] + 2 * inf["contraction_terms"] + inf["scatter_terms"])
        kernel, work = "gain_pair_kernel (+ chunk reduction)", \
            "7 FLOP per pair product + 2 per nonzero-weight term + 1 per scatter update"
    else:
        ns, ns_k = ctx.n_pnt, (ctx.n_pnt + 63) // 64 * 64
        flop = 2.0 * ns * ((nc + 127) // 128 * 128) * ((ns + 255) // 256 * 256) * ns_k * (3 if name == "bf16x3" else 1)
        kernel, work = "cmatrix_gain_kernel (tcgen05)", "dense tile MACs x 2 (x3 passes for bf16x3)"
    ach = flop / g_avg / 1e12
    return {"bound": "tensor", "kernel": kernel, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak, "peak_source": f"{peak_kind} bf16 dense (MEASURED_PEAKS.json)", "work": work,
            "flop_per_launch": flop, "traffic": None, "launch_ms": g_avg * 1000.0}


def one_step_q(gd, ctx, f0, nc):
    import torch
    f = f0.clone()
    q = torch.zeros(f.shape, dtype=torch.float64, device=f.device)
    ctx.step(f, nc, nc, gd.DT_COURANT, 0.5, q=q)
    torch.cuda.synchronize()
    return q


def alternatives(args, ctx, f0, nc, stream, flush, peak, peak_kind):
    """Step throughput of the other gain paths on the same workload, with the
    relative L2 difference of their Q from the main path's Q on the input."""
    import torch
    import gpu_determ_gb300 as gd
    names = [a for a in args.alternatives.split(",") if a and a != args.gain]
    if not names:
        return {}
    out = {}
    q_main = one_step_q(gd, ctx, f0, nc)
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
        ms = e0.elapsed_time(e1)
        q = one_step_q(gd, ctx, f0, nc)
        rel = float(torch.linalg.norm(q - q_main) / torch.linalg.norm(q_main))
        out[name] = {"value": nc * args.steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / args.steps,
                     "q_rel_l2_vs_main": rel,
                     "roofline": gain_roofline(name, ctx, f0, nc, stream, flush, peak, peak_kind,
                                               max(2, args.steps))}
    ctx.set_gain_path(GAIN_PATHS[args.gain])
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
