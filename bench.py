#!/usr/bin/env python
"""Benchmark of the GB300 Hermite-TENO hot path.

Workload (one GPU): 2D Euler, 1024 x 1024 cells on [0,1]^2, seeded four-quadrant Riemann data,
gamma 1.4, zero-gradient boundaries, characteristic TENO5 per direction + three-point
Gauss-Legendre transverse reconstruction, HLLC flux, SSP-RK3, CFL 0.4, plain FP64.  A step is
one SSP-RK3 time step (3 residual evaluations + stage updates) over the whole grid; the metric
is cell-updates per second (interior cells x completed steps / seconds).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (launched under torchrun) every rank advances its own replica of the workload (the
path has no exchange step at this size: replicas only), timed between barriers; the reported
value is the sum over ranks divided by the slowest rank's time.
--impl reference times the reference algorithm on the host cores (the CPU oracle, the
reference's own sources cannot be built on the GPU host), rank 0 only.

Besides the headline line's plain FP64 value, "paths" reports the other measured workloads:
the plain FP64 stage as one fused launch on the same timed steps (checked bit for bit against
the headline run), the mixed-precision path on the same grid (with its density error against
FP64), the Hermite-WENO 2048^2 blob/shock case (FP64 and mixed), the 4096^2 learned-routing case
(FP64, FP32, FP32 + learned classifier, with training and audit figures) and the batch of 256
uneven grids.  --no-fused / --no-mixed / --no-hermite / --no-learned / --no-batch skip them.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "hermite-teno_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

METRIC = "2D Euler Mcell-updates/s, plain FP64 vs FP32+learned; L1 err vs FP64"
UNIT = "Mcell-updates/s"
NX = NY = 1024
SEED = 0
WORKLOAD = "fv2d_fourquadrant_1024x1024_teno5_hllc_ssprk3_fp64"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--start-step", type=int, default=100)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-hermite", action="store_true")
    ap.add_argument("--no-sod", action="store_true")
    ap.add_argument("--hermite-steps", type=int, default=10,
                    help="steps of both Hermite arms (the same window from the initial state)")
    ap.add_argument("--hermite-n", type=int, default=2048, help="grid side of the Hermite 2D path")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-fused", action="store_true")
    ap.add_argument("--c5-steps", type=int, default=500,
                    help="steps of the 4096^2 learned-routing case: the FP64 arm runs them, the FP32 "
                         "arms run from the same initial state to the FP64 arm's end time")
    ap.add_argument("--c5-epochs", type=int, default=10)
    ap.add_argument("--c5-audit-every", type=int, default=50)
    ap.add_argument("--c5-classify-every", type=int, default=10,
                    help="second learned arm: the classifier runs every this many steps and its masks "
                         "serve the steps between (the first learned arm classifies every step)")
    ap.add_argument("--c5-margin", type=int, default=-1,
                    help="erosion of the second arm's route masks in faces (default 2 ceil(cfl * classify-every))")
    ap.add_argument("--c5-threshold", type=float, default=0.99,
                    help="routing threshold: a stencil takes the linear weights when all three "
                         "predicted cut-off probabilities exceed it")
    ap.add_argument("--batch-steps", type=int, default=100)
    return ap.parse_args()


def dist_setup(torch):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(torch, world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(torch, world, x):
    from hteno import replicas

    return replicas.reduce(torch, x, "max", "cuda") if world > 1 else x


def config_block(args, world, timed_from_step):
    return {"workload": WORKLOAD, "nx": NX, "ny": NY, "recon": "teno5", "flux": "hllc",
            "timed_from_step": timed_from_step,
            "bc": "zero-gradient", "cfl": 0.4, "gamma": 1.4, "seed": SEED,
            "parallelism": f"replicas{world}" if world > 1 else "single-gpu",
            "l2": "working set ~0.45 GB per GPU > 129 MB L2 (no flush needed)"}


# ---- clocks --------------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r for r in csv.reader(io.StringIO(getattr(self, "out", ""))) if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if present."""
    p = REPO / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        if kernel in d:
            return d[kernel]
    return None


def fp64_pipe_from_profiles(kernel: str):
    """FP64-pipe figures of `kernel` from the committed ncu summary, if present: pipe utilisation
    and FP64 thread-instructions executed per algorithmic flop."""
    p = REPO / "profiles" / "fp64_pipe.json"
    if p.exists():
        d = json.loads(p.read_text())
        if kernel in d:
            return d[kernel]
    return None


def cpu_baseline_sample(threads: int):
    """The oracle (CPU restatement of the reference, OpenMP over rows) on a bounded sample of the
    same workload: a 512 x 512 four-quadrant grid, 10 steps."""
    import oracle
    from hteno import ic

    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    q = ic.four_quadrant(512, 512, SEED)
    oracle.fv2d_run(q, 1, flux=1)  # warm
    t0 = time.perf_counter()
    _, _, n = oracle.fv2d_run(q, 10, flux=1)
    dt = time.perf_counter() - t0
    return {"value": 512 * 512 * n / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "512x512 four-quadrant TENO5+HLLC FP64, 10 steps, CPU oracle (OpenMP)"}


# ---- reference arm ---------------------------------------------------------------------------
def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from hteno import ic

    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    q = ic.four_quadrant(NX, NY, SEED)
    for _ in range(max(0, args.warmup)):
        q, _, _ = oracle.fv2d_run(q, 1, flux=1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q, _, _ = oracle.fv2d_run(q, 1, flux=1)
    el = time.perf_counter() - t0
    value = NX * NY * args.steps / el / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(args, 1, max(0, args.warmup)), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full {NX}x{NY} grid, one step per timed step; the reference's "
                                       "own sources need Eigen3 and cannot be built on the GPU host, so "
                                       "its CPU restatement (pinned bitwise to it) runs instead"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- GB300 arm -------------------------------------------------------------------------------
def batch_path(hteno, torch, stream, steps, world):
    """256 independent grids with sides drawn from {64, ..., 512} (seeded, non-square allowed),
    seeded four-quadrant data each, TENO5 + HLLC, mixed precision, per-instance dt; `steps`
    steps of every instance timed with CUDA events (one graph replay per step)."""
    from hteno import ic

    rng = np.random.default_rng(4)
    sides = rng.integers(64, 513, size=(256, 2))
    cfgs = [hteno.config(dims=2, nx=int(nx), ny=int(ny), flux=hteno.FLUX_HLLC, recon=hteno.RECON_TENO5,
                         precision=hteno.PREC_MIXED) for nx, ny in sides]
    cells = int(sum(int(nx) * int(ny) for nx, ny in sides))
    with hteno.Batch(cfgs) as b:
        b.set_stream(stream.cuda_stream)
        for k, (nx, ny) in enumerate(sides):
            b.set_state(k, ic.four_quadrant(int(nx), int(ny), 1000 + k))
        tile = b.tile()
        b.step(3)  # warm-up (graph capture, first replays)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        b.step_async(steps)
        ev1.record(stream)
        ev1.synchronize()
        b.sync()
        ms = ev0.elapsed_time(ev1)
        done = [b.time(k)[1] for k in range(len(cfgs))]
        status = [b.time(k)[2] for k in range(len(cfgs))]
    return {"value": cells * steps * world / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms / steps,
            "instances": len(cfgs), "cells": cells, "steps": steps, "tile": list(tile),
            "min_steps_done": min(done), "unhealthy_instances": int(sum(1 for s in status if s)),
            "note": "one persistent launch per RK stage over all instances' tiles, a step replayed "
                    "as one CUDA graph; FP32 reconstruction/fluxes, FP64 state; "
                    "unhealthy_instances: grids whose state reached a non-positive density or "
                    "pressure in some RK stage, which the plain FP64 solver (the reference's "
                    "arithmetic bit for bit, no positivity limiter) does on the same seeded data "
                    "within these steps: 14 of the 256, every grid flagged here among them"}


def fused_fp64_path(hteno, torch, cfg, stream, start_state, ref_state, steps, value_plain, kernels,
                    ncell, world):
    """The plain FP64 stage as one fused launch per stage (hteno_set_fp64_fused, tiles of 32 x 16
    cells with face values and fluxes in shared memory) on the headline's timed window: the same
    K steps from the same start state, timed with CUDA events, and its state compared with the
    five-launch path's bit for bit."""
    with hteno.Solver(cfg) as s:
        s.set_stream(stream.cuda_stream)
        s.set_fp64_fused(True)
        s.set_state(start_state)
        s.step_async(steps)  # warm-up over the same steps
        s.sync()
        s.set_state(start_state)  # dt follows from the state alone: the timed steps again
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        s.step_async(steps)
        ev1.record(stream)
        ev1.synchronize()
        s.sync()
        ms = ev0.elapsed_time(ev1)
        same = bool(np.array_equal(s.get_state(), ref_state))
        launches = s.launches_per_step()
    value = ncell * steps * world / (ms / 1e3) / 1e6
    five = sum(k["bytes_per_launch"] * k["launches"] for k in kernels) / steps / ncell
    return {"value": value, "unit": UNIT, "ms_per_step": ms / steps, "vs_five_launch": value / value_plain,
            "same_bits_as_five_launch": same, "launches_per_step": launches,
            "hbm_bytes_per_cell_update": {"fused": 3 * 193.0, "five_launch": five},
            "note": "one launch per stage reads the state once (3-cell halo) and writes it once; the "
                    "tile's halo face rows and columns and its edge fluxes are computed again by the "
                    "neighbouring tiles (+12 % FP64 instructions, measured), and the FP64-bound "
                    "stage pays for that: the five-launch path stays the default"}


def kernel_shares(hteno, solver, steps):
    """Per-kernel share of `steps` more steps, with CUDA events around every launch."""
    import ctypes

    lib = hteno.lib()
    lib.hteno_enable_kernel_timing(solver.h, 1)
    solver.step(steps)
    kt = (hteno.KernelTime * 32)()
    cnt = ctypes.c_int()
    lib.hteno_kernel_timing(solver.h, kt, 32, ctypes.byref(cnt))
    lib.hteno_enable_kernel_timing(solver.h, 0)
    rows = [(kt[k].name.decode(), kt[k].ms) for k in range(cnt.value) if kt[k].launches]
    tot = sum(ms for _, ms in rows) or 1.0
    return {name: round(ms / tot, 4) for name, ms in rows}


def hermite_path(hteno, torch, stream, steps, world, n=2048):
    """Hermite-WENO 2D (FVHermite::System2D) on n x n: 32 seeded Gaussian density blobs on
    rho = 1, p = 1, a Mach-2 shock entering from x = 0, moments by face differences.  Both arms
    (plain FP64, mixed) are timed over the same window, `steps` steps from the initial state;
    the mixed arm's density error is taken against the FP64 state at the FP64 arm's end time."""
    from hteno import ic

    f = ic.blobs_shock_fn(5)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    q = np.ascontiguousarray(f(X, Y))
    v, w = ic.face_difference_moments(f, n, n, 0.0, 1.0, 0.0, 1.0)
    out = {}
    ref = None
    for prec in (hteno.PREC_FP64, hteno.PREC_MIXED):
        cfg = hteno.config(dims=2, scheme=hteno.SCHEME_HERMITE, nx=n, ny=n, flux=hteno.FLUX_RUSANOV,
                           precision=prec)
        with hteno.Solver(cfg) as s:
            s.set_stream(stream.cuda_stream)
            if prec == hteno.PREC_MIXED:  # steps the mixed arm takes to the FP64 arm's end time
                s.set_state(q)
                s.set_moments(v, w)
                s.step(1 << 20, ref[0])
                nmix = s.time()[1]
            s.set_state(q)
            s.set_moments(v, w)
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            s.step_async(steps if prec == hteno.PREC_FP64 else nmix, ref[0] if ref else float("inf"))
            ev1.record(stream)
            ev1.synchronize()
            s.sync()
            ms = ev0.elapsed_time(ev1)
            k = s.time()[1]
            name = "fp64" if prec == hteno.PREC_FP64 else "fp32_mixed"
            out[name] = {"value": n * n * k * world / (ms / 1e3) / 1e6, "unit": UNIT,
                         "ms_per_step": ms / k, "steps": k, "t": s.time()[0]}
            if prec == hteno.PREC_FP64:
                ref = (s.time()[0], s.get_state())
            else:
                l1, linf = density_errors(s.get_state(), ref[1])
                out[name].update({"l1_rho_vs_fp64": l1, "linf_rho_vs_fp64": linf})
                out[name]["kernel_shares"] = kernel_shares(hteno, s, 2)  # separate, after the timing
    out["speedup_mixed_vs_fp64"] = out["fp64"]["ms_per_step"] / out["fp32_mixed"]["ms_per_step"]
    out["workload"] = f"hermite2d_blobs_mach2_{n}x{n}_rusanov_ssprk3"
    out["window"] = f"both arms from the initial state to the FP64 arm's time after {steps} steps"
    return out


def learned_path(hteno, torch, stream, args, world, n=4096):
    """The learned-routing workload: 4096 x 4096 seeded four-quadrant data, TENO5 + HLLC.
    The classifier trains on rows the plain FP64 solver records from runs with fresh seeds of the
    1024^2 four-quadrant problem and the 400-cell Sod tube.  Three arms run over the same window:
    plain FP64 runs `c5_steps` steps from the initial state; FP32 (mixed) and FP32 + learned
    routing (a plain-TENO audit every `c5_audit_every` steps) run from the same initial state to
    the FP64 arm's end time.  Each arm is timed over its whole run; densities are compared at
    that end time."""
    from hteno import ic, learned

    out = {"workload": f"fv2d_fourquadrant_{n}x{n}_teno5_hllc_learned_routing"}
    t0 = time.perf_counter()
    x, y = learned.harvest_runs(hteno, torch, seeds=[201, 202, 203, 204], n=1024,
                                snapshots=(0, 20, 40, 60), keep=1.0)
    t1 = time.perf_counter()
    m = hteno.Mlp(seed=0)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    loss = m.train(x, y, epochs=args.c5_epochs, batch=16384, lr=3e-3)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    acc, routed, mis = learned.accuracy(m, torch, x, y, args.c5_threshold)
    out["training"] = {"rows": int(x.shape[0]), "smooth_fraction": float((y == 7).float().mean().item()),
                       "harvest_s": t1 - t0, "train_s": t3 - t2, "epochs": args.c5_epochs,
                       "rows_per_s": x.shape[0] * args.c5_epochs / (t3 - t2), "final_loss": loss,
                       "bit_accuracy": acc, "routed_fraction": routed, "misrouted_of_routed": mis,
                       "deterministic": "per-CTA partial gradients summed in CTA order"}
    del x, y
    q = ic.four_quadrant(n, n, 7)
    # twice the distance a discontinuity can travel between classifications (cfl 0.4)
    margin = args.c5_margin if args.c5_margin >= 0 else 2 * int(np.ceil(0.4 * args.c5_classify_every - 1e-9))

    def timed_run(s, nsteps, t_end=float("inf")):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        s.step_async(nsteps, t_end)
        ev1.record(stream)
        ev1.synchronize()
        s.sync()
        return ev0.elapsed_time(ev1), s.time()

    cfg64 = hteno.config(dims=2, nx=n, ny=n, flux=hteno.FLUX_HLLC, precision=hteno.PREC_FP64)
    with hteno.Solver(cfg64) as s:
        s.set_stream(stream.cuda_stream)
        s.set_state(q)
        ms64, (t_ref, n64, _) = timed_run(s, nsteps=args.c5_steps)
        ref = s.get_state()
        u64 = s.uniform_cells()
    out["fp64"] = {"value": n * n * n64 * world / (ms64 / 1e3) / 1e6, "unit": UNIT,
                   "ms_per_step": ms64 / n64, "steps": n64, "t_end": t_ref,
                   "uniform_cell_fraction": u64 / (3.0 * n * n * n64)}
    cfg32 = hteno.config(dims=2, nx=n, ny=n, flux=hteno.FLUX_HLLC, precision=hteno.PREC_MIXED)
    arms = (("fp32_plain", None, 1, 0), ("fp32_learned", m, 1, 0),
            ("fp32_learned_every%d" % args.c5_classify_every, m, args.c5_classify_every, margin))
    end_state = None
    for name, router, every, marg in arms:
        with hteno.Solver(cfg32) as s:
            s.set_stream(stream.cuda_stream)
            if router is not None:
                s.set_router(router, args.c5_threshold, args.c5_audit_every)
                s.set_router_schedule(every, marg)
            s.set_state(q)  # (the tile tuner runs when the state is first set)
            s.step(1 << 20, t_ref)  # untimed: the number of steps this arm takes to the end time
            nsteps = s.time()[1]
            s.set_state(q)
            ms, (t_end, nsteps, _) = timed_run(s, nsteps, t_ref)
            st = s.router_stats() if router is not None else None
            got = s.get_state()
            if router is None:
                end_state = got
            uc = s.uniform_cells()
            l1, linf = density_errors(got, ref)
            shift = shock_shift(got, ref)
            shares = kernel_shares(hteno, s, 2)  # a separate pass after the timed run
            a64 = None
            if router is not None:  # the FP64 judge at 5 points of an untimed replay of the run
                s.set_state(q)
                a64 = {"routed": 0, "misrouted64": 0, "routed_resolved": 0, "misrouted64_resolved": 0,
                       "snapshots": 0}
                for _ in range(5):
                    s.step(nsteps // 5, t_ref)
                    a = s.router_audit64()
                    for key in ("routed", "misrouted64", "routed_resolved", "misrouted64_resolved"):
                        a64[key] += a[key]
                    a64["snapshots"] += 1
                a64["misrouted64_of_routed"] = a64["misrouted64"] / max(1, a64["routed"])
                a64["misrouted64_of_routed_resolved"] = a64["misrouted64_resolved"] / max(1, a64["routed_resolved"])
        d = {"value": n * n * nsteps * world / (ms / 1e3) / 1e6, "unit": UNIT,
             "ms_per_step": ms / nsteps, "steps": nsteps, "t_end": t_end,
             "speedup_vs_fp64": (ms64 / n64) / (ms / nsteps),
             "l1_rho_vs_fp64": l1, "linf_rho_vs_fp64": linf, "shock_shift_cells": shift,
             "uniform_cell_fraction": uc / (3.0 * n * n * nsteps), "kernel_shares": shares}
        if st is not None:
            d["router"] = {"audited_stencils": st["seen"], "routed_fraction": st["routed"] / max(1, st["seen"]),
                           "flat_fraction": st["flat"] / max(1, st["seen"]),
                           "routed_of_nonflat": st["routed"] / max(1, st["seen"] - st["flat"]),
                           "network_rows_last_step": st["network_rows"],
                           "misrouted_of_routed_float": st["misrouted"] / max(1, st["routed"]),
                           "fp64_judge": a64,
                           "plain_teno_smooth_fraction": st["smooth"] / max(1, st["seen"]),
                           "audited_steps": st["audits"], "threshold": args.c5_threshold,
                           "audit_every": args.c5_audit_every, "classify_every": every,
                           "margin_faces": marg}
        out[name] = d
    out["learned_vs_fp32_plain"] = out["fp32_plain"]["ms_per_step"] / out["fp32_learned"]["ms_per_step"]
    sched = "fp32_learned_every%d" % args.c5_classify_every
    out["learned_every_vs_fp32_plain"] = out["fp32_plain"]["ms_per_step"] / out[sched]["ms_per_step"]
    # the ceiling of any router: 5 steps from the FP32 arm's end state with every stencil
    # reconstructed by TENO5, then with every stencil taking the linear weights (what routing
    # everything would save at the most; not a valid scheme at discontinuities)
    ceil = {}
    for rname, recon in (("teno5", hteno.RECON_TENO5), ("linear", hteno.RECON_LINEAR)):
        c = hteno.config(dims=2, nx=n, ny=n, flux=hteno.FLUX_HLLC, precision=hteno.PREC_MIXED, recon=recon)
        with hteno.Solver(c) as s:
            s.set_stream(stream.cuda_stream)
            s.set_state(end_state)
            s.step(1)
            s.set_state(end_state)
            ms, _ = timed_run(s, 5)
        ceil[rname + "_ms_per_step"] = ms / 5
    ceil["max_saving"] = 1.0 - ceil["linear_ms_per_step"] / ceil["teno5_ms_per_step"]
    ceil["note"] = ("5 steps from the FP32 arm's end state: every stencil by TENO5 vs every stencil by the "
                    "linear weights; no router can save more than max_saving of a step")
    out["routing_ceiling"] = ceil
    out["smooth_2048"] = learned_smooth(hteno, torch, stream, world, m)
    m.close()
    out["window"] = (f"every arm from the initial state: FP64 {args.c5_steps} steps, the FP32 arms to the "
                     "FP64 arm's end time; errors at that time")
    return out


def learned_smooth(hteno, torch, stream, world, m, n=2048, steps=100):
    """What the trained network gains where the data allow it: a smooth periodic flow on n x n (no
    discontinuity, no flat stencil), FP64 over `steps` steps from the initial state, FP32 and FP32
    + learned routing (classified every 20 steps, masks eroded by 8 faces) from the same state to
    the FP64 arm's end time, each timed over its whole run; density errors against FP64."""
    from hteno import ic

    q = ic.smooth_waves_2d(n, n)
    out = {"workload": f"fv2d_smooth_waves_{n}x{n}_periodic_teno5_hllc"}

    def timed(s, k, t_end=float("inf")):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        s.step_async(k, t_end)
        ev1.record(stream)
        ev1.synchronize()
        s.sync()
        return ev0.elapsed_time(ev1)

    c64 = hteno.config(dims=2, nx=n, ny=n, flux=hteno.FLUX_HLLC, bc=hteno.BC_PERIODIC, precision=hteno.PREC_FP64)
    with hteno.Solver(c64) as s:
        s.set_stream(stream.cuda_stream)
        s.set_state(q)
        ms = timed(s, steps)
        t_ref = s.time()[0]
        ref = s.get_state()
    out["fp64"] = {"value": n * n * steps * world / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms / steps}
    c32 = hteno.config(dims=2, nx=n, ny=n, flux=hteno.FLUX_HLLC, bc=hteno.BC_PERIODIC, precision=hteno.PREC_MIXED)
    for name, router in (("fp32_plain", None), ("fp32_learned_every20", m)):
        with hteno.Solver(c32) as s:
            s.set_stream(stream.cuda_stream)
            if router is not None:
                s.set_router(router, 0.99, 0)
                s.set_router_schedule(20, 8)
            s.set_state(q)
            s.step(1 << 20, t_ref)
            k = s.time()[1]
            s.set_state(q)
            ms = timed(s, k, t_ref)
            l1, linf = density_errors(s.get_state(), ref)
            d = {"value": n * n * k * world / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms / k, "steps": k,
                 "l1_rho_vs_fp64": l1, "linf_rho_vs_fp64": linf}
            if router is not None:
                d["fp64_judge_end"] = s.router_audit64()
            out[name] = d
    out["learned_vs_fp32_plain"] = out["fp32_plain"]["ms_per_step"] / out["fp32_learned_every20"]["ms_per_step"]
    return out


def sod_path(hteno, torch):
    """The 1D benchmark tube: 400 cells, Sod data, TENO5 + HLLC, CFL 0.5, plain FP64, to t = 0.2
    (a latency case): wall time of the whole run through the C-ABI on the GPU and of the CPU
    oracle (one thread, as the reference's 1D solver runs), and the largest difference."""
    import oracle
    from hteno import ic

    q = ic.sod(400)
    cfg = hteno.config(dims=1, nx=400, flux=hteno.FLUX_HLLC, recon=hteno.RECON_TENO5, cfl=0.5,
                       precision=hteno.PREC_FP64)
    with hteno.Solver(cfg) as s:
        s.set_state(q)
        s.step(1 << 20, 0.2)  # warm
        s.set_state(q)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(1 << 20, 0.2)
        gpu_s = time.perf_counter() - t0
        _, n, _ = s.time()
        got = s.get_state()
    t0 = time.perf_counter()
    want, _, n_o = oracle.fv1d_run(q, 1 << 20, t_final=0.2, flux=1, recon=0, cfl=0.5)
    cpu_s = time.perf_counter() - t0
    return {"workload": "fv1d_sod_400_teno5_hllc_cfl0.5_t0.2_fp64", "steps": n, "gpu_wall_s": gpu_s,
            "cpu_oracle_wall_s": cpu_s, "cpu_cores": 1, "max_abs_diff_vs_oracle": float(np.abs(got - want).max()),
            "value": 400 * n / gpu_s / 1e6, "unit": UNIT}


def density_errors(a, b):
    from hteno import metrics

    return metrics.density_errors(a, b)


def shock_shift(a, b):
    from hteno import metrics

    return metrics.shock_shift(a[0], b[0])


def mixed_path(hteno, torch, q, stream, args, t_end, ref_state, ms_plain, world):
    """Times K steps of the mixed path after W warm-up steps (the same counts as the plain run),
    then finishes the run at the plain run's end time and reports the density error."""
    cfg = hteno.config(dims=2, nx=NX, ny=NY, flux=hteno.FLUX_HLLC, recon=hteno.RECON_TENO5,
                       precision=hteno.PREC_MIXED)
    with hteno.Solver(cfg) as s:
        s.set_stream(stream.cuda_stream)
        s.set_state(q)
        s.step_async(max(args.warmup, args.start_step))
        s.sync()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        s.step_async(args.steps)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        s.step(1 << 20, t_end)
        t, n, _ = s.time()
        l1, linf = density_errors(s.get_state(), ref_state)
    return {"value": NX * NY * args.steps * world / (ms / 1e3) / 1e6, "unit": UNIT,
            "ms_per_step": ms / args.steps, "speedup_vs_fp64": ms_plain / ms,
            "l1_rho_vs_fp64": l1, "linf_rho_vs_fp64": linf, "t": t, "steps_to_t": n,
            "note": "FP32 reconstruction/fluxes, FP64 state and SSP-RK3; error against the plain "
                    "FP64 GPU state at the same time (bit-identical to the CPU oracle)"}


def run_gpu(args):
    import torch

    import hteno
    from hteno import ic

    world, rank, local = dist_setup(torch)
    lib = hteno.lib()
    q = ic.four_quadrant(NX, NY, SEED)
    ncell = NX * NY
    cfg = hteno.config(dims=2, nx=NX, ny=NY, flux=hteno.FLUX_HLLC, recon=hteno.RECON_TENO5,
                       precision=hteno.PREC_FP64)
    stream = torch.cuda.Stream()
    solver = hteno.Solver(cfg)
    solver.set_stream(stream.cuda_stream)
    solver.set_state(q)
    launches = solver.launches_per_step()

    # warm-up: W steps, and on to the start step of the timed region (the middle of the
    # configuration's 200-step run, so the timed steps see its typical wave pattern rather than
    # the nearly uniform first steps, where constant windows shortcut the reconstruction)
    solver.step_async(max(args.warmup, args.start_step))
    solver.sync()
    start_state = solver.get_state()

    # timed region: K steps, device-resident, CUDA events on the solver's stream, nothing else
    # inside it (per-kernel times come from a separate pass below)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
                    if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else local)
    uni0 = solver.uniform_cells()
    barrier(torch, world)
    torch.cuda.synchronize()
    with clocks:
        time.sleep(0.3)
        ev0.record(stream)
        solver.step_async(args.steps)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
    barrier(torch, world)
    solver.sync()
    ms = ev0.elapsed_time(ev1)
    t_plain, _, _ = solver.time()
    ref_state = solver.get_state()
    uniform_fraction = (solver.uniform_cells() - uni0) / (3.0 * ncell * args.steps)
    ms_max = allreduce_max(torch, world, ms)
    value = ncell * args.steps * world / (ms_max / 1e3) / 1e6

    # per-kernel times of the same K steps, replayed from the timed region's start state with CUDA
    # events bracketing every launch (set_state restarts the clock at 0; dt follows from the state
    # alone, so the replayed steps are the timed ones)
    import ctypes

    solver.set_state(start_state)
    lib.hteno_enable_kernel_timing(solver.h, 1)
    solver.step_async(args.steps)
    solver.sync()
    kt = (hteno.KernelTime * 16)()
    cnt = ctypes.c_int()
    lib.hteno_kernel_timing(solver.h, kt, 16, ctypes.byref(cnt))
    lib.hteno_enable_kernel_timing(solver.h, 0)
    kernels = []
    for k in range(cnt.value):
        e = kt[k]
        if e.launches:
            kernels.append({"name": e.name.decode(), "launches": e.launches, "ms": e.ms,
                            "bytes_per_launch": e.bytes_per_launch, "flops_per_launch": e.flops_per_launch})
    tot = sum(k["ms"] for k in kernels) or 1.0
    for k in kernels:
        k["share"] = k["ms"] / tot
    dom = max(kernels, key=lambda k: k["ms"])
    avg_s = dom["ms"] / dom["launches"] / 1e3
    hbm, hbm_src = peaks()
    fp64_peak = hteno.measure_fma_peak(0)
    achieved = dom["flops_per_launch"] / avg_s / 1e12
    step_flops = sum(k["flops_per_launch"] * k["launches"] for k in kernels) / args.steps
    roofline = {"bound": "fp64", "kernel": dom["name"], "achieved": achieved, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                "peak_source": "measured FP64 FMA throughput of this GPU (hteno_measure_fma_peak; "
                               "MEASURED_PEAKS.json has no FP64 figure)",
                "traffic": traffic_from_profiles(dom["name"]),
                "flops_note": "algorithmic flops of the reference per launch (+,-,*,/,sqrt = 1, pow = 1), "
                              "op-counted on the oracle, for every face of the launch including the "
                              "uniform-region faces the path skips exactly",
                "hbm": {"achieved": dom["bytes_per_launch"] / avg_s / 1e9, "peak": hbm, "unit": "GB/s",
                        "frac": dom["bytes_per_launch"] / avg_s / 1e9 / hbm,
                        "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)" if hbm_src == "measured"
                                       else "fallback 6.8 TB/s"},
                "fp64_pipe": fp64_pipe_from_profiles(dom["name"]),
                "step": {"achieved_tflops": step_flops * args.steps / (ms / 1e3) / 1e12,
                         "frac_of_fp64_peak": step_flops * args.steps / (ms / 1e3) / 1e12 / fp64_peak},
                "uniform_cell_fraction": uniform_fraction,
                "kernels": kernels,
                "note": "the bit-reproducible FP64 kernels are bound by the FP64 pipe (2 FP64 operations "
                        "per SM per cycle on GB300), not by HBM; uniform_cell_fraction is the share of "
                        "cell-stages of the timed steps whose exactly zero residual was taken without "
                        "computing their faces"}

    # end to end through the C-ABI with pinned host buffers: every step copies the state in,
    # advances one step and reads the state back
    e2e = None
    if not args.no_e2e:
        # the same K steps as the timed region: the host holds the state, each step uploads it,
        # advances it and downloads the result, which is the next step's input
        hq = torch.from_numpy(start_state).pin_memory()
        hout = torch.empty_like(hq).pin_memory()
        e2e_steps = max(1, args.steps)
        barrier(torch, world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            solver.set_state(hq)
            solver.step(1)
            solver.get_state(hout)
            hq, hout = hout, hq
        el = time.perf_counter() - t0
        el = allreduce_max(torch, world, el)
        nbytes = q.nbytes
        e2e = {"value": ncell * e2e_steps * world / el / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}

    # the mixed path (FP32 reconstruction and fluxes, FP64 state and RK accumulation) on the same
    # workload, advanced to the same time as the plain path; density error against the plain
    # FP64 state, which is bit-identical to the CPU oracle
    paths = {}
    if not args.no_fused:
        paths["fp64_fused"] = fused_fp64_path(hteno, torch, cfg, stream, start_state, ref_state,
                                              args.steps, value, kernels, ncell, world)
    if not args.no_mixed:
        paths["fp32_mixed"] = mixed_path(hteno, torch, q, stream, args, t_plain, ref_state, ms_max, world)
    if not args.no_sod and rank == 0:
        paths["sod_1d_400"] = sod_path(hteno, torch)
    if not args.no_hermite:
        paths[f"hermite_{args.hermite_n}"] = hermite_path(hteno, torch, stream, args.hermite_steps, world,
                                                           n=args.hermite_n)
    if not args.no_learned:
        paths["learned_4096"] = learned_path(hteno, torch, stream, args, world)
    if not args.no_batch:
        paths["batch_256_mixed"] = batch_path(hteno, torch, stream, args.batch_steps, world)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(args, world, max(args.warmup, args.start_step)),
            "gpu_launches": launches * args.steps,
            "clocks": clocks.summary(), "roofline": roofline, "e2e": e2e, "paths": paths}
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(os.cpu_count() or 1)
    solver.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    args = parse()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
