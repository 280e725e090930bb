#!/usr/bin/env python
"""Benchmark of the GB300 Richards-equation step: cells*steps/s.

Default workload: the combined configuration, 768x768x96 cells (56.6M) of three-layer soil
(sand / loam / clay at seeded interface depths, in-layer ln Ks GRF sigma 1.5), dry start
h = -5 m, 50 mm/h rain for 1800 s then none, free-drainage bottom, mixed-form modified Picard
(|dh|_inf < 1e-6 m) with a Picard-count time step in [10, 120] s.  A "step" is one time step
over the whole grid, all its Picard iterations included.  The timed arm is the learned +
mixed-precision solver (FP32 flexible CG with z = M_line^-1 r + NN(r) inside FP64 iterative
refinement to a true relative residual of 1e-12, network time policy and iteration fallback);
the Picard kernels (constitutive relations, assembly, final update) compute in float-float
arithmetic on the FP32 pipe (--picard-fp64: native FP64).  The same steps are then run with the
plain FP64 path (native FP64 Picard kernels, FP64 Jacobi-PCG at rtol 1e-12) for the comparison
and the head error between the two.  Inputs are seeded and synthetic; the working set (> 10 GB)
is far larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--config c0..c4] [--scheme pca|picard] [--precision fp64|mixed]
                    [--pc jacobi|line|unet|unet-line] [--picard-fp64]

--impl reference times the CPU restatement of the reference path (oracle/, OpenMP on every
host core) on a bounded window of the same workload; under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Richards cells·steps/s at 1e-8 m head error: learned+mixed vs plain FP64 PCG"
UNIT = "cells·steps/s"

# per-configuration defaults: scheme, precision, inner preconditioner, timed steps,
# oracle window (columns per side) for the CPU legs
DEFAULTS = {
    "c0": dict(scheme="picard", precision="fp64", pc="jacobi", steps=120, window=40),
    "c1": dict(scheme="picard", precision="fp64", pc="jacobi", steps=20, window=64),
    "c2": dict(scheme="picard", precision="mixed", pc="jacobi", steps=10, window=64),
    "c3": dict(scheme="picard", precision="mixed", pc="unet-line", steps=10, window=64),
    "c4": dict(scheme="picard", precision="mixed", pc="line", steps=20, window=64),
}

# algorithmic bytes per cell of one launch as the hot-path scope table states them (the
# roofline's `achieved`): the fused Picard / PCA assembly 72 (read h, theta^n, ln Ks, ln alpha;
# write the four operator entries and the right-hand side), the Picard update 32, the step-start
# copy 16.  Kernels without such a figure use their own compulsory bytes (the library's labels).
SCOPE_BYTES_PER_CELL = {"k_pic_assemble_ff": 72.0, "k_pic_assemble": 72.0, "k_assemble": 72.0,
                        "k_pic_update": 32.0, "k_copy64": 16.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c4", choices=sorted(DEFAULTS))
    ap.add_argument("--scheme", default=None, choices=["pca", "picard"])
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"])
    ap.add_argument("--pc", default=None, choices=["jacobi", "line", "unet", "unet-line"])
    ap.add_argument("--inner-rtol", type=float, default=None,
                    help="relative reduction of each FP32 inner solve (mixed precision; "
                         "default 1e-6: two refinement sweeps reach 1e-12)")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain FP64 arm (comparison and head error)")
    ap.add_argument("--unet-weights", default=None,
                    help="trained network (.npz written by python -m frehg_gb300.learned); "
                         "default: the committed layered-soil network when it exists, else "
                         "a bounded training run before the timed steps")
    ap.add_argument("--train-steps", type=int, default=300)
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-window", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--picard-fp64", action="store_true",
                    help="Picard kernels in native FP64 instead of float-float on the FP32 pipe")
    ap.add_argument("--profile-steps", type=int, default=1)
    ap.add_argument("--staged-assembly", action="store_true",
                    help="stage the Picard assembly's inputs through TMA (same results)")
    ap.add_argument("--learned-window", type=int, default=128,
                    help="columns per side of the learned-preconditioner record (0: skip)")
    ap.add_argument("--nx", type=int, default=None, help="window of the workload (smaller case)")
    ap.add_argument("--ny", type=int, default=None)
    a = ap.parse_args()
    d = DEFAULTS[a.config]
    a.scheme = a.scheme or d["scheme"]
    a.precision = a.precision or d["precision"]
    a.pc = a.pc or (d["pc"] if a.precision == "mixed" else "jacobi")
    a.steps = a.steps or d["steps"]
    a.ref_window = a.ref_window or d["window"]
    if a.pc != "jacobi" and a.precision != "mixed":
        ap.error(f"--pc {a.pc} runs in the mixed-precision solve (--precision mixed)")
    return a


def workload(args, nx=None, ny=None, precision=None, pc=None):
    """The configuration's workload (optionally a window of nx x ny columns) with the solver
    selected by precision / pc (default: the command line's)."""
    from frehg_gb300 import workloads as W
    prec = 1 if (precision or args.precision) == "mixed" else 0
    pc = pc or args.pc
    if nx is None and args.nx:
        nx, ny = args.nx, args.ny or args.nx
    kw = {} if nx is None else dict(nx=nx, ny=ny)
    if args.config == "c0":
        w = W.config0(args.scheme, **kw)
    elif args.config == "c1":
        w = W.config1(args.scheme, precision=prec, **kw)
    elif args.config == "c2":
        w = W.config2(args.scheme, **kw)
    elif args.config == "c3":
        w = W.config3(args.scheme, precision=prec, pc=pc if prec else "jacobi", **kw)
    else:
        w = W.config4(precision=prec, pc=pc if prec else "jacobi", **kw)
    w.solver.precision = prec
    w.solver.pc_type = (pc if prec else "jacobi").encode()
    # float-float Picard kernels with the mixed-precision solve, FP64 ones with the FP64 solve
    # (the library's default) or where --picard-fp64 asks for them
    w.params.picard_fp64 = 1 if getattr(args, "picard_fp64", False) or not prec else 0
    if prec:
        w.solver.ir_rtol = 1e-12
        w.solver.inner_rtol = args.inner_rtol or 1e-6
    return w


FULL_COLUMNS = {"c0": 40, "c1": 256, "c2": 512, "c3": 256, "c4": 768}


def window(args, side, **kw):
    """A bounded sample of the workload: the same generator on side x side columns.  Returns
    the full workload's name and the window."""
    full = args.nx or FULL_COLUMNS[args.config]
    fully = args.ny or full
    side = min(side, full, fully)
    w = workload(args, nx=side, ny=side, **kw)
    return w.name.replace(f"{side}x{side}x", f"{full}x{fully}x", 1), w


def workload_config(args, name, cells):
    """The `config` both arms print: what the workload is, nothing about the solver that ran."""
    return {"workload": name, "cells": int(cells), "scheme": args.scheme,
            "l2": "working set larger than the 129 MB L2 (no flush needed)"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id):
        self.bus_id = bus_id
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                   "-lms", "200"]
            if self.bus_id:
                cmd += ["-i", self.bus_id]
            self.proc = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        self.f.close()
        os.unlink(self.f.name)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(smax), reasons=sorted(reasons),
                       samples=len(sm))
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def measured_bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if d.get("bf16_tflops"):
            return d["bf16_tflops"], "measured (burst)"
    return 1900.0, "fallback (burst)"


def network_roofline(net, w, stream):
    """One forward application of the network on the workload's grid, timed with CUDA events
    (mean of 3 after 2 warm-up applications) against the dense BF16 tensor peak."""
    import torch
    from frehg_gb300.abi import check, load_library
    from frehg_gb300.learned import UNet
    lib = load_library()
    n = w.cells
    g = torch.Generator(device="cuda").manual_seed(0)
    r = torch.randn(n, device="cuda", generator=g)
    lnk = torch.randn(n, device="cuda", generator=g)
    cap = torch.rand(n, device="cuda", generator=g)
    y = torch.empty(n, device="cuda")

    def apply():
        check(lib.frehg_unet_forward(net.handle, w.nx, w.ny, w.nz, r.data_ptr(), lnk.data_ptr(),
                                     cap.data_ptr(), y.data_ptr(), stream.cuda_stream), "forward")

    for _ in range(2):
        apply()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        apply()
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1) / 3
    flops = UNet.flops(w.nx, w.ny, w.nz)
    peak, kind = measured_bf16_peak()
    tf = flops / (ms / 1000.0) / 1e12
    del r, lnk, cap, y
    torch.cuda.empty_cache()
    return {"bound": "tensor", "kernel": "U-Net forward (k_conv3_tcz / k_conv3_tc: tcgen05.mma "
                                          "BF16, FP32 accumulators in TMEM)",
            "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
            "peak_source": kind, "ms_per_application": ms, "flop_per_application": flops}


def ncu_table():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def ncu_traffic(kernel):
    """(DRAM bytes per cell, limiter) of `kernel` from the committed ncu summary (profiles/)"""
    v = ncu_table().get(kernel)
    if isinstance(v, dict):
        return v.get("dram_bytes_per_cell"), v.get("limiter")
    return v, None


def scheme_name(args):
    return "mixed-form Picard" if args.scheme == "picard" else "PCA (ReSolver::advanceStep)"


def cpu_rate(args, seconds, max_steps=None):
    """Time the oracle (FP64 CPU restatement of the step, OpenMP on every host core) on a
    bounded window of the workload: the timed steps of the GPU arm (the first args.steps steps),
    repeated from the initial state until about `seconds` have passed; returns
    (cells*steps/s, threads, sample description)."""
    from oracle import oracle
    oracle.build()
    full_name, w = window(args, args.ref_window, precision="fp64", pc="jacobi")
    threads = oracle.num_threads()
    el, steps, passes = 0.0, 0, 0
    while el < seconds and not (max_steps and steps >= max_steps):
        o = oracle.OracleRe(w.nx, w.ny, w.nz, w.params)
        w.apply(o)
        passes += 1
        t0 = time.perf_counter()
        for _ in range(args.steps):
            o.advance_step()
            steps += 1
            if el + time.perf_counter() - t0 >= seconds or (max_steps and steps >= max_steps):
                break
        el += time.perf_counter() - t0
        del o
    rate = w.cells * steps / el
    sample = (f"{steps} {scheme_name(args)} steps ({passes} pass(es) over the first "
              f"{args.steps}) of {full_name}'s generator on a {w.nx}x{w.ny}x{w.nz} window "
              f"({w.cells} cells), {el:.1f} s, {threads} OpenMP threads, FP64 CG+Jacobi "
              f"rtol 1e-12")
    return rate, threads, sample


def run_reference(args):
    """The reference's CPU path: the oracle restatement, all host threads, per-step samples of
    a bounded window of the same workload."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from oracle import oracle
    oracle.build()
    full_name, w = window(args, args.ref_window, precision="fp64", pc="jacobi")
    full_cells = (args.nx or FULL_COLUMNS[args.config]) * (args.ny or args.nx or
                                                           FULL_COLUMNS[args.config]) * w.nz
    o = oracle.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    for _ in range(args.warmup):
        o.advance_step()
    o = oracle.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.advance_step()
    el = time.perf_counter() - t0
    value = w.cells * args.steps / el
    threads = oracle.num_threads()
    sample = (f"first {args.steps} {scheme_name(args)} steps of {full_name}'s generator on a "
              f"{w.nx}x{w.ny}x{w.nz} window ({w.cells} cells), {threads} OpenMP threads, CPU "
              f"restatement of the reference path (FP64, CG+Jacobi rtol 1e-12)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded soil fields)",
        "config": workload_config(args, full_name, full_cells),
        "arm": {"sample_window": f"{w.nx}x{w.ny}x{w.nz}", "precision": "fp64",
                "solver": "cg+jacobi rtol 1e-12"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def trained_net(args):
    """The network of the learned arm: loaded from --unet-weights, or trained here (outside the
    timed region) on pairs from plain solves of seeded three-layer soils at 64x64x32."""
    from frehg_gb300 import learned as Lr
    net = Lr.UNet(0)
    path = args.unet_weights or (Lr.DEFAULT_WEIGHTS if os.path.exists(Lr.DEFAULT_WEIGHTS)
                                 else None)
    if path:
        net.load(path)
        info = {"weights": os.path.relpath(path, ROOT)}
        try:
            import numpy as np
            info.update(json.loads(str(np.load(path)["info"])))
        except Exception:
            pass
        return net, info
    t0 = time.perf_counter()
    seeds = list(range(100, 100 + args.train_seeds))
    data = Lr.generate_pairs(seeds, 64, 64, 32, snapshots=(0, 2), iters=(0, 2, 5, 10, 20, 40),
                             pc=args.pc)
    t1 = time.perf_counter()
    losses = Lr.train(net, data, steps=args.train_steps, lr=1e-3)
    t2 = time.perf_counter()
    k = max(1, len(losses) // 10)
    info = {"pairs": int(data["r"].shape[0]), "pair_shape": "64x64x32", "seeds": len(seeds),
            "adam_steps": args.train_steps, "lr": 1e-3, "pairs_s": round(t1 - t0, 2),
            "train_s": round(t2 - t1, 2),
            "loss_first": float(sum(losses[:k]) / k), "loss_last": float(sum(losses[-k:]) / k),
            "note": "bounded training budget for the benchmark run"}
    del data
    return net, info


def learned_record(args, stream, net, info):
    """The learned preconditioner forced on for every solve, beside the same refinement without
    it (line-PCG), on a window of the learned-preconditioner configuration: three-layer soil,
    Picard steps, FP32 Krylov under FP64 refinement to a true relative residual of 1e-12.
    Reports per arm the inner (FP32) iterations, the time of the solves and of the steps (CUDA
    events), the network applications and fallbacks, and the head difference between the arms."""
    import torch
    import numpy as np
    from frehg_gb300 import workloads as W
    from frehg_gb300.abi import check
    from frehg_gb300.re_solver import Grid, ReSolver
    n = args.learned_window
    steps = 3
    out, heads = {}, {}
    for pc in ("line", "unet-line"):
        w = W.config3("picard", nx=n, ny=n, nz=128, steps=steps, pc=pc)
        s = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
        s.set_stream(stream.cuda_stream)
        w.apply(s)
        if pc != "line":
            check(s._lib.frehg_re_attach_unet(s._h, net.handle), "attach_unet")
            check(s._lib.frehg_re_set_learned_policy(s._h, 0, 1e9), "policy")
        its, c0 = [], s.counters()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            a = s.counters()
            s.advance_step()
            its.append(int(s.counters().ksp_iterations - a.ksp_iterations))
        e1.record(stream)
        stream.synchronize()
        c1 = s.counters()
        heads[pc] = s.interior("h").copy()
        out[pc] = {"inner_iterations_per_step": its,
                   "picard_iterations": int(c1.picard_iterations - c0.picard_iterations),
                   "ms_steps": round(e0.elapsed_time(e1), 2),
                   "ms_solves": round((c1.net_ms + c1.plain_ms) - (c0.net_ms + c0.plain_ms), 2),
                   "network_solves": int(c1.net_solves - c0.net_solves),
                   "fallbacks": int(c1.fcg_fallbacks - c0.fcg_fallbacks)}
        del s
    dh = np.abs(heads["line"] - heads["unet-line"])
    return {"workload": f"c3-picard-{n}x{n}x128 window, {steps} steps",
            "network": info, "line": out["line"], "learned_forced_on": out["unet-line"],
            "head_difference_m": float(dh.max()),
            "solve_time_ratio_learned_over_line": round(
                out["unet-line"]["ms_solves"] / max(out["line"]["ms_solves"], 1e-9), 3)}


def time_arm(args, w, net, stream, barrier, steps, warmup):
    """W warm-up steps, reset, K timed steps (CUDA events on the library's stream).  Returns the
    solver, elapsed ms and the counter deltas of the timed steps."""
    import torch
    from frehg_gb300.abi import check
    from frehg_gb300.re_solver import Grid, ReSolver
    s = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    s.set_stream(stream.cuda_stream)
    if getattr(args, "staged_assembly", False):
        s.set_assembly_staging(True)

    def reset():
        s.set_params(w.params)
        w.apply(s)
        if net is not None:
            check(s._lib.frehg_re_attach_unet(s._h, net.handle), "attach_unet")

    reset()
    for _ in range(warmup):
        s.advance_step()
    reset()
    c0 = s.counters()
    v0 = s.water_volume()
    top0, bot0 = s.boundary_volumes()
    el0 = s.elastic_volume()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        s.advance_step()
    e1.record(stream)
    stream.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    c1 = s.counters()
    d = {f: getattr(c1, f) - getattr(c0, f) for f in
         ("ksp_iterations", "picard_iterations", "kernel_launches", "ir_sweeps", "fcg_fallbacks",
          "net_solves", "net_skipped", "net_ms", "plain_ms")}
    top, bot = s.boundary_volumes()
    mass = (s.water_volume() - v0) + (s.elastic_volume() - el0) - ((top - top0) + (bot - bot0))
    d["mass_error_rel"] = abs(mass) / v0
    return s, ms, d, reset


def step_roofline(args, w, cnt, ms):
    """The whole timed region against the copy peak, with the hot-path scope table's per-cell
    algorithmic bytes: 16 per step (step-start copy), 72 + 32 per Picard iteration (or per PCA
    step: assembly, update/corrector) and 80 per Krylov iteration in FP64, 40 per FP32 inner
    iteration (half the vector and coefficient bytes)."""
    its = cnt["picard_iterations"] if args.scheme == "picard" else args.steps
    per_krylov = 40.0 if args.precision == "mixed" else 80.0
    b = w.cells * (16.0 * args.steps + 104.0 * its + per_krylov * cnt["ksp_iterations"])
    gbs = b / (ms / 1000.0) / 1e9
    peak, kind = measured_peaks()
    return {"bytes_per_step": b / args.steps, "achieved": gbs, "peak": peak, "unit": "GB/s",
            "frac": gbs / peak, "peak_source": kind,
            "formula": "cells x (16 x steps + 104 x " +
                       ("Picard iterations" if args.scheme == "picard" else "steps") +
                       f" + {per_krylov:.0f} x Krylov iterations)"}


def rank_ops(world, local, backend="nccl"):
    """The replicas' host-side coordination: (barrier, max_over_ranks).  One process per GPU,
    no collective on the data path; the barrier brackets the timed region and the slowest
    rank's time sets the job's.  backend "nccl" on GPUs (the device is synchronised as well),
    "gloo" for the CPU tests of this logic."""
    import torch
    pg = None
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", local))
            else:
                dist.init_process_group(backend)
        pg = dist
    on_gpu = backend == "nccl"

    def barrier():
        if pg:
            pg.barrier()
        if on_gpu:
            torch.cuda.synchronize()

    def max_over_ranks(v):
        if not pg:
            return v
        t = torch.tensor([float(v)], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def replica_rate(cells, steps, world, ms_max):
    """whole-job cells·steps/s of `world` replicas that each ran `steps` steps of `cells`
    cells, the slowest taking ms_max milliseconds"""
    return cells * steps * world / (ms_max / 1000.0)


def run_gpu(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    barrier, max_over_ranks = rank_ops(world, local)

    from frehg_gb300 import build as B
    B.build()

    learned = args.pc.startswith("unet")
    net, net_info = trained_net(args) if learned else (None, None)
    w = workload(args)
    stream = torch.cuda.Stream()
    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id
    except Exception:
        pass
    clocks = Clocks(bus)
    clocks.start()
    s, ms, cnt, reset = time_arm(args, w, net, stream, barrier, args.steps, args.warmup)
    clk = clocks.stop()
    ms_max = max_over_ranks(ms)
    value = replica_rate(w.cells, args.steps, world, ms_max)
    h_fast = s.interior("h").copy()

    # end to end through the public API: per step H2D of the top forcing (rain or qtop per
    # column) from pinned host memory, the step, D2H of the head and water-content fields into
    # pinned memory (asynchronous: each step's copy overlaps the next step; the timer stops
    # after the last copy has landed)
    reset()
    qv = w.params.rain_rate if w.params.rain_rate != 0.0 else w.params.qtop
    q_host = torch.full((w.ny * w.nx,), float(qv), dtype=torch.float64).pin_memory()
    h_host = torch.empty((w.nz, w.ny, w.nx), dtype=torch.float64).pin_memory()
    wc_host = torch.empty((w.nz, w.ny, w.nx), dtype=torch.float64).pin_memory()
    qn, hn, wn = q_host.numpy(), h_host.numpy(), wc_host.numpy()

    def e2e_step():
        s.set_top_flux_field(qn)
        s.advance_step()
        s.interior_async("h", hn)
        s.interior_async("wc", wn)

    # untimed warm-up steps through the same calls (first touches of the pinned buffers and
    # of the copy stream), then the K timed steps from the same initial state as the device arm
    for _ in range(args.warmup):
        e2e_step()
    s.sync()
    reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    s.sync()
    e1.record(stream)
    stream.synchronize()
    barrier()
    e2e_ms = max_over_ranks(max(e0.elapsed_time(e1), 1000.0 * (time.perf_counter() - t0)))
    e2e_value = replica_rate(w.cells, args.steps, world, e2e_ms)

    # per-kernel durations from CUDA events on the launching stream (profiling pass)
    reset()
    s.set_profiling(1)
    for _ in range(args.profile_steps):
        s.advance_step()
    stats = s.kernel_stats() if args.profile_steps > 0 else [
        {"name": "none", "launches": 1, "total_ms": 1.0, "bytes_per_launch": 0.0}]
    s.set_profiling(0)
    del s
    tot = sum(st["total_ms"] for st in stats) or 1.0
    dom = max(stats, key=lambda st: st["total_ms"])
    # per launch that did work (inner Krylov launches after convergence return at once)
    per_launch_ms = dom["total_ms"] / max(1, dom["launches"] - dom.get("idle_launches", 0))
    scope_bpc = SCOPE_BYTES_PER_CELL.get(dom["name"])
    alg_bytes = scope_bpc * w.cells if scope_bpc else dom["bytes_per_launch"]
    achieved = alg_bytes / (per_launch_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    tr, limiter = ncu_traffic(dom["name"])
    roofline = {
        "bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind, "limiter": limiter,
        "traffic": None if tr is None else tr * w.cells,
        "bytes_per_launch": alg_bytes,
        "bytes_per_cell": alg_bytes / w.cells,
        "bytes_per_cell_source": ("hot-path scope table" if scope_bpc else
                                  "kernel's compulsory bytes"),
        "kernel_compulsory_bytes_per_cell": dom["bytes_per_launch"] / w.cells,
        "ms_per_launch": per_launch_ms,
        "share_of_step": dom["total_ms"] / tot,
        # GBps: algorithmic bytes of the launches that did work (inner Krylov iterations are
        # launched in whole chunks; those after convergence return at once: idle_launches)
        "kernels": {st["name"]: {"launches": st["launches"],
                                 "idle_launches": st.get("idle_launches", 0),
                                 "ms": round(st["total_ms"], 4),
                                 "share": round(st["total_ms"] / tot, 4),
                                 "GBps": round(st["bytes_per_launch"] *
                                               (st["launches"] - st.get("idle_launches", 0)) /
                                               (st["total_ms"] / 1000.0) / 1e9, 1)
                                 if st["total_ms"] > 0 else 0.0,
                                 # ncu's FP64-pipe active fraction (profiles/), the bound of the
                                 # kernels whose HBM fraction is low
                                 "fp64_pipe_pct_ncu": (ncu_table().get(st["name"]) or {}).get(
                                     "fp64_pipe_pct", None) if isinstance(
                                     ncu_table().get(st["name"]), dict) else None}
                    for st in stats},
    }

    # the network: its tensor-pipe roofline on this grid, and the forced-on record
    lnet, linfo = net, net_info
    want_rec = args.learned_window > 0 and rank == 0 and args.scheme == "picard"
    if lnet is None and want_rec:
        lnet, linfo = trained_net(argparse.Namespace(**dict(vars(args), pc="unet-line")))
    net_roof = network_roofline(lnet, w, stream) if lnet is not None else None
    learned_rec = None
    if want_rec:
        torch.cuda.empty_cache()
        learned_rec = learned_record(args, stream, lnet, linfo)

    # the plain FP64 GPU path on the same inputs and steps (FP64 Jacobi-PCG, native FP64
    # Picard kernels): throughput and head error
    comparison = None
    ff_kernels = args.scheme == "picard" and not w.params.picard_fp64
    if not args.no_compare and (args.precision != "fp64" or args.pc != "jacobi" or ff_kernels):
        torch.cuda.empty_cache()
        from frehg_gb300.abi import SolverConfig
        p64 = type(w.params).from_buffer_copy(w.params)
        p64.picard_fp64 = 1
        w64 = dataclasses.replace(w, params=p64,
                                  solver=SolverConfig("cg", "jacobi", rtol=w.solver.rtol,
                                                      max_it=w.solver.max_it))
        s64, ms64, cnt64, _ = time_arm(args, w64, None, stream, barrier, args.steps,
                                       args.warmup)
        ms64 = max_over_ranks(ms64)
        h64 = s64.interior("h")
        del s64
        dh = np.abs(h_fast - h64)
        v64 = replica_rate(w.cells, args.steps, world, ms64)
        comparison = {
            "plain_fp64": {"value": v64, "ms_per_step": ms64 / args.steps,
                           "cg_iterations": cnt64["ksp_iterations"],
                           "picard_iterations": cnt64["picard_iterations"],
                           "mass_error_rel": cnt64["mass_error_rel"]},
            "speedup": value / v64,
            "head_error_vs_plain_fp64_m": {"max": float(dh.max()),
                                           "l2_rms": float(np.sqrt(np.mean(dh * dh))),
                                           "after_steps": args.steps},
        }

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        torch.cuda.empty_cache()
        rate, threads, sample = cpu_rate(args, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    solver = (f"cg+jacobi rtol 1e-12 (fp64)" if args.precision == "fp64" else
              f"fp32 {'fcg' if learned else 'pcg'} + {args.pc} under fp64 refinement to "
              f"true relative residual 1e-12")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("f64" if args.precision == "fp64" else "f64+f32" + ("+bf16" if learned else ""))
                 + ("+ff" if args.scheme == "picard" and not w.params.picard_fp64 else ""),
        "data": "synthetic (seeded soil fields)",
        "config": workload_config(args, w.name, w.cells),
        "arm": {"precision": args.precision, "pc": args.pc, "solver": solver,
                "staged_assembly": bool(args.staged_assembly),
                "parallelism": f"replicas x{world}",
                "picard_arith": ("native fp64" if args.scheme != "picard" or w.params.picard_fp64
                                 else "float-float (two fp32, ~48-bit significand) for the "
                                      "constitutive relations, face fluxes and final update; "
                                      "Picard residual's storage difference and combination, "
                                      "refinement residual and mass sums fp64"),
                "picard_iterations": cnt["picard_iterations"],
                "cg_iterations": cnt["ksp_iterations"], "ir_sweeps": cnt["ir_sweeps"],
                "mass_error_rel": cnt["mass_error_rel"]},
        "comparison": comparison,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(q_host.numel() * 8),
                "d2h_bytes_per_step": int(h_host.numel() * 8 + wc_host.numel() * 8)},
        "roofline": dict(roofline, step=step_roofline(args, w, cnt, ms_max)),
        "roofline_network": net_roof,
        "learned": learned_rec,
        "cpu_baseline": cpu,
        "gpu_launches": int(cnt["kernel_launches"]),
        "clocks": clk,
    }
    if learned:
        line["arm"]["learned"] = dict(net_info, net_solves=cnt["net_solves"],
                                         net_skipped=cnt["net_skipped"],
                                         fcg_fallbacks=cnt["fcg_fallbacks"],
                                         net_solve_ms=round(cnt["net_ms"], 2),
                                         plain_solve_ms=round(cnt["plain_ms"], 2),
                                         policy="probe every 32 solves, keep if <= 1.0x plain time")
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
