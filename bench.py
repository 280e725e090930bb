#!/usr/bin/env python
"""Benchmark of the GB300 Richards-equation step: cells*steps/s.

Default workload: the 256x256x128 heterogeneous infiltration (ln Ks GRF sigma 1, correlated
ln alpha, hydrostatic start, 20 mm/h rain, bottom head fixed, dt 60 s), plain FP64 with CG +
Jacobi at rtol 1e-12, run with the reference's PCA step.  A "step" is one Richards time step
over the whole grid.  Inputs are seeded and synthetic; the working set (~1 GB) is larger than
L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference path (oracle/, OpenMP on every
host core) on a bounded window of the same workload; under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2"])
    ap.add_argument("--scheme", default="pca", choices=["pca", "picard"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--pc", default="jacobi", choices=["jacobi", "line"],
                    help="inner preconditioner of the mixed solve")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-window", type=int, default=128,
                    help="columns per side of the CPU sample window")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=2)
    ap.add_argument("--nx", type=int, default=None, help="window of the workload (smaller case)")
    ap.add_argument("--ny", type=int, default=None)
    return ap.parse_args()


def workload(args, nx=None, ny=None):
    from frehg_gb300 import workloads as W
    prec = 1 if args.precision == "mixed" else 0
    if nx is None and args.nx:
        nx, ny = args.nx, args.ny or args.nx
    if args.config == "c0":
        kw = {} if nx is None else dict(nx=nx, ny=ny)
        w = W.config0(args.scheme, **kw)
    elif args.config == "c2":
        kw = {} if nx is None else dict(nx=nx, ny=ny)
        w = W.config2(args.scheme, **kw)
    else:
        kw = {} if nx is None else dict(nx=nx, ny=ny)
        w = W.config1(args.scheme, precision=prec, **kw)
    if args.pc != "jacobi":
        if prec != 1:
            raise SystemExit("--pc line needs --precision mixed")
        w.solver.pc_type = args.pc.encode()
    return w


def window(w_full, args, side):
    """A bounded sample of the workload: the same generator on side x side columns."""
    side = min(side, w_full.nx, w_full.ny)
    return workload(args, nx=side, ny=side)


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


def ncu_traffic(kernel):
    """DRAM bytes per cell of `kernel` from the committed ncu summary (profiles/), or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return d.get(kernel)


def cpu_rate(args, w_full, seconds, max_steps=None):
    """Time the oracle (CPU restatement of the reference PCA step, OpenMP on every host core) on a
    bounded window of the workload; returns (cells*steps/s, threads, sample description)."""
    from oracle import oracle
    oracle.build()
    w = window(w_full, args, args.ref_window)
    o = oracle.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    threads = oracle.num_threads()
    t0 = time.perf_counter()
    steps = 0
    while True:
        o.advance_step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_steps and steps >= max_steps):
            break
    rate = w.cells * steps / el
    sample = (f"first {steps} PCA steps of the workload's generator on a {w.nx}x{w.ny}x{w.nz} "
              f"window ({w.cells} cells), {el:.1f} s, {threads} OpenMP threads")
    return rate, threads, sample


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    w_full = workload(args)
    from oracle import oracle
    oracle.build()
    w = window(w_full, args, args.ref_window)
    o = oracle.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    for _ in range(args.warmup):
        o.advance_step()
    w.apply(o)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.advance_step()
    el = time.perf_counter() - t0
    value = w.cells * args.steps / el
    threads = oracle.num_threads()
    sample = (f"{args.steps} PCA steps on a {w.nx}x{w.ny}x{w.nz} window of the workload "
              f"({w.cells} cells), {threads} OpenMP threads, CPU restatement of ReSolver::advanceStep")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded GRF soil fields)",
        "config": {"workload": w_full.name, "sample_window": f"{w.nx}x{w.ny}x{w.nz}",
                   "scheme": args.scheme, "precision": "fp64", "solver": "cg+jacobi rtol 1e-12"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    from frehg_gb300 import build as B
    B.build()
    from frehg_gb300.re_solver import Grid, ReSolver

    w = workload(args)
    s = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)

    def reset():
        s.set_params(w.params)
        w.apply(s)

    reset()
    for _ in range(args.warmup):
        s.advance_step()
    reset()
    c0 = s.counters()
    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id
    except Exception:
        pass
    clocks = Clocks(bus)
    clocks.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        s.advance_step()
    e1.record(stream)
    stream.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    c1 = s.counters()
    ms_max = ms
    if pg:
        t = torch.tensor([ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms_max = float(t.item())
    value = w.cells * args.steps * world / (ms_max / 1000.0)
    ksp_its = c1.ksp_iterations - c0.ksp_iterations
    launches = c1.kernel_launches - c0.kernel_launches

    # end to end through the public API: per step H2D of the top-flux forcing from pinned host
    # memory, the step, D2H of the head and water-content fields into pinned host memory
    reset()
    q_host = torch.full((w.ny * w.nx,), float(w.params.qtop), dtype=torch.float64).pin_memory()
    h_host = torch.empty((w.nz, w.ny, w.nx), dtype=torch.float64).pin_memory()
    wc_host = torch.empty((w.nz, w.ny, w.nx), dtype=torch.float64).pin_memory()
    qn, hn, wn = q_host.numpy(), h_host.numpy(), wc_host.numpy()
    barrier()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        s.set_top_flux_field(qn)
        s.advance_step()
        s.interior("h", out=hn)
        s.interior("wc", out=wn)
    e1.record(stream)
    stream.synchronize()
    barrier()
    e2e_wall = time.perf_counter() - t0
    e2e_ms = max(e0.elapsed_time(e1), 1000.0 * e2e_wall)
    if pg:
        t = torch.tensor([e2e_ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = w.cells * args.steps * world / (e2e_ms / 1000.0)

    # per-kernel durations from CUDA events on the launching stream (profiling pass)
    reset()
    s.set_profiling(1)
    for _ in range(args.profile_steps):
        s.advance_step()
    stats = s.kernel_stats() if args.profile_steps > 0 else [
        {"name": "none", "launches": 1, "total_ms": 1.0, "bytes_per_launch": 0.0}]
    s.set_profiling(0)
    tot = sum(st["total_ms"] for st in stats) or 1.0
    dom = max(stats, key=lambda st: st["total_ms"])
    per_launch_ms = dom["total_ms"] / dom["launches"]
    achieved = dom["bytes_per_launch"] / (per_launch_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    tr = ncu_traffic(dom["name"])
    roofline = {
        "bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind,
        "traffic": None if tr is None else tr * w.cells,
        "bytes_per_launch": dom["bytes_per_launch"], "ms_per_launch": per_launch_ms,
        "share_of_step": dom["total_ms"] / tot,
        "kernels": {st["name"]: {"launches": st["launches"], "ms": round(st["total_ms"], 4),
                                 "share": round(st["total_ms"] / tot, 4),
                                 "GBps": round(st["bytes_per_launch"] * st["launches"] /
                                               (st["total_ms"] / 1000.0) / 1e9, 1)
                                 if st["total_ms"] > 0 else None}
                    for st in stats},
    }
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        del s
        torch.cuda.empty_cache()
        rate, threads, sample = cpu_rate(args, w, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded GRF soil fields, hydrostatic start)",
        "config": {"workload": w.name, "cells": w.cells, "scheme": args.scheme,
                   "precision": args.precision, "solver": "cg+jacobi rtol 1e-12",
                   "parallelism": f"replicas x{world}",
                   "l2": "working set ~1 GB > 129 MB L2 (no flush needed)",
                   "cg_iterations": ksp_its, "cg_iterations_per_step": ksp_its / args.steps},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(q_host.numel() * 8),
                "d2h_bytes_per_step": int(h_host.numel() * 8 + wc_host.numel() * 8)},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
