"""Learned preconditioner (not in reference): data generation, training and use.

The network, its forward/backward/Adam kernels and the flexible-CG solver run in the CUDA
library (csrc/unet.cu, csrc/mixed.cu); this module only drives them.  Device buffers for the
training set are torch tensors (plumbing).

Training data are (residual, error) pairs the plain solver produces: for seeded three-layer
soils (sand / loam / clay, in-layer ln Ks GRF sigma 1.5) at 128x128x64, the PCA head system of
several time levels is solved with FP64 Jacobi-PCG, then the iteration is re-run and at chosen
iteration numbers k the scaled residual r~_k and a target are stored together with ln K and the
moisture capacity C of the state.  The preconditioner is z = M r~ + NN(r~), so the target is the
part of the error x~* - x~_k that M r~ misses: e~ - r~ for M = I ("unet", the unit-diagonal
Jacobi step) or e~ - M_line^-1 r~ ("unet-line", the vertical-line solve).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from .abi import SolverConfig, check, load_library

PAIR_ITERS = (0, 2, 5, 10, 20, 40, 80, 160)


class UNet:
    """Handle on the library's U-Net (FP32 master weights on the device)."""

    def __init__(self, seed: int = 0):
        self._lib = load_library()
        h = C.c_void_p()
        check(self._lib.frehg_unet_create(int(seed), C.byref(h)), "unet_create")
        self._h = h
        n = C.c_int64()
        check(self._lib.frehg_unet_num_params(h, C.byref(n)), "unet_num_params")
        self.nparam = n.value
        self.scaling = (0.0, 1.0, 1.0)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.frehg_unet_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        p = np.empty(self.nparam, dtype=np.float32)
        check(self._lib.frehg_unet_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))),
              "unet_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self._lib.frehg_unet_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))),
              "unet_set_params")

    def set_scaling(self, kmean, kscale, cscale):
        self.scaling = (float(kmean), float(kscale), float(cscale))
        check(self._lib.frehg_unet_set_input_scaling(self._h, *self.scaling), "unet_scaling")

    def save(self, path):
        np.savez(path, params=self.params(), scaling=np.array(self.scaling))

    def load(self, path):
        d = np.load(path)
        self.set_params(d["params"])
        self.set_scaling(*[float(v) for v in d["scaling"]])

    def loss_grad(self, nx, ny, nz, r, lnk, cap, target, stream=None):
        loss = C.c_double()
        check(self._lib.frehg_unet_loss_grad(self._h, nx, ny, nz, r, lnk, cap, target,
                                             C.byref(loss), None, stream), "unet_loss_grad")
        return loss.value

    def set_loss_weight(self, w):
        check(self._lib.frehg_unet_set_loss_weight(self._h, float(w)), "unet_loss_weight")

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, stream=None):
        check(self._lib.frehg_unet_adam_step(self._h, lr, b1, b2, eps, stream), "unet_adam")

    @staticmethod
    def flops(nx, ny, nz):
        f = C.c_double()
        check(load_library().frehg_unet_flops(nx, ny, nz, C.byref(f)), "unet_flops")
        return f.value


TARGETS = {"unet": 1, "unet-line": 2}


def layered_workload(nx, ny, nz, seed, dt=60.0):
    """three-layer heterogeneous soil (the learned-preconditioner configuration's generator;
    training seeds are 100 + i, the benchmark's own soil uses seed 5)"""
    from . import workloads as W
    w = W.config3("pca", nx=nx, ny=ny, nz=nz, steps=1, seed=seed, precision=0)
    w.params.dt = dt
    return w


def generate_pairs(seeds, nx=128, ny=128, nz=64, snapshots=(0, 3, 6, 9), iters=PAIR_ITERS,
                   pc="unet-line", device="cuda"):
    """(residual, target) pairs from plain solves; returns a dict of torch tensors on the GPU
    (r, t = target, lnk, cap, snap = the snapshot index of each pair)."""
    import torch
    from .re_solver import Grid, ReSolver
    lib = load_library()
    n = nx * ny * nz
    npair = len(seeds) * len(snapshots) * len(iters)
    R = torch.empty((npair, n), dtype=torch.float32, device=device)
    E = torch.empty((npair, n), dtype=torch.float32, device=device)
    LNK = torch.empty((len(seeds) * len(snapshots), n), dtype=torch.float32, device=device)
    CAP = torch.empty_like(LNK)
    snap_of = []
    it_arr = (C.c_int * len(iters))(*iters)
    q = s = 0
    for seed in seeds:
        w = layered_workload(nx, ny, nz, seed)
        w.solver = SolverConfig("cg", "jacobi", rtol=1e-12, max_it=20000)
        g = ReSolver(Grid(nx, ny, nz, 1.0, 1.0, 0.05), w.params)
        w.apply(g)
        done = 0
        for snap in snapshots:
            while done < snap:
                g.advance_step()
                done += 1
            check(lib.frehg_re_training_pairs(g._h, len(iters), it_arr, TARGETS[pc],
                                              R[q].data_ptr(), E[q].data_ptr(),
                                              LNK[s].data_ptr(), CAP[s].data_ptr()),
                  "training_pairs")
            snap_of += [s] * len(iters)
            q += len(iters)
            s += 1
        del g
    torch.cuda.synchronize()
    return dict(r=R, t=E, lnk=LNK, cap=CAP, snap=np.array(snap_of), shape=(nx, ny, nz), pc=pc)


def input_scaling(data):
    lnk = data["lnk"]
    cap = data["cap"]
    kmean = float(lnk.mean())
    kstd = float(lnk.std())
    cstd = float(cap.std())
    return kmean, (1.0 / kstd if kstd > 0 else 1.0), (1.0 / cstd if cstd > 0 else 1.0)


def pair_weights(data):
    """1 / mean((t / rms r)^2) per pair: the loss of every pair becomes its relative error, so
    pairs whose error is large next to their residual (late iterations, smooth residuals) do not
    drown the others"""
    if "w" not in data:
        r2 = (data["r"].double() ** 2).mean(dim=1)
        t2 = (data["t"].double() ** 2).mean(dim=1)
        data["w"] = (r2 / t2.clamp_min(1e-300)).cpu().numpy()
    return data["w"]


def pair_loss(net: UNet, data, q):
    """relative loss of pair q (no parameter update)"""
    nx, ny, nz = data["shape"]
    s = int(data["snap"][q])
    net.set_loss_weight(pair_weights(data)[q])
    return net.loss_grad(nx, ny, nz, data["r"][q].data_ptr(), data["lnk"][s].data_ptr(),
                         data["cap"][s].data_ptr(), data["t"][q].data_ptr())


def train(net: UNet, data, steps=5000, lr=1e-3, seed=0, log_every=0):
    """Adam on randomly drawn pairs with the relative per-pair loss; returns the loss history"""
    nx, ny, nz = data["shape"]
    net.set_scaling(*input_scaling(data))
    wts = pair_weights(data)
    rng = np.random.default_rng(seed)
    npair = data["r"].shape[0]
    losses = []
    t0 = time.time()
    for it in range(steps):
        q = int(rng.integers(npair))
        s = int(data["snap"][q])
        net.set_loss_weight(wts[q])
        loss = net.loss_grad(nx, ny, nz, data["r"][q].data_ptr(), data["lnk"][s].data_ptr(),
                             data["cap"][s].data_ptr(), data["t"][q].data_ptr())
        net.adam(lr)
        losses.append(loss)
        if log_every and (it + 1) % log_every == 0:
            print(f"  step {it + 1}: loss {np.mean(losses[-log_every:]):.4e} "
                  f"({time.time() - t0:.1f} s)", flush=True)
    return losses


DEFAULT_WEIGHTS = __import__("os").path.join(__import__("os").path.dirname(__file__), "data",
                                             "unet_line_c3.npz")


def time_application(nx, ny, nz, repeat=3, warmup=2, weights=DEFAULT_WEIGHTS, seed=0):
    """Time one forward application of the network on seeded inputs of nx x ny x nz cells
    (residual and ln K standard normal, C uniform in [0, 1)) with CUDA events on the stream of
    the launches; returns (ms per application, TFLOP/s)."""
    import os
    import torch
    lib = load_library()
    net = UNet(0)
    if weights and os.path.exists(weights):
        net.load(weights)
    n = nx * ny * nz
    g = torch.Generator(device="cuda").manual_seed(seed)
    r = torch.randn(n, device="cuda", generator=g)
    lnk = torch.randn(n, device="cuda", generator=g)
    cap = torch.rand(n, device="cuda", generator=g)
    y = torch.empty(n, device="cuda")
    st = torch.cuda.Stream()

    def app():
        check(lib.frehg_unet_forward(net.handle, nx, ny, nz, r.data_ptr(), lnk.data_ptr(),
                                     cap.data_ptr(), y.data_ptr(), st.cuda_stream), "forward")

    for _ in range(warmup):
        app()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(repeat):
        app()
    e1.record(st)
    st.synchronize()
    ms = e0.elapsed_time(e1) / repeat
    return ms, UNet.flops(nx, ny, nz) / (ms * 1e-3) / 1e12


def main(argv=None):
    """Train the preconditioner network with the layered-soil recipe and save it:
    pairs from plain solves of `--seeds` three-layer soils (seeds 100, 101, ...) at the given
    shape, snapshots after 0/3/6/9 steps, iterations PAIR_ITERS (32 pairs per soil; 64 soils give
    2,048 pairs), Adam at `--lr` for `--steps` steps; the held-out relative loss (soil 99) is
    printed before and after training."""
    import argparse
    import json
    import os
    ap = argparse.ArgumentParser(prog="python -m frehg_gb300.learned")
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--pc", default="unet-line", choices=sorted(TARGETS))
    ap.add_argument("--seeds", type=int, default=64)
    ap.add_argument("--shape", type=int, nargs=3, default=(128, 128, 64))
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--apply", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="instead of training: time the saved network's forward application")
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args(argv)
    from .build import build
    build()
    if a.apply:
        ms, tf = time_application(*a.apply, repeat=a.repeat, weights=a.out)
        print(json.dumps({"cells": list(a.apply), "ms_per_application": round(ms, 3),
                          "tflops": round(tf, 1)}))
        return 0
    t0 = time.time()
    data = generate_pairs(list(range(100, 100 + a.seeds)), *a.shape, pc=a.pc)
    held = generate_pairs([99], *a.shape, snapshots=(3,), pc=a.pc)
    t1 = time.time()
    net = UNet(0)
    net.set_scaling(*input_scaling(data))

    def held_loss():
        return float(np.mean([pair_loss(net, held, q) for q in range(held["r"].shape[0])]))

    before = held_loss()
    losses = train(net, data, steps=a.steps, lr=a.lr, log_every=max(1, a.steps // 10))
    after = held_loss()
    t2 = time.time()
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    info = {"pc": a.pc, "pairs": int(data["r"].shape[0]), "seeds": a.seeds,
            "shape": list(a.shape), "adam_steps": a.steps, "lr": a.lr,
            "held_out_loss_before": before, "held_out_loss_after": after,
            "train_loss_first_10pct": float(np.mean(losses[:max(1, len(losses) // 10)])),
            "train_loss_last_10pct": float(np.mean(losses[-max(1, len(losses) // 10):])),
            "pairs_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1)}
    np.savez(a.out, params=net.params(), scaling=np.array(net.scaling), info=json.dumps(info))
    print(json.dumps(info))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
