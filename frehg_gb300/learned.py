"""Learned preconditioner (not in reference): data generation, training and use.

The network, its forward/backward/Adam kernels and the flexible-CG solver run in the CUDA
library (csrc/unet.cu, csrc/mixed.cu); this module only drives them.  Device buffers for the
training set are torch tensors (plumbing).

Training data are (residual, error) pairs the plain solver produces: for seeded three-layer
soils (sand / loam / clay, in-layer ln Ks GRF sigma 1.5) at 128x128x64, the PCA head system of
several time levels is solved with FP64 Jacobi-PCG, then the iteration is re-run and at chosen
iteration numbers k the scaled residual r~_k and error x~* - x~_k are stored together with
ln K and the moisture capacity C of the state.
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

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, stream=None):
        check(self._lib.frehg_unet_adam_step(self._h, lr, b1, b2, eps, stream), "unet_adam")

    @staticmethod
    def flops(nx, ny, nz):
        f = C.c_double()
        check(load_library().frehg_unet_flops(nx, ny, nz, C.byref(f)), "unet_flops")
        return f.value


def layered_workload(nx, ny, nz, seed, dt=60.0):
    """three-layer heterogeneous soil (the learned-preconditioner configuration's generator)"""
    from . import workloads as W
    w = W.config1("pca", nx=nx, ny=ny, nz=nz, steps=1)
    classes, cls, Ks = W.layered_soil(nx, ny, nz, seed_layers=1000 + seed, seed_k=2000 + seed)
    w.classes, w.class_index, w.Ks, w.alpha = classes, cls.ravel(), Ks, None
    w.params.dt = dt
    # water table at the same relative depth as the 6.4 m deep benchmark column (4 m)
    depth = nz * w.params.dz
    table = 0.625 * depth
    w.h0 = np.broadcast_to(W.hydrostatic_head(nz, w.params.dz, table)[:, None, None],
                           (nz, ny, nx)).copy()
    w.params.hbot = depth - table
    w.name = f"layered-{nx}x{ny}x{nz}-seed{seed}"
    return w


def generate_pairs(seeds, nx=128, ny=128, nz=64, snapshots=(0, 3, 6, 9), iters=PAIR_ITERS,
                   device="cuda"):
    """(residual, error) pairs from plain solves; returns a dict of torch tensors on the GPU."""
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
            check(lib.frehg_re_training_pairs(g._h, len(iters), it_arr, R[q].data_ptr(),
                                              E[q].data_ptr(), LNK[s].data_ptr(),
                                              CAP[s].data_ptr()), "training_pairs")
            snap_of += [s] * len(iters)
            q += len(iters)
            s += 1
        del g
    torch.cuda.synchronize()
    return dict(r=R, e=E, lnk=LNK, cap=CAP, snap=np.array(snap_of), shape=(nx, ny, nz))


def input_scaling(data):
    lnk = data["lnk"]
    cap = data["cap"]
    kmean = float(lnk.mean())
    kstd = float(lnk.std())
    cstd = float(cap.std())
    return kmean, (1.0 / kstd if kstd > 0 else 1.0), (1.0 / cstd if cstd > 0 else 1.0)


def correction_targets(data):
    """The preconditioner is z = r~ + NN(r~) (Jacobi step on the unit-diagonal operator plus a
    learned correction), so the network is trained on e~ - r~."""
    data["t"] = data["e"] - data["r"]
    return data


def train(net: UNet, data, steps=5000, lr=1e-3, seed=0, log_every=0):
    """Adam on randomly drawn pairs (target e~ - r~); returns the loss history"""
    if "t" not in data:
        correction_targets(data)
    nx, ny, nz = data["shape"]
    net.set_scaling(*input_scaling(data))
    rng = np.random.default_rng(seed)
    npair = data["r"].shape[0]
    losses = []
    t0 = time.time()
    for it in range(steps):
        q = int(rng.integers(npair))
        s = int(data["snap"][q])
        loss = net.loss_grad(nx, ny, nz, data["r"][q].data_ptr(), data["lnk"][s].data_ptr(),
                             data["cap"][s].data_ptr(), data["t"][q].data_ptr())
        net.adam(lr)
        losses.append(loss)
        if log_every and (it + 1) % log_every == 0:
            print(f"  step {it + 1}: loss {np.mean(losses[-log_every:]):.4e} "
                  f"({time.time() - t0:.1f} s)", flush=True)
    return losses
