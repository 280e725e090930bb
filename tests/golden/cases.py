"""Cases of the golden fixtures: inputs (built by frehg_gb300.workloads), steps and the steps
whose head and water content the fixture keeps.  Shared by gen_golden.py (which runs the
reference's own code) and tests/test_golden_gpu.py (which runs the GPU step)."""
from __future__ import annotations

import dataclasses
import hashlib
from typing import Callable

import numpy as np

from frehg_gb300 import workloads as W


@dataclasses.dataclass
class Case:
    build: Callable
    steps: int
    saved: tuple
    uniform_col: float | None = None


def _layered():
    w = W.config0("pca", nx=10, ny=9, nz=30, steps=20)
    classes, cls, Ks = W.layered_soil(w.nx, w.ny, w.nz, 5, 11)
    w.classes, w.class_index, w.Ks = classes, cls.ravel(), Ks
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.5)
    w.params.htop = 0.05
    return w


def _saturating():
    w = W.config0("pca", nx=6, ny=5, nz=20, steps=30)
    w.params.use_full3d = 0
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.05)
    w.h0[:3] = 0.02
    w.params.htop = 0.1
    return w


def _recharge():
    w = W.config1("pca", nx=12, ny=10, nz=16, steps=8)
    q = np.zeros((w.ny, w.nx))
    q[2:7, 3:9] = -4e-6
    w.top_flux = q
    return w


def _adaptive_grf():
    w = W.config1("pca", nx=10, ny=8, nz=20, steps=25)
    w.params.adaptive_dt = 1
    w.params.dt, w.params.dt_min, w.params.dt_max = 5.0, 0.5, 120.0
    return w


def _qbot_box():
    w = W.small_box()
    w.params.bc_type[4] = 2
    w.params.qbot = 1e-7
    return w


CASES = {
    "box_closed_4x4x8": Case(W.small_box, 40, (10, 20, 40)),
    "box_qbot_4x4x8": Case(_qbot_box, 40, (40,)),
    "b2gw_sor_column": Case(lambda: W.b2gw_column(pc="sor", rtol=1e-10), 400,
                            (1, 100, 200, 400), uniform_col=0.033),
    "b2gw_jacobi_column": Case(lambda: W.b2gw_column(pc="jacobi", rtol=1e-10), 400,
                               (1, 100, 200, 400), uniform_col=0.033),
    "c0_pca_12x10x40": Case(lambda: W.config0("pca", nx=12, ny=10, nz=40), 25, (1, 5, 25)),
    "c0_pca_40x40x100": Case(lambda: W.config0("pca"), 120, (1, 30, 120)),
    "c1_pca_20x16x24": Case(lambda: W.config1("pca", nx=20, ny=16, nz=24), 12, (1, 12)),
    "layered_10x9x30": Case(_layered, 20, (1, 20)),
    "saturating_vertical_6x5x20": Case(_saturating, 30, (1, 10, 30)),
    "recharge_12x10x16": Case(_recharge, 8, (8,)),
    "adaptive_grf_10x8x20": Case(_adaptive_grf, 25, (25,)),
}


def input_digest(w, case) -> str:
    """SHA-256 over the inputs that define a case apart from the per-cell Ks / alpha fields
    (parameters, class map, initial state, forcing).  Those fields come from FFTs and exp,
    whose last bits may differ between machines, so the fixture stores them and the tests use
    the stored values."""
    h = hashlib.sha256()
    # picard_fp64 only chooses the GPU's Picard kernels, not the step's inputs: hashed as 0,
    # the value the fixtures were written with
    p = type(w.params).from_buffer_copy(bytes(w.params))
    p.picard_fp64 = 0
    h.update(bytes(p))
    h.update(bytes(w.solver))
    for a in (w.h0, w.wc0, w.class_index, w.top_flux):
        if a is not None:
            h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    if w.classes is not None:
        for c in w.classes:
            h.update(bytes(c))
    h.update(repr((w.nx, w.ny, w.nz, case.steps, case.uniform_col)).encode())
    return h.hexdigest()
