"""The benchmarked paths against the FP64 oracle, step by step, and the configurations at their
stated sizes.

* The combined workload's path (768x768x96 generator on a 32x32x96 window: three-layer soil,
  dry start, rain pulse, free drainage, Picard-count dt) exactly as the benchmark runs it:
  mixed precision (FP32 Krylov under FP64 refinement to 1e-12), vertical-line preconditioner,
  float-float Picard kernels; and the learned arm with the benchmark's trained network forced
  on for every solve.  Per step: head within 1e-8 m of the oracle (max norm), equal Picard
  iteration counts and time steps; on the GPU the cumulative water budget closes below 1e-12.
* 40x40x100 loam infiltration, 120 steps, with the Picard and the PCA scheme (the PCA scheme at
  this size is also checked against the reference's own outputs in test_golden_gpu.py).
* 256x256x128 heterogeneous loam: 3 PCA steps and 1 Picard step against the oracle.
* The 512x512x128 loam's and the three-layer soil's generators on windows, Picard with the
  mixed line-PCG solve.

The oracle solves with FP64 Jacobi-PCG at the same rtol (it has no mixed precision, line or
learned preconditioner: those change how the linear systems are solved, not their solutions).
"""
import os

import numpy as np
import pytest

from frehg_gb300 import workloads as W
from frehg_gb300.abi import SolverConfig

pytestmark = pytest.mark.gpu

H_TOL = 1e-8


def gpu_solver(w):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    return g


def oracle_solver(oracle_mod, w):
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    solver = w.solver
    w.solver = SolverConfig("cg", "jacobi", rtol=solver.rtol, max_it=solver.max_it)
    try:
        w.apply(o)
    finally:
        w.solver = solver
    return o


def budget_rel(g, v0):
    top, bot = g.boundary_volumes()
    v1 = g.water_volume()
    return abs((v1 - v0) - (top + bot) + g.elastic_volume()) / v0


def compare(g, o, steps, picard=True):
    worst = 0.0
    for s in range(steps):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        worst = max(worst, dh)
        assert dh <= H_TOL, f"step {s}: head differs from the oracle by {dh:.3e} m"
        if picard:
            assert g.counters().last_picard_iterations == o.last_picard_its(), f"step {s}"
        assert g.dt_used() == pytest.approx(o.dt_used(), rel=1e-12, abs=0), f"step {s}"
    return worst


def combined_window(pc):
    return W.config4(nx=32, ny=32, nz=96, steps=40, precision=1, pc=pc)


def test_combined_window_line(gpu_lib, oracle_mod):
    w = combined_window("line")
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    v0 = g.water_volume()
    worst = compare(g, o, w.steps)
    rel = budget_rel(g, v0)
    print(f"\n  combined window, mixed line-PCG, float-float: max head difference {worst:.2e} m, "
          f"budget {rel:.1e}")
    assert rel < 1e-12


def test_combined_window_learned_forced_on(gpu_lib, oracle_mod):
    from frehg_gb300 import learned as Lr
    from frehg_gb300.abi import check
    if not os.path.exists(Lr.DEFAULT_WEIGHTS):
        pytest.skip("no trained network in the package data")
    net = Lr.UNet(0)
    net.load(Lr.DEFAULT_WEIGHTS)
    w = combined_window("unet-line")
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    check(g._lib.frehg_re_attach_unet(g._h, net.handle), "attach_unet")
    check(g._lib.frehg_re_set_learned_policy(g._h, 0, 1e9), "policy")  # every solve
    v0 = g.water_volume()
    worst = compare(g, o, w.steps)
    c = g.counters()
    rel = budget_rel(g, v0)
    print(f"\n  combined window, learned FCG forced on: {c.net_solves} network solves, "
          f"{c.fcg_fallbacks} fallbacks, max head difference {worst:.2e} m, budget {rel:.1e}")
    assert c.net_solves > 0 and c.net_skipped == 0
    assert rel < 1e-12


def test_config0_picard_full_size(gpu_lib, oracle_mod):
    w = W.config0("picard")  # 40x40x100, 120 steps of 30 s
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    v0 = g.water_volume()
    worst = compare(g, o, w.steps)
    print(f"\n  40x40x100 Picard, 120 steps: max head difference {worst:.2e} m")
    assert budget_rel(g, v0) < 1e-12


def test_config0_pca_full_size(gpu_lib, oracle_mod):
    w = W.config0("pca")  # 40x40x100, 120 steps of 30 s, the reference's scheme
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    worst = compare(g, o, w.steps, picard=False)
    print(f"\n  40x40x100 PCA, 120 steps: max head difference {worst:.2e} m")


def test_config1_full_size_pca(gpu_lib, oracle_mod):
    w = W.config1("pca", steps=3)  # 256x256x128
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    worst = compare(g, o, w.steps, picard=False)
    print(f"\n  256x256x128 PCA, 3 steps: max head difference {worst:.2e} m")


def test_config1_full_size_picard_mixed_line(gpu_lib, oracle_mod):
    w = W.config1("picard", steps=1, precision=1)
    w.solver.pc_type = b"line"
    w.solver.ir_rtol = 1e-12
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    worst = compare(g, o, w.steps)
    print(f"\n  256x256x128 Picard (mixed line, float-float), 1 step: max head difference "
          f"{worst:.2e} m")


def test_config2_window_picard_mixed_line(gpu_lib, oracle_mod):
    """512x512x128 loam's generator (its own seeds) on a 48x48x128 window, the benchmark's
    mixed line-PCG Picard path, 8 steps"""
    w = W.config2("picard", nx=48, ny=48, steps=8)
    w.solver.pc_type = b"line"
    w.solver.ir_rtol = 1e-12
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    v0 = g.water_volume()
    worst = compare(g, o, w.steps)
    print(f"\n  512x512x128 generator, 48x48 window, 8 Picard steps: max head difference "
          f"{worst:.2e} m")
    assert budget_rel(g, v0) < 1e-12


def test_config3_window_picard_mixed_line(gpu_lib, oracle_mod):
    """the three-layer soil (learned-preconditioner configuration's generator) on a 24x24x128
    window, Picard with the mixed line-PCG solve, 6 steps: the first step's attempts at 60, 30,
    15 and 7.5 s fail to converge and the step is taken at 3.75 s, on both"""
    w = W.config3("picard", nx=24, ny=24, steps=6, precision=1, pc="line")
    g, o = gpu_solver(w), oracle_solver(oracle_mod, w)
    v0 = g.water_volume()
    worst = compare(g, o, w.steps)
    print(f"\n  three-layer soil, 24x24x128 window, 6 Picard steps: max head difference "
          f"{worst:.2e} m")
    assert budget_rel(g, v0) < 1e-12
