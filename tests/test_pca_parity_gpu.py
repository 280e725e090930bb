"""GPU PCA step vs the CPU oracle (restatement of ReSolver::advanceStep) on identical inputs.

Tolerance: pressure head within 1e-8 m (max norm) after every step; water content within
1e-9; adaptive dt sequences equal to 1e-12 relative.  Both sides solve with CG + Jacobi
(PETSc semantics) at the stated rtol, so differences come from rounding order only.
"""
import numpy as np
import pytest

from frehg_gb300 import workloads as W

pytestmark = pytest.mark.gpu

H_TOL = 1e-8
WC_TOL = 1e-9


def pair(w, oracle_mod):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(g)
    w.apply(o)
    return g, o


def step_compare(g, o, steps, h_tol=H_TOL, wc_tol=WC_TOL, check_dt=False):
    worst_h = worst_w = 0.0
    for s in range(steps):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        dw = np.abs(g.interior("wc") - o.interior("wc")).max()
        worst_h, worst_w = max(worst_h, dh), max(worst_w, dw)
        assert dh <= h_tol, f"step {s}: head differs by {dh:.3e} m"
        assert dw <= wc_tol, f"step {s}: water content differs by {dw:.3e}"
        if check_dt:
            assert abs(g.dt() - o.dt()) <= 1e-12 * o.dt(), f"step {s}: dt {g.dt()} vs {o.dt()}"
    return worst_h, worst_w


def test_closed_box(gpu_lib, oracle_mod):
    w = W.small_box()
    g, o = pair(w, oracle_mod)
    v0 = g.water_volume()
    step_compare(g, o, w.steps)
    v1 = g.water_volume()
    assert abs(v1 - v0) / v0 < 1e-10  # test_re_3d.cpp:210-227 on the GPU


def test_closed_box_vertical_only(gpu_lib, oracle_mod):
    w = W.small_box(full3d=False)
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_bottom_flux_box(gpu_lib, oracle_mod):
    w = W.small_box()
    w.params.bc_type[4] = 2
    w.params.qbot = 1e-7
    g, o = pair(w, oracle_mod)
    v0 = g.water_volume()
    step_compare(g, o, w.steps)
    expected = 1e-7 * 2.0 * 1.0 * 5.0 * 40 * 16
    assert abs((g.water_volume() - v0) - expected) / expected < 1e-6


def test_config0_pca_small(gpu_lib, oracle_mod):
    w = W.config0("pca", nx=12, ny=10, nz=40, steps=25)
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_config1_pca_small(gpu_lib, oracle_mod):
    w = W.config1("pca", nx=24, ny=20, nz=32, steps=12)
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_layered_classes_ponded(gpu_lib, oracle_mod):
    w = W.config0("pca", nx=10, ny=9, nz=30, steps=20)
    classes, cls, Ks = W.layered_soil(w.nx, w.ny, w.nz, 5, 11)
    w.classes, w.class_index, w.Ks = classes, cls.ravel(), Ks
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.5)
    w.params.htop = 0.05
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_vertical_only_saturating_box(gpu_lib, oracle_mod):
    """full_3d off with a ponded top: lateral faces open only between saturated cells, the
    reallocation sweep and the x-/y- ghost overwrite rules all fire."""
    w = W.config0("pca", nx=6, ny=5, nz=20, steps=30)
    w.params.use_full3d = 0
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.05)
    w.h0[:3] = 0.02
    w.params.htop = 0.1
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_b2gw_adaptive_dt(gpu_lib, oracle_mod):
    w = W.b2gw_column(pc="jacobi", rtol=1e-10)
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(1, 1, 100, 1, 1, 0.01), w.params)
    o = oracle_mod.OracleRe(1, 1, 100, w.params)
    for s in (g, o):
        s.initialize_uniform_column(0.033)
        s.attach_solver(w.solver)
    step_compare(g, o, 400, check_dt=True)


def test_first_step_bottom_dirichlet_quirk(gpu_lib, oracle_mod):
    """Step 1 folds the zero-initialised bottom ghost (hn) into the RHS, later steps hbot
    (ReSolver.cpp:524-525 with the ghost set by enforceHeadBc :655-657)."""
    w = W.config1("pca", nx=8, ny=8, nz=16, steps=3)
    g, o = pair(w, oracle_mod)
    step_compare(g, o, w.steps)


def test_reinitialised_handle_steps_like_a_fresh_one(gpu_lib):
    """Stepping, then setting the initial state again, reproduces a fresh handle's run (the
    first step's zero ghosts included)."""
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config1("pca", nx=16, ny=12, nz=24, steps=3)
    grid = Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz)
    fresh, reused = ReSolver(grid, w.params), ReSolver(grid, w.params)
    w.apply(fresh)
    w.apply(reused)
    for _ in range(2):
        reused.advance_step()
    reused.set_params(w.params)
    w.apply(reused)
    for _ in range(w.steps):
        fresh.advance_step()
        reused.advance_step()
        assert np.array_equal(fresh.interior("h"), reused.interior("h"))
    assert fresh.time() == reused.time()
