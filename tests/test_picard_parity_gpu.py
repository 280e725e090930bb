"""GPU mixed-form modified Picard step vs the oracle's FP64 statement of it (not in reference).

Per step: head within 1e-8 m (max norm), equal Picard iteration counts; cumulative mass
balance closes below 1e-12 relative on the GPU.  The GPU kernels run in float-float arithmetic
(picard_fp64 = 0, set here: the library's default picks it with the mixed-precision solve only)
unless a test selects native FP64 (picard_fp64 = 1)."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def pair(w, oracle_mod):
    from frehg_gb300.re_solver import Grid, ReSolver
    if w.params.picard_fp64 < 0:
        w.params.picard_fp64 = 0
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(g)
    w.apply(o)
    return g, o


def run_compare(g, o, steps, h_tol=1e-8):
    worst = 0.0
    for s in range(steps):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        worst = max(worst, dh)
        assert dh <= h_tol, f"step {s}: head differs by {dh:.3e}"
        assert g.counters().last_picard_iterations == o.last_picard_its(), f"step {s}"
        assert abs(g.dt_used() - o.dt_used()) <= 1e-12 * o.dt_used()
    return worst


def test_config0_picard_small(gpu_lib, oracle_mod):
    w = W.config0("picard", nx=10, ny=8, nz=40, steps=12)
    g, o = pair(w, oracle_mod)
    run_compare(g, o, w.steps)


@pytest.mark.parametrize("fp64", [0, 1])
def test_config0_picard_harmonic(gpu_lib, oracle_mod, fp64):
    w = W.config0("picard", nx=8, ny=6, nz=30, steps=8)
    w.params.face_mean = 1
    w.params.picard_fp64 = fp64
    g, o = pair(w, oracle_mod)
    run_compare(g, o, w.steps)


@pytest.mark.parametrize("fp64", [0, 1])
def test_config1_picard_small(gpu_lib, oracle_mod, fp64):
    w = W.config1("picard", nx=16, ny=12, nz=24, steps=6)
    w.params.picard_fp64 = fp64
    g, o = pair(w, oracle_mod)
    worst = run_compare(g, o, w.steps)
    print(f"\n  picard_fp64={fp64}: max head difference to the oracle {worst:.2e} m")


def test_rain_pulse_and_picard_dt(gpu_lib, oracle_mod):
    """50 mm/h for the first 300 s then dry, dt adapted from the Picard count."""
    w = W.config1("picard", nx=10, ny=10, nz=20, steps=12)
    p = w.params
    p.rain_rate = -50e-3 / 3600.0
    p.rain_until = 300.0
    p.picard_dt_adapt = 1
    p.dt, p.dt_min, p.dt_max = 60.0, 10.0, 120.0
    g, o = pair(w, oracle_mod)
    run_compare(g, o, w.steps)


def test_mass_balance_closes(gpu_lib):
    """sum V theta + elastic storage - initial = cumulative boundary inflow, < 1e-12 relative"""
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config1("picard", nx=12, ny=12, nz=24, steps=10)
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    v0 = g.water_volume()
    for _ in range(w.steps):
        g.advance_step()
    v1 = g.water_volume()
    top, bot = g.boundary_volumes()
    el = g.elastic_volume()
    err = abs((v1 - v0) + el - (top + bot)) / v0
    assert err < 1e-12, err


def test_config4_window(gpu_lib, oracle_mod):
    """The combined configuration's physics on a 14x10x96 window: three soil classes with an
    in-class Ks field, dry start, rain limited by the h = 0 surface (no ponding), 1 m
    head-change limit per Picard iteration, free-drainage bottom, Picard-count dt.  The rain
    stops at 300 s here, so the 40 steps (dt >= 10 s) cover its end; the water budget closes."""
    w = W.config4(nx=14, ny=10, nz=96, steps=40, precision=0)
    w.params.rain_until = 300.0
    g, o = pair(w, oracle_mod)
    v0 = g.water_volume()
    run_compare(g, o, w.steps)
    top, bot = g.boundary_volumes()
    assert top > 0.0
    err = abs((g.water_volume() - v0) + g.elastic_volume() - (top + bot)) / v0
    assert err < 1e-12, err


def test_picard_head_change_limit(gpu_lib, oracle_mod):
    """With a 0.05 m per-iteration limit the ponded-top infiltration needs more Picard
    iterations but GPU and oracle agree iteration for iteration."""
    w = W.config0("picard", nx=6, ny=5, nz=30, steps=4)
    w.params.picard_dh_max = 0.05
    w.params.picard_max_it = 200
    g, o = pair(w, oracle_mod)
    run_compare(g, o, w.steps)
    assert g.counters().last_picard_iterations > 3
