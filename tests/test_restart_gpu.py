"""Checkpoint / restart of the GPU step state (the groundwater part of the reference's
writeCheckpointNow / loadCheckpointState with primeAdaptiveDt): a new handle restarted from a
checkpoint continues exactly like the run that wrote it (heads, water contents, dt sequence and
time bit for bit) — the reference's restart-equals-continuous gate."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def new(w):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    return g


def continuous_vs_restart(w, before, after, column=False):
    a = new(w)
    if column:
        a.initialize_uniform_column(0.033)
    for _ in range(before):
        a.advance_step()
    cp = a.checkpoint()
    b = new(w)
    if column:
        b.initialize_uniform_column(0.5)  # a different start, overwritten by the restart
    b.restart(cp)
    for s in range(after):
        a.advance_step()
        b.advance_step()
        assert np.array_equal(a.interior("h"), b.interior("h")), f"step {s}"
        assert np.array_equal(a.interior("wc"), b.interior("wc")), f"step {s}"
        assert a.dt() == b.dt() and a.time() == b.time()
    assert a.boundary_volumes() == b.boundary_volumes()


def test_restart_pca_adaptive_column(gpu_lib):
    """b2-gw column, adaptive dt: 40 steps, checkpoint, 30 more"""
    continuous_vs_restart(W.b2gw_column(pc="jacobi", rtol=1e-10), 40, 30, column=True)


def test_restart_pca_3d(gpu_lib):
    """heterogeneous 3D box with top flux and bottom Dirichlet (ghost rules after step 1)"""
    continuous_vs_restart(W.config1("pca", nx=16, ny=12, nz=24, steps=6), 3, 3)


def test_restart_picard_rain_mixed(gpu_lib):
    """combined workload's physics on a window, mixed precision with the line solve: dt from
    the Picard count, rain stopping after the checkpoint"""
    w = W.config4(nx=16, ny=12, nz=96, steps=20, precision=1, pc="line")
    w.params.rain_until = 200.0
    continuous_vs_restart(w, 10, 10)


def test_restart_mixed_tiny_first_residual(gpu_lib):
    """A near-equilibrium Picard run whose first refinement residual is below 2^-30: the first
    solves' right-hand-side scale comes from the previous solve, which the checkpoint carries,
    so the restarted handle takes the same scaling path as the continuous run."""
    w = W.config1("picard", nx=16, ny=12, nz=24, steps=6, precision=1)
    w.solver.pc_type = b"line"
    w.params.qtop = -1e-12
    continuous_vs_restart(w, 3, 3)


def test_checkpoint_refused_after_surface_exchange(gpu_lib):
    from frehg_gb300.abi import FREHG_ERR_STATE, FrehgError
    w = W.config1("pca", nx=8, ny=6, nz=10, steps=2)
    g = new(w)
    g.advance_step()
    g.surface_exchange(np.full(w.nx * w.ny, 0.01), np.zeros(w.nx * w.ny), 1.0)
    with pytest.raises(FrehgError) as e:
        g.checkpoint()
    assert e.value.code == FREHG_ERR_STATE
    g.advance_step()
    g.checkpoint()  # between steps again


@pytest.mark.parametrize("scheme", ["pca", "picard"])
def test_restart_from_reference_layout_record(gpu_lib, scheme):
    """A checkpoint record in the reference's layout (gw_<name> halo arrays, dt, time, the
    "internal-with-halo" tag) written by one handle and read by a new one: the FP64 path's next
    steps equal the continuous run's bit for bit."""
    w = W.config1(scheme, nx=16, ny=12, nz=24, steps=6)
    a = new(w)
    for _ in range(3):
        a.advance_step()
    rec = a.checkpoint_record()
    assert rec["storage_layout"] == "internal-with-halo"
    assert rec["gw_h"].size == 18 * 14 * 26 and np.array_equal(rec["h"], rec["gw_h"])
    b = new(w)
    b.restart_from_record(rec)
    for s in range(3):
        a.advance_step()
        b.advance_step()
        assert np.array_equal(a.interior("h"), b.interior("h")), f"step {s}"
        assert np.array_equal(a.interior("wc"), b.interior("wc")), f"step {s}"
        assert a.dt() == b.dt() and a.time() == b.time()


def test_restart_from_oracle_record(gpu_lib, oracle_mod):
    """The oracle (the reference's step restated with the reference's halo storage) writes the
    record after three steps; a GPU handle restarted from it follows the oracle's next steps
    within 1e-8 m."""
    w = W.config1("pca", nx=16, ny=12, nz=24, steps=6)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    for _ in range(3):
        o.advance_step()
    rec = {"gw_h": o.field("h").ravel(), "gw_wc": o.field("wc").ravel(), "dt": o.dt(),
           "time": o.time()}
    g = new(w)
    g.restart_from_record(rec)
    for s in range(3):
        o.advance_step()
        g.advance_step()
        assert np.abs(g.interior("h") - o.interior("h")).max() <= 1e-8, f"step {s}"
        assert abs(g.dt() - o.dt()) <= 1e-12 * o.dt()


def test_record_missing_or_mismatched_fields(gpu_lib):
    w = W.config1("pca", nx=8, ny=6, nz=10, steps=1)
    g = new(w)
    g.advance_step()
    rec = g.checkpoint_record()
    with pytest.raises(RuntimeError, match="missing field 'gw_wc'"):
        g.restart_from_record({k: v for k, v in rec.items() if k != "gw_wc"})
    bad = dict(rec, gw_h=rec["gw_h"][:-1])
    with pytest.raises(RuntimeError, match="size mismatch"):
        g.restart_from_record(bad)


def test_constitutive_values_follow_a_soil_change(gpu_lib):
    """A converged float-float Picard step hands its last update's constitutive values to the
    next step; a change of the soil in between must discard them.  The step after the change
    equals, bit for bit, that of a handle built with the new soil and restarted from the same
    state."""
    import dataclasses
    w = W.config1("picard", nx=16, ny=12, nz=24, steps=3, precision=1)
    w.solver.pc_type = b"line"
    a = new(w)
    a.advance_step()
    a.advance_step()
    cp = a.checkpoint()
    alpha2 = w.alpha * 1.3
    a.set_cell_fields(w.Ks, alpha2)
    a.advance_step()
    b = new(dataclasses.replace(w, alpha=alpha2))
    b.restart(cp)
    b.advance_step()
    assert np.array_equal(a.interior("h"), b.interior("h"))
    assert np.array_equal(a.interior("wc"), b.interior("wc"))
