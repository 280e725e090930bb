"""CPU checks of the oracle's modified Picard step (not in reference): closable mass budget,
Picard convergence, harmonic vs arithmetic face means, free drainage, rain pulse."""
import numpy as np

from frehg_gb300 import workloads as W


def run(oracle_mod, w, steps):
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    v0 = o.water_volume()
    its = []
    for _ in range(steps):
        o.advance_step()
        its.append(o.last_picard_its())
    return o, v0, its


def test_picard_mass_budget_closes(oracle_mod):
    w = W.config1("picard", nx=8, ny=8, nz=20)
    o, v0, its = run(oracle_mod, w, 6)
    top, bot = o.boundary_volumes()
    err = abs((o.water_volume() - v0) + o.elastic_volume() - (top + bot)) / v0
    assert err < 1e-12
    assert all(1 <= m <= w.params.picard_max_it for m in its)


def test_free_drainage_drains_and_ponding_wets(oracle_mod):
    w = W.config0("picard", nx=4, ny=4, nz=30)
    o, v0, _ = run(oracle_mod, w, 10)
    top, bot = o.boundary_volumes()
    assert top > 0.0          # ponded top infiltrates
    assert bot <= 0.0         # unit-gradient bottom only drains
    h = o.interior("h")
    assert h[0].mean() > -2.0  # the top layer wetted


def test_harmonic_differs_from_arithmetic(oracle_mod):
    a = W.config1("picard", nx=6, ny=6, nz=16)
    b = W.config1("picard", nx=6, ny=6, nz=16)
    b.params.face_mean = 1
    oa, _, _ = run(oracle_mod, a, 4)
    ob, _, _ = run(oracle_mod, b, 4)
    assert np.abs(oa.interior("h") - ob.interior("h")).max() > 1e-9


def test_rain_pulse_stops(oracle_mod):
    w = W.config1("picard", nx=4, ny=4, nz=12)
    w.params.rain_rate = -50e-3 / 3600.0
    w.params.rain_until = 120.0
    o, _, _ = run(oracle_mod, w, 2)       # t = 0, 60 s: raining
    t2, _ = o.boundary_volumes()
    o.advance_step()                      # t = 120 s: dry
    t3, _ = o.boundary_volumes()
    assert abs(t2 - 2 * 60.0 * 50e-3 / 3600.0 * 16) < 1e-12
    assert t3 == t2
