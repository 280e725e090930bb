"""Pins of the CPU oracle against the reference's own known-answer and invariant tests.

The reference ships no golden vectors for this path; these are its tests re-run against the
restatement: tests/re/test_re_constitutive.cpp, tests/re/test_re_3d.cpp,
tests/re/test_re_b2_gw.cpp, tests/linear/test_petsc_linear_solver.cpp and
tests/linear/test_assembly_backend_independent.cpp.
"""
import numpy as np
import pytest

from frehg_gb300 import workloads as W
from frehg_gb300.abi import SoilParams, SolverConfig


def vg_soil(**kw):
    s = SoilParams(alpha=1.43, n=1.56, theta_s=0.33, theta_r=0.0, Ks_z=2.89e-6, use_vg=1,
                   use_mvg=0, air_entry=-0.02)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_vg_closed_forms(oracle_mod):
    # test_re_constitutive.cpp:12-30
    s = vg_soil()
    wc = oracle_mod.vg("theta", s, -0.5)
    K = oracle_mod.vg("conductivity", s, -0.5, s.Ks_z)
    assert s.theta_r < wc < s.theta_s
    assert 0.0 < K <= s.Ks_z


@pytest.mark.parametrize("wc0", [0.05, 0.1, 0.15, 0.2, 0.25, 0.3])
def test_vg_round_trip(oracle_mod, wc0):
    # test_re_constitutive.cpp:32-46 and :64-75
    s = vg_soil()
    h = oracle_mod.vg("head", s, wc0)
    assert abs(oracle_mod.vg("theta", s, h) - wc0) < 1e-10


def test_mvg_round_trip(oracle_mod):
    # test_re_constitutive.cpp:48-62
    s = vg_soil(use_mvg=1)
    h = oracle_mod.vg("head", s, 0.15)
    assert abs(oracle_mod.vg("theta", s, h) - 0.15) < 1e-10


def _run_box(oracle_mod, w):
    r = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(r)
    t0 = r.water_volume()
    for _ in range(w.steps):
        r.advance_step()
    return r, t0, r.water_volume()


def test_closed_box_conserves(oracle_mod):
    # test_re_3d.cpp:133-150: rel < 1e-10 and bounded state
    w = W.small_box()
    r, t0, t1 = _run_box(oracle_mod, w)
    assert abs(t1 - t0) / t0 < 1e-10
    wc = r.interior("wc")
    assert wc.min() >= w.params.soil.theta_r - 1e-12 and wc.max() <= w.params.soil.theta_s + 1e-12


def test_lateral_conductivity_changes_result(oracle_mod):
    # test_re_3d.cpp:152-169
    a, a0, a1 = _run_box(oracle_mod, W.small_box())
    wb = W.small_box()
    wb.params.soil.Ks_x = 0.0
    wb.params.soil.Ks_y = 0.0
    b, b0, b1 = _run_box(oracle_mod, wb)
    assert np.abs(a.interior("wc") - b.interior("wc")).max() > 1e-7
    assert abs(a1 - a0) / a0 < 1e-10 and abs(b1 - b0) / b0 < 1e-10


def test_single_class_map_bit_identical(oracle_mod):
    # test_re_3d.cpp:171-190
    u, _, _ = _run_box(oracle_mod, W.small_box())
    w = W.small_box()
    w.classes = [w.params.soil]
    w.class_index = np.zeros(w.cells, np.int32)
    m, _, _ = _run_box(oracle_mod, w)
    assert np.array_equal(u.interior("wc"), m.interior("wc"))


def test_layered_map_changes_result(oracle_mod):
    # test_re_3d.cpp:192-218
    fast = W.small_box(Ks=5e-5)
    a, _, _ = _run_box(oracle_mod, fast)
    w = W.small_box(Ks=5e-5)
    slow = w.params.soil.copy(Ks_x=2e-6, Ks_y=2e-6, Ks_z=2e-6)
    idx = np.zeros((w.nz, w.ny, w.nx), np.int32)
    idx[w.nz // 2:] = 1
    w.classes = [w.params.soil, slow]
    w.class_index = idx.ravel()
    b, _, _ = _run_box(oracle_mod, w)
    assert np.abs(a.interior("wc") - b.interior("wc")).max() > 1e-6


def test_bottom_fixed_flux_mass(oracle_mod):
    # test_re_3d.cpp:220-274: added volume = qbot * dx * dy * dt * steps * columns, rel < 1e-6
    w = W.small_box()
    w.params.bc_type[4] = 2
    w.params.qbot = 1e-7
    r, t0, t1 = _run_box(oracle_mod, w)
    expected = 1e-7 * 2.0 * 1.0 * 5.0 * 40 * 16
    assert t1 - t0 > 0 and abs((t1 - t0) - expected) / expected < 1e-6


def test_b2gw_first_step_wets_top(oracle_mod):
    # test_re_b2_gw.cpp:109-153 (CG + SOR, rtol 1e-8)
    w = W.b2gw_column(pc="sor", rtol=1e-8)
    r = oracle_mod.OracleRe(1, 1, 100, w.params)
    r.initialize_uniform_column(0.033)
    r.attach_solver(w.solver)
    h0, wc0 = r.interior("h")[0, 0, 0], r.interior("wc")[0, 0, 0]
    r.advance_step()
    assert r.interior("h")[0, 0, 0] > h0 + 1e-6
    assert r.interior("wc")[0, 0, 0] > wc0 + 1e-8


@pytest.mark.parametrize("pc", ["sor", "jacobi"])
def test_b2gw_adaptive_snapshot_steps(oracle_mod, pc):
    """The adaptive run reaches the legacy save times 11700/23400/35100/46800 s at exactly the
    step indices the reference's legacy-replay test lists (test_re_b2_gw.cpp:196-197), ends on
    the dt_max plateau (:398) and its first 12 dts are the x1.25 ramp (:384-390)."""
    w = W.b2gw_column(pc=pc, rtol=1e-10)
    r = oracle_mod.OracleRe(1, 1, 100, w.params)
    r.initialize_uniform_column(0.033)
    r.attach_solver(w.solver)
    targets = [11700, 23400, 35100, 46800]
    idx, dts, t, n = [], [], 0.0, 0
    while t < 46800 + 1e-9:
        dts.append(r.dt())
        r.advance_step()
        t += r.dt_used()
        if len(idx) < 4 and t >= targets[len(idx)] - 1e-6:
            idx.append(n)
        n += 1
    assert idx == [5894, 11744, 17594, 23444]
    assert abs(r.dt() - 2.0) < 1e-12
    ramp = [1e-4 * 1.25 ** q for q in range(12)]
    assert max(abs(a - b) / b for a, b in zip(dts[:12], ramp)) < 1e-12


def _laplacian(nx, ny, xe):
    n = nx * ny
    coef = np.zeros((n, 7))
    b = np.zeros(n)
    for j in range(ny):
        for i in range(nx):
            r = j * nx + i
            coef[r, 0] = 4.0
            b[r] = 4.0 * xe(r)
            for slot, (di, dj) in zip((1, 2, 3, 4), ((-1, 0), (1, 0), (0, -1), (0, 1))):
                ii, jj = i + di, j + dj
                if 0 <= ii < nx and 0 <= jj < ny:
                    coef[r, slot] = -1.0
                    b[r] += -1.0 * xe(jj * nx + ii)
    return coef, b


def test_manufactured_laplacian_cg_jacobi(oracle_mod):
    # test_petsc_linear_solver.cpp:70-102: CG + Jacobi rtol 1e-13 recovers x, L2 < 1e-9
    xe = lambda g: 1.5 + np.sin(0.1 * g)
    coef, b = _laplacian(6, 5, xe)
    x, reason, its, _ = oracle_mod.ksp_solve_stencil(6, 5, 1, coef.ravel(), b, "cg", "jacobi", 1e-13)
    assert reason > 0 and its > 0
    assert np.sqrt(((x - xe(np.arange(30))) ** 2).sum()) < 1e-9


def test_backend_independent_assembly(oracle_mod):
    # test_assembly_backend_independent.cpp:49-81: L2 < 1e-8
    xe = lambda g: 0.5 + 0.001 * g
    coef, b = _laplacian(9, 7, xe)
    x, reason, _, _ = oracle_mod.ksp_solve_stencil(9, 7, 1, coef.ravel(), b, "cg", "jacobi", 1e-13)
    assert reason > 0
    assert np.sqrt(((x - xe(np.arange(63))) ** 2).sum()) < 1e-8
