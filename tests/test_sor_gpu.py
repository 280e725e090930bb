"""PCSOR on the GPU (pc_type "sor", the reference's groundwater default, Orchestrator.cpp:489)
against the oracle's PETSc-semantics CG + symmetric SOR (omega 1): equal iteration counts and
solutions within 1e-9 relative on the seam, and the PCA step with SOR against the oracle step by
step.  Systems up to 65,536 unknowns sweep in one block; larger ones launch a kernel per
hyperplane, so both forms are covered."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W
from frehg_gb300.abi import SolverConfig

from tests.test_linear_seam_gpu import assemble, laplacian, spd_stencil

pytestmark = pytest.mark.gpu


def test_manufactured_laplacian_sor(gpu_lib, oracle_mod):
    from frehg_gb300.linear import makeLinearSolver
    xe = lambda g: 1.5 + np.sin(0.1 * g)
    coef, b = laplacian(6, 5, xe)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "sor", rtol=1e-13))
    A = solver.createSystem(6, 5, 1)
    assemble(A, coef, 6, 5, 1)
    x = solver.solve(A, b)
    assert np.sqrt(((x - xe(np.arange(30))) ** 2).sum()) < 1e-9
    _, reason, its, _ = oracle_mod.ksp_solve_stencil(6, 5, 1, coef.ravel(), b, "cg", "sor", 1e-13)
    assert solver.getIterationCount() == its and solver.getConvergedReason() == reason


@pytest.mark.parametrize("shape", [(7, 6, 11), (16, 12, 9), (1, 1, 50), (3, 40, 1), (1, 1, 1),
                                   (48, 40, 40)])
def test_random_spd_sor_matches_oracle(gpu_lib, oracle_mod, shape):
    from frehg_gb300.linear import makeLinearSolver
    nx, ny, nz = shape
    coef, b = spd_stencil(nx, ny, nz, seed=nx * 100 + ny * 10 + nz)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "sor", rtol=1e-12))
    A = solver.createSystem(nx, ny, nz)
    assemble(A, coef, nx, ny, nz) if nx * ny * nz < 20000 else assemble_coo(A, coef, nx, ny, nz)
    x = solver.solve(A, b)
    xo, reason, its, _ = oracle_mod.ksp_solve_stencil(nx, ny, nz, coef.ravel(), b, "cg", "sor",
                                                      1e-12)
    assert reason > 0
    assert solver.getIterationCount() == its, (solver.getIterationCount(), its)
    assert np.abs(x - xo).max() <= 1e-9 * max(1.0, np.abs(xo).max())
    # a second solve on the same system (graph reused) gives the same answer
    x2 = solver.solve(A, b)
    assert np.array_equal(x, x2)


def assemble_coo(sys_, coef, nx, ny, nz):
    """the same rows through addCOO (one call)"""
    n = nx * ny * nz
    r = np.arange(n)
    k, i, j = r % nz, (r // nz) % nx, r // (nz * nx)
    offs = [0, -nz, nz, -nz * nx, nz * nx, -1, 1]
    present = [np.ones(n, bool), i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1]
    rows, cols, vals = [], [], []
    for q in range(7):
        m = present[q]
        rows.append(r[m])
        cols.append(r[m] + offs[q])
        vals.append(coef[m, q])
    sys_.zeroEntries()
    sys_.addCOO(np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))
    sys_.endAssembly()


def test_sor_rejects_mixed_precision(gpu_lib):
    from frehg_gb300.abi import FREHG_ERR_UNSUPPORTED, FrehgError
    from frehg_gb300.linear import makeLinearSolver
    with pytest.raises(FrehgError) as e:
        makeLinearSolver("gb300", SolverConfig("cg", "sor", precision=1))
    assert e.value.code == FREHG_ERR_UNSUPPORTED


def _pair(w, oracle_mod):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(g)
    w.apply(o)
    return g, o


@pytest.mark.parametrize("case", ["c1", "layered", "c0_full_plane_path"])
def test_pca_step_with_sor(gpu_lib, oracle_mod, case):
    if case == "c1":
        w = W.config1("pca", nx=16, ny=12, nz=24, steps=6)
    elif case == "layered":
        w = W.config0("pca", nx=10, ny=9, nz=30, steps=10)
        classes, cls, Ks = W.layered_soil(w.nx, w.ny, w.nz, 5, 11)
        w.classes, w.class_index, w.Ks = classes, cls.ravel(), Ks
        w.h0 = np.full((w.nz, w.ny, w.nx), -0.5)
        w.params.htop = 0.05
    else:
        w = W.config0("pca", nx=40, ny=40, nz=100, steps=3)  # 160,000 cells: one launch per plane
    w.solver.pc_type = b"sor"
    g, o = _pair(w, oracle_mod)
    for s in range(w.steps):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: head differs by {dh:.3e} m"
        assert g.counters().last_ksp_iterations == o.last_ksp_its(), f"step {s}"


def test_picard_step_with_sor(gpu_lib, oracle_mod):
    w = W.config0("picard", nx=8, ny=6, nz=30, steps=5)
    w.solver.pc_type = b"sor"
    w.params.picard_fp64 = 1
    g, o = _pair(w, oracle_mod)
    for s in range(w.steps):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: head differs by {dh:.3e} m"
        assert g.counters().last_picard_iterations == o.last_picard_its(), f"step {s}"
