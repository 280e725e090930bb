"""The linear-solver seam on the GPU (LinearSolver / SparseSystem / makeLinearSolver):
the reference's own linear tests, iteration-count parity with the PETSc-semantics oracle, and
failures made on the host (NaN input, max_it exhausted, malformed rows)."""
import numpy as np
import pytest

from frehg_gb300.abi import FREHG_ERR_BAD_ARG, FREHG_ERR_NONFINITE, FREHG_ERR_NOT_CONVERGED
from frehg_gb300.abi import FREHG_ERR_UNSUPPORTED, FrehgError, SolverConfig

pytestmark = pytest.mark.gpu


def assemble(sys_, coef, nx, ny, nz):
    """addRow in Decomp3D owned order from 7-slot rows (C, W, E, S, N, Up, Down)."""
    sys_.zeroEntries()
    sys_.beginAssembly()
    offs = [0, -nz, nz, -nz * nx, nz * nx, -1, 1]
    for r in range(nx * ny * nz):
        k, i, j = r % nz, (r // nz) % nx, r // (nz * nx)
        present = [True, i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1]
        cols = [r + o for o, p in zip(offs, present) if p]
        vals = [coef[r, q] for q, p in enumerate(present) if p]
        sys_.addRow(r, cols, vals)
    sys_.endAssembly()


def laplacian(nx, ny, xe):
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
                    b[r] -= xe(jj * nx + ii)
    return coef, b


def spd_stencil(nx, ny, nz, seed):
    """random symmetric diagonally dominant 7-point system in owned order"""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    coef = np.zeros((n, 7))
    up = {2: nz, 4: nz * nx, 6: 1}
    pair = {2: 1, 4: 3, 6: 5}
    for r in range(n):
        k, i, j = r % nz, (r // nz) % nx, r // (nz * nx)
        for slot, ok in ((2, i < nx - 1), (4, j < ny - 1), (6, k < nz - 1)):
            if ok:
                v = -rng.uniform(0.1, 2.0)
                coef[r, slot] = v
                coef[r + up[slot], pair[slot]] = v
    coef[:, 0] = -coef[:, 1:].sum(axis=1) + rng.uniform(1e-3, 0.5, n)
    return coef, rng.standard_normal(n)


def test_manufactured_laplacian(gpu_lib, oracle_mod):
    # tests/linear/test_petsc_linear_solver.cpp:70-102 through the GPU backend
    from frehg_gb300.linear import makeLinearSolver
    xe = lambda g: 1.5 + np.sin(0.1 * g)
    coef, b = laplacian(6, 5, xe)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-13))
    A = solver.createSystem(6, 5, 1)
    assemble(A, coef, 6, 5, 1)
    solver.setup(A)
    x = solver.solve(A, b)
    assert np.sqrt(((x - xe(np.arange(30))) ** 2).sum()) < 1e-9
    _, reason, its, rn = oracle_mod.ksp_solve_stencil(6, 5, 1, coef.ravel(), b, "cg", "jacobi", 1e-13)
    assert solver.getIterationCount() == its and solver.getConvergedReason() == reason
    assert solver.getResidualNorm() >= 0.0


def test_pattern_reuse_and_backend_independent(gpu_lib):
    # test_petsc_linear_solver.cpp:128-159 and test_assembly_backend_independent.cpp:49-81
    from frehg_gb300.linear import makeLinearSolver
    xe = lambda g: 0.5 + 0.001 * g
    coef, b = laplacian(9, 7, xe)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-13))
    A = solver.createSystem(9, 7, 1)
    assemble(A, coef, 9, 7, 1)
    x1 = solver.solve(A, b)
    assemble(A, coef, 9, 7, 1)
    x2 = solver.solve(A, b)
    assert np.abs(x1 - x2).max() <= 1e-12
    assert np.sqrt(((x2 - xe(np.arange(63))) ** 2).sum()) < 1e-8


@pytest.mark.parametrize("shape", [(7, 6, 11), (16, 12, 9), (1, 1, 50), (3, 40, 1)])
def test_random_spd_matches_oracle(gpu_lib, oracle_mod, shape):
    from frehg_gb300.linear import makeLinearSolver
    nx, ny, nz = shape
    coef, b = spd_stencil(nx, ny, nz, seed=nx * 100 + ny * 10 + nz)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-12))
    A = solver.createSystem(nx, ny, nz)
    assemble(A, coef, nx, ny, nz)
    x = solver.solve(A, b)
    xo, reason, its, _ = oracle_mod.ksp_solve_stencil(nx, ny, nz, coef.ravel(), b, "cg",
                                                      "jacobi", 1e-12)
    assert reason > 0
    assert abs(solver.getIterationCount() - its) <= 1
    assert np.abs(x - xo).max() <= 1e-9 * max(1.0, np.abs(xo).max())


def test_more_tiles_than_partial_slots(gpu_lib, oracle_mod):
    """n0 = nz = 1 and a long axis 1: 5000 tiles of 32x8 threads, more than the reduction
    partial slots, so blocks must stride over tiles."""
    from frehg_gb300.linear import makeLinearSolver
    nx, ny, nz = 40000, 1, 1
    n = nx
    coef = np.zeros((n, 7))
    coef[:, 0] = 3.0
    coef[1:, 1] = -1.0
    coef[:-1, 2] = -1.0
    b = np.random.default_rng(3).standard_normal(n)
    solver = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-12))
    A = solver.createSystem(nx, ny, nz)
    A.zeroEntries()
    rows = np.repeat(np.arange(n), 3)
    cols = np.stack([np.arange(n) - 1, np.arange(n), np.arange(n) + 1], 1).ravel()
    vals = np.stack([coef[:, 1], coef[:, 0], coef[:, 2]], 1).ravel()
    keep = (cols >= 0) & (cols < n)
    A.addCOO(rows[keep], cols[keep], vals[keep])
    A.endAssembly()
    x = solver.solve(A, b)
    xo, reason, its, _ = oracle_mod.ksp_solve_stencil(nx, ny, nz, coef.ravel(), b, "cg",
                                                      "jacobi", 1e-12)
    assert abs(solver.getIterationCount() - its) <= 1
    assert np.abs(x - xo).max() <= 1e-10


def test_failures_are_reported(gpu_lib):
    from frehg_gb300.linear import makeLinearSolver
    coef, b = spd_stencil(5, 4, 6, seed=1)
    # max_it exhausted -> KSP_DIVERGED_ITS -> FREHG_ERR_NOT_CONVERGED (the reference throws)
    s1 = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-14, max_it=1))
    A = s1.createSystem(5, 4, 6)
    assemble(A, coef, 5, 4, 6)
    with pytest.raises(FrehgError) as e:
        s1.solve(A, b)
    assert e.value.code == FREHG_ERR_NOT_CONVERGED and s1.getConvergedReason() == -3
    # NaN in the host input -> DIVERGED_NANORINF -> FREHG_ERR_NONFINITE
    s2 = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-10))
    B = s2.createSystem(5, 4, 6)
    assemble(B, coef, 5, 4, 6)
    bad = b.copy()
    bad[7] = np.nan
    with pytest.raises(FrehgError) as e:
        s2.solve(B, bad)
    assert e.value.code == FREHG_ERR_NONFINITE
    # the solver object stays usable after a failure
    x = s2.solve(B, b)
    assert np.isfinite(x).all()
    # a column outside the 7-point stencil is rejected at assembly
    with pytest.raises(FrehgError) as e:
        B.addRow(0, [0, 17], [1.0, 1.0])
    assert e.value.code == FREHG_ERR_BAD_ARG
    # a non-symmetric operator is rejected (CG needs SPD)
    C = s2.createSystem(3, 1, 1)
    C.zeroEntries()
    C.addRow(0, [0, 1], [4.0, -1.0])
    C.addRow(1, [0, 1, 2], [-2.0, 4.0, -1.0])
    C.addRow(2, [1, 2], [-1.0, 4.0])
    with pytest.raises(FrehgError) as e:
        C.endAssembly()
    assert e.value.code == FREHG_ERR_UNSUPPORTED


def test_unknown_backend_and_types(gpu_lib):
    from frehg_gb300.linear import makeLinearSolver
    with pytest.raises(RuntimeError):
        makeLinearSolver("trilinos", SolverConfig())
    with pytest.raises(FrehgError) as e:
        makeLinearSolver("gb300", SolverConfig("gmres", "jacobi"))
    assert e.value.code == FREHG_ERR_UNSUPPORTED
