"""The FP64 Jacobi-PCG iteration as one cooperative launch (k_cg_iter: direction, grid barrier,
stencil product with p.w, grid barrier, update with the norms) against the three-kernel form
and the PETSc-semantics oracle: iteration counts within one (the two forms sum the dot
products over different block partitions) and the same solution to 1e-10 relative, on ragged
boxes, single columns and rows, a box whose tiles outnumber the resident blocks, and the RE
step's own solves.  Not in reference: the reference's KSP solve is PetscLinearSolver.cpp:200-220.
"""
import numpy as np
import pytest

from frehg_gb300.abi import SolverConfig

pytestmark = pytest.mark.gpu


def spd_coo(nx, ny, nz, seed):
    """random symmetric diagonally dominant 7-point system in Decomp3D owned order
    (row = k + nz (i + nx j)) as COO triplets, its 7-slot rows (C, W, E, S, N, Up, Down) for
    the oracle, and a right-hand side"""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    r = np.arange(n)
    k, i, j = r % nz, (r // nz) % nx, r // (nz * nx)
    coef = np.zeros((n, 7))
    for slot, pair, step, ok in ((2, 1, nz, i < nx - 1), (4, 3, nz * nx, j < ny - 1),
                                 (6, 5, 1, k < nz - 1)):
        v = -rng.uniform(0.1, 2.0, n)
        coef[ok, slot] = v[ok]
        coef[r[ok] + step, pair] = v[ok]
    coef[:, 0] = -coef[:, 1:].sum(axis=1) + rng.uniform(1e-3, 0.5, n)
    offs = [0, -nz, nz, -nz * nx, nz * nx, -1, 1]
    rows, cols, vals = [], [], []
    for q, o in enumerate(offs):
        m = coef[:, q] != 0.0
        rows.append(r[m])
        cols.append(r[m] + o)
        vals.append(coef[m, q])
    return (np.concatenate(rows), np.concatenate(cols), np.concatenate(vals), coef,
            rng.standard_normal(n))


def solve(nx, ny, nz, rows, cols, vals, b, fused, rtol=1e-12):
    from frehg_gb300.linear import makeLinearSolver
    s = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=rtol, max_it=20000))
    s.setFusedIteration(fused)
    A = s.createSystem(nx, ny, nz)
    A.zeroEntries()
    A.addCOO(rows, cols, vals)
    A.endAssembly()
    x = s.solve(A, b)
    return x, s.getIterationCount(), s.getConvergedReason()


@pytest.mark.parametrize("shape", [(7, 6, 11), (16, 12, 9), (1, 1, 50), (3, 40, 1),
                                   (33, 17, 5), (20000, 1, 1)])
def test_fused_matches_three_kernels_and_oracle(gpu_lib, oracle_mod, shape):
    nx, ny, nz = shape
    rows, cols, vals, coef, b = spd_coo(nx, ny, nz, seed=nx + 7 * ny + 13 * nz)
    xf, itf, rf = solve(nx, ny, nz, rows, cols, vals, b, True)
    x3, it3, r3 = solve(nx, ny, nz, rows, cols, vals, b, False)
    assert rf > 0 and r3 > 0
    assert abs(itf - it3) <= 1, (itf, it3)
    scale = max(1.0, np.abs(x3).max())
    assert np.abs(xf - x3).max() <= 1e-10 * scale
    if nx * ny * nz <= 5000:
        xo, reason, its, _ = oracle_mod.ksp_solve_stencil(nx, ny, nz, coef.ravel(), b, "cg",
                                                          "jacobi", 1e-12)
        assert reason > 0 and abs(itf - its) <= 1, (itf, its)
        assert np.abs(xf - xo).max() <= 1e-9 * max(1.0, np.abs(xo).max())


def test_fused_many_chunks_large_box(gpu_lib):
    """96 x 80 x 64 (491,520 unknowns): more tiles than resident blocks, so blocks stride over
    tiles, and hundreds of iterations over several graph chunks."""
    nx, ny, nz = 96, 80, 64
    rows, cols, vals, _, b = spd_coo(nx, ny, nz, seed=5)
    xf, itf, _ = solve(nx, ny, nz, rows, cols, vals, b, True)
    x3, it3, _ = solve(nx, ny, nz, rows, cols, vals, b, False)
    print(f"\n  {nx}x{ny}x{nz}: iterations fused {itf}, three kernels {it3}")
    assert itf > 64 and abs(itf - it3) <= 1
    assert np.abs(xf - x3).max() <= 1e-10 * max(1.0, np.abs(x3).max())


@pytest.mark.parametrize("shape", [(24, 20, 32), (72, 64, 16)])
def test_re_step_solves_fused(gpu_lib, oracle_mod, shape):
    """PCA steps with FP64 Jacobi-PCG: the form asked for is what runs (profiled kernel names;
    by default one launch up to 65,536 cells, three kernels above) and the heads equal the
    three-kernel form's and the oracle's to 1e-8 m."""
    from frehg_gb300 import workloads as W
    from frehg_gb300.re_solver import Grid, ReSolver
    nx, ny, nz = shape
    w = W.config1("pca", nx=nx, ny=ny, nz=nz, steps=3)
    runs = []
    for fused in (True, False, None):
        g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
        w.apply(g)
        if fused is not None:
            g.set_fused_iteration(fused)
        g.set_profiling(True)
        for _ in range(w.steps):
            g.advance_step()
        names = {st["name"] for st in g.kernel_stats()}
        one = fused if fused is not None else nx * ny * nz <= 65536
        assert ("k_cg_iter" in names) == one, names
        assert ("k_cg_spmv" in names) == (not one), names
        runs.append(g.interior("h"))
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    for _ in range(w.steps):
        o.advance_step()
    assert np.abs(runs[0] - runs[1]).max() <= 1e-10
    assert np.abs(runs[0] - o.interior("h")).max() <= 1e-8


def test_grid_barrier_wait_runs_out(gpu_lib):
    """The barrier's bounded wait: a block that never arrives (nothing else would release the
    other) makes the other's wait run out; the kernel ends, the flag is set and the context
    stays usable (a solve runs after it)."""
    import ctypes as C
    flag = C.c_int(-1)
    for skip in (1, 0):
        assert gpu_lib.frehg_check_grid_barrier(skip, 1 << 12, C.byref(flag)) == 0, \
            gpu_lib.frehg_last_error()
        assert flag.value == 1
    assert gpu_lib.frehg_check_grid_barrier(-1, 1 << 12, C.byref(flag)) == 0
    assert flag.value == 0
    rows, cols, vals, _, b = spd_coo(6, 5, 4, seed=1)
    _, its, reason = solve(6, 5, 4, rows, cols, vals, b, True)
    assert reason > 0 and its > 0
