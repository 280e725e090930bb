"""Mixed precision: FP32 Jacobi-PCG with compensated dots under FP64 iterative refinement to
the FP64 true residual (not in reference).  Heads are checked per step (1e-8 m) against the
FP64 oracle on the same inputs and against the plain FP64 GPU path, and the true residual of
every solve is verified."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W
from frehg_gb300.abi import SolverConfig

pytestmark = pytest.mark.gpu


def make(w):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    return g


def oracle(oracle_mod, w):
    """the oracle on the same inputs, FP64 Jacobi-PCG at the workload's rtol"""
    from tests.test_bench_path_gpu import oracle_solver
    return oracle_solver(oracle_mod, w)


@pytest.mark.parametrize("scheme", ["pca", "picard"])
def test_mixed_matches_fp64(gpu_lib, oracle_mod, scheme):
    w64 = W.config1(scheme, nx=32, ny=24, nz=32, steps=8)
    w32 = W.config1(scheme, nx=32, ny=24, nz=32, steps=8, precision=1)
    w32.solver.ir_rtol = 1e-12
    a, b, o = make(w64), make(w32), oracle(oracle_mod, w32)
    for s in range(w64.steps):
        a.advance_step()
        b.advance_step()
        o.advance_step()
        ho = o.interior("h")
        dh = np.abs(ho - b.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: mixed vs oracle head error {dh:.3e}"
        dh = np.abs(a.interior("h") - b.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: mixed vs fp64 head error {dh:.3e}"
        if scheme == "picard":
            assert b.counters().last_picard_iterations == o.last_picard_its(), s


def test_mixed_seam_true_residual(gpu_lib):
    from frehg_gb300.linear import makeLinearSolver
    from tests.test_linear_seam_gpu import assemble, spd_stencil
    nx, ny, nz = 12, 10, 16
    coef, b = spd_stencil(nx, ny, nz, seed=7)
    s = makeLinearSolver("gb300", SolverConfig("cg", "jacobi", rtol=1e-12, precision=1,
                                               ir_rtol=1e-11, inner_rtol=1e-4))
    A = s.createSystem(nx, ny, nz)
    assemble(A, coef, nx, ny, nz)
    x = s.solve(A, b)
    # true residual in FP64 on the host
    n = nx * ny * nz
    offs = [0, -nz, nz, -nz * nx, nz * nx, -1, 1]
    ax = np.zeros(n)
    for r in range(n):
        k, i, j = r % nz, (r // nz) % nx, r // (nz * nx)
        present = [True, i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1]
        for q, (o, p) in enumerate(zip(offs, present)):
            if p:
                ax[r] += coef[r, q] * x[r + o]
    assert np.linalg.norm(b - ax) <= 1.5e-11 * np.linalg.norm(b)


@pytest.mark.parametrize("shape", [(32, 24, 32), (30, 14, 27)])
@pytest.mark.parametrize("scheme", ["pca", "picard"])
def test_line_preconditioner(gpu_lib, oracle_mod, scheme, shape):
    """Vertical-line PCG inside the refinement: same heads as the oracle and as FP64 Jacobi-PCG
    on the GPU (1e-8 m) with fewer inner iterations.  (30, 14, 27): axis 0 not a multiple of 4
    (scalar SpMV) and a column length that is not a multiple of the sweep's load batch."""
    nx, ny, nz = shape
    w64 = W.config1(scheme, nx=nx, ny=ny, nz=nz, steps=6)
    wj = W.config1(scheme, nx=nx, ny=ny, nz=nz, steps=6, precision=1)
    wl = W.config1(scheme, nx=nx, ny=ny, nz=nz, steps=6, precision=1)
    for w in (wj, wl):
        w.solver.ir_rtol = 1e-12
    wl.solver.pc_type = b"line"
    a, j, l, o = make(w64), make(wj), make(wl), oracle(oracle_mod, wl)
    for s in range(w64.steps):
        for g in (a, j, l, o):
            g.advance_step()
        dh = np.abs(o.interior("h") - l.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: line-PCG vs oracle head error {dh:.3e}"
        dh = np.abs(o.interior("h") - j.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: mixed Jacobi vs oracle head error {dh:.3e}"
        dh = np.abs(a.interior("h") - l.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: line-PCG vs fp64 head error {dh:.3e}"
    its_j, its_l = j.counters().ksp_iterations, l.counters().ksp_iterations
    print(f"\n  {scheme} {shape}: inner iterations jacobi {its_j}  line {its_l}")
    assert its_l < its_j


def test_line_needs_mixed(gpu_lib):
    from frehg_gb300.abi import FrehgError
    w = W.config1("pca", nx=8, ny=8, nz=8, steps=1)
    w.solver.pc_type = b"line"
    with pytest.raises(FrehgError, match="precision"):
        make(w)
