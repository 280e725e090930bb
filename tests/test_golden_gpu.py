"""GPU PCA step against the reference's own outputs (tests/golden/, written by
tests/golden/gen_golden.py from the reference's ReSolver::advanceStep compiled from its tree).

Same inputs (the fixture's per-cell fields, the others rebuilt and checked by digest); after every
saved step the head is within 1e-8 m (max norm) and the water content within 1e-9 of the
reference; every step's dt equals the reference's to 1e-12 relative and its Krylov iteration count
is the reference's (PETSc CG semantics, same preconditioner)."""
import numpy as np
import pytest

from tests.golden.cases import CASES
from tests.golden_util import build_inputs

pytestmark = pytest.mark.gpu

H_TOL = 1e-8
WC_TOL = 1e-9


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference(gpu_lib, name):
    from frehg_gb300.re_solver import Grid, ReSolver
    case, w, fx = build_inputs(name)
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    if case.uniform_col is not None:
        g.initialize_uniform_column(case.uniform_col)
        g.attach_solver(w.solver)
    else:
        w.apply(g)
    worst = 0.0
    for s in range(1, case.steps + 1):
        g.advance_step()
        assert g.dt_used() == pytest.approx(fx["dt_used"][s - 1], rel=1e-12, abs=0), f"step {s}"
        assert g.counters().last_ksp_iterations == fx["ksp_its"][s - 1], f"step {s}: KSP its"
        if s in case.saved:
            dh = np.abs(g.interior("h") - fx[f"h_{s}"]).max()
            dw = np.abs(g.interior("wc") - fx[f"wc_{s}"]).max()
            worst = max(worst, dh)
            assert dh <= H_TOL, f"step {s}: head differs from the reference by {dh:.3e} m"
            assert dw <= WC_TOL, f"step {s}: water content differs by {dw:.3e}"
    print(f"\n  {name}: max head difference to the reference {worst:.2e} m")
