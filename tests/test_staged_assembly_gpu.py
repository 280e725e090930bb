"""The TMA-staged float-float Picard assembly (cp.async.bulk.tensor into a three-stage shared
memory ring, mbarrier pipeline) writes exactly the bits of the unstaged float-float kernel:
checked after every step of Picard runs whose shapes cover full and partial tiles, slabs of one
level (the levels above and below each slab staged) and the top and bottom closures.  The steps
themselves take the staged kernel (frehg_re_set_assembly_staging), so the runs also check it
against the oracle."""
import ctypes as C

import numpy as np
import pytest

from frehg_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def run(w, steps, oracle_mod=None):
    from frehg_gb300.abi import check
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    g.set_assembly_staging(True)
    w.apply(g)
    o = None
    if oracle_mod is not None:
        from tests.test_bench_path_gpu import oracle_solver
        o = oracle_solver(oracle_mod, w)
    for s in range(steps):
        g.advance_step()
        bad = C.c_int64(-1)
        check(g._lib.frehg_re_check_staged_assembly(g._h, C.byref(bad)), "check")
        assert bad.value == 0, f"step {s}: {bad.value} entries differ"
        if o is not None:
            o.advance_step()
            dh = np.abs(g.interior("h") - o.interior("h")).max()
            assert dh <= 1e-8, f"step {s}: head differs from the oracle by {dh:.3e} m"
            assert g.counters().last_picard_iterations == o.last_picard_its()


@pytest.mark.parametrize("shape", [(64, 16, 96), (70, 21, 24), (32, 8, 40), (2, 3, 7)])
def test_staged_equals_unstaged(gpu_lib, oracle_mod, shape):
    nx, ny, nz = shape
    w = W.config4(nx=nx, ny=ny, nz=nz, steps=4, precision=1, pc="line")
    run(w, 4, oracle_mod)


def test_staged_with_top_flux_and_dirichlet_bottom(gpu_lib):
    w = W.config1("picard", nx=40, ny=12, nz=32, steps=3, precision=1)
    w.solver.pc_type = b"line"
    run(w, 3)


def test_staged_unsupported_case_reports(gpu_lib):
    from frehg_gb300.abi import FREHG_ERR_UNSUPPORTED
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config4(nx=15, ny=8, nz=10, steps=1, precision=1, pc="line")  # odd nx
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    g.advance_step()  # the unstaged kernel serves it
    bad = C.c_int64(-1)
    assert g._lib.frehg_re_check_staged_assembly(g._h, C.byref(bad)) == FREHG_ERR_UNSUPPORTED


def test_staged_wait_runs_out_and_handle_recovers(gpu_lib):
    """The staged kernel's bounded waits: with a producer that issues nothing (nothing else
    would fill a stage) every consumer's first wait runs out, the kernel ends and reports error
    word 2; the handle then steps normally and the staged kernel still matches the unstaged."""
    from frehg_gb300.abi import check
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config4(nx=64, ny=16, nz=24, steps=2, precision=1, pc="line")
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    g.set_assembly_staging(True)
    w.apply(g)
    g.advance_step()
    err = C.c_int(-1)
    check(g._lib.frehg_re_check_staged_wait(g._h, C.byref(err)), "check_staged_wait")
    assert err.value == 2
    g.advance_step()
    bad = C.c_int64(-1)
    check(g._lib.frehg_re_check_staged_assembly(g._h, C.byref(bad)), "check")
    assert bad.value == 0
