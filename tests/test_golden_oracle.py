"""The oracle against the reference's outputs stored in tests/golden/ (no reference tree needed).

The fixtures were written by tests/golden/gen_golden.py from the reference's own
ReSolver::advanceStep (compiled by oracle/ref.py).  On the machine that wrote them the oracle
reproduces them bit for bit; elsewhere the C library's pow/exp/log may round differently in the
last bit, so the bound is 1e-12 m in head and 1e-13 in water content.
"""
import platform

import numpy as np
import pytest

from tests.golden.cases import CASES
from tests.golden_util import load, build_inputs

EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference(oracle_mod, name):
    case, w, fx = build_inputs(name)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    if case.uniform_col is not None:
        o.initialize_uniform_column(case.uniform_col)
        o.attach_solver(w.solver)
    else:
        w.apply(o)
    for s in range(1, case.steps + 1):
        o.advance_step()
        assert o.dt_used() == pytest.approx(fx["dt_used"][s - 1], rel=1e-12, abs=0)
        assert o.last_ksp_its() == fx["ksp_its"][s - 1], f"step {s}"
        if s in case.saved:
            dh = np.abs(o.interior("h") - fx[f"h_{s}"]).max()
            dw = np.abs(o.interior("wc") - fx[f"wc_{s}"]).max()
            if EXACT:
                assert dh == 0.0 and dw == 0.0, f"step {s}: {dh:.3e} m / {dw:.3e}"
            else:
                assert dh <= 1e-12 and dw <= 1e-13, f"step {s}: {dh:.3e} m / {dw:.3e}"
