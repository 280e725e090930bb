"""Write the golden fixtures of tests/golden/ from the reference's own code (oracle/_ref).

Each case builds its inputs with frehg_gb300.workloads (seeded, deterministic), runs the
reference's ReSolver::advanceStep compiled from the reference tree (oracle/ref.py) and stores
the head and water content after the listed steps, the dt and KSP iteration count of every
step, the per-cell Ks / alpha fields where the case has them, and a SHA-256 of the other inputs
so that a test can check it rebuilt the same inputs.
Run from the repository root:  python tests/golden/gen_golden.py [case ...]
The GPU tests (tests/test_golden_gpu.py) compare the GPU step with these files; nothing at run
time needs the reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from tests.golden.cases import CASES, input_digest  # noqa: E402


def generate(name):
    from oracle import ref
    case = CASES[name]
    w = case.build()
    r = ref.RefRe(w.nx, w.ny, w.nz, w.params)
    if case.uniform_col is not None:
        r.initialize_uniform_column(case.uniform_col)
        r.attach_solver(w.solver)
    else:
        w.apply(r)
    out = {"input_sha": np.array(input_digest(w, case)), "saved": np.array(case.saved)}
    if w.Ks is not None:
        out["Ks"] = np.ascontiguousarray(w.Ks, dtype=np.float64)
    if w.alpha is not None:
        out["alpha"] = np.ascontiguousarray(w.alpha, dtype=np.float64)
    dts, dtn, its = [], [], []
    for s in range(1, case.steps + 1):
        r.advance_step()
        dts.append(r.dt_used())
        dtn.append(r.dt())
        its.append(r.last_ksp_its())
        if s in case.saved:
            out[f"h_{s}"] = r.interior("h")
            out[f"wc_{s}"] = r.interior("wc")
    out["dt_used"] = np.array(dts)
    out["dt_next"] = np.array(dtn)
    out["ksp_its"] = np.array(its, dtype=np.int32)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {case.steps} steps, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    for n in sys.argv[1:] or list(CASES):
        generate(n)
