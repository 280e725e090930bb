"""Host-side mirror of the linear-solver seam (include/frehg2/linear/LinearSolver.hpp:18-33,
SparseSystem.hpp:15-40, LinearSolverFactory.hpp:22) over the C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import SolverConfig, check, dptr, load_library


class SparseSystem:
    """7-point system in Decomp3D owned order (row = (j*nx + i)*nz + k); nz = 1 is Decomp2D."""

    def __init__(self, solver: "GpuLinearSolver", nx: int, ny: int, nz: int = 1):
        self._lib = load_library()
        self.nx, self.ny, self.nz = nx, ny, nz
        h = C.c_void_p()
        check(self._lib.frehg_system_create(solver._h, nx, ny, nz, C.byref(h)), "createSystem")
        self._h = h
        self._solver = solver

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.frehg_system_destroy(self._h)
            self._h = None

    def n(self):
        return self.nx * self.ny * self.nz

    def preallocate(self, dd=None):
        return None

    def zeroEntries(self):
        check(self._lib.frehg_system_zero_entries(self._h), "zeroEntries")

    def beginAssembly(self):
        check(self._lib.frehg_system_begin_assembly(self._h), "beginAssembly")

    def endAssembly(self):
        check(self._lib.frehg_system_end_assembly(self._h), "endAssembly")

    def addRow(self, global_row, cols, vals):
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        check(self._lib.frehg_system_add_row(self._h, int(global_row), int(cols.size),
                                             cols.ctypes.data_as(C.POINTER(C.c_int)), dptr(vals)),
              "addRow")

    def addCOO(self, rows, cols, vals):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        check(self._lib.frehg_system_add_coo(self._h, rows.ctypes.data_as(C.POINTER(C.c_int)),
                                             cols.ctypes.data_as(C.POINTER(C.c_int)), dptr(vals),
                                             int(vals.size), 0), "addCOO")

    def setRhs(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        check(self._lib.frehg_system_set_rhs(self._h, dptr(b), 0), "setRhs")

    def getSolution(self, x=None):
        if x is None:
            x = np.empty(self.n())
        check(self._lib.frehg_system_get_solution(self._h, dptr(x), 0), "getSolution")
        return x


class GpuLinearSolver:
    """LinearSolver for the "gb300" backend (CG + Jacobi on the GPU)."""

    def __init__(self, cfg: SolverConfig):
        self._lib = load_library()
        self.config = cfg
        h = C.c_void_p()
        check(self._lib.frehg_cg_create(C.byref(cfg), C.byref(h)), "makeLinearSolver")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.frehg_cg_destroy(self._h)
            self._h = None

    def createSystem(self, nx, ny, nz=1) -> SparseSystem:
        return SparseSystem(self, nx, ny, nz)

    def setup(self, A: SparseSystem):
        check(self._lib.frehg_cg_setup(self._h, A._h), "setup")

    def solve(self, A: SparseSystem, b, x=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        if x is None:
            x = np.empty_like(b)
        check(self._lib.frehg_cg_solve(self._h, A._h, dptr(b), dptr(x), 0), "solve")
        return x

    def getIterationCount(self):
        v = C.c_int()
        check(self._lib.frehg_cg_iteration_count(self._h, C.byref(v)), "getIterationCount")
        return v.value

    def getResidualNorm(self):
        v = C.c_double()
        check(self._lib.frehg_cg_residual_norm(self._h, C.byref(v)), "getResidualNorm")
        return v.value

    def getConvergedReason(self):
        v = C.c_int()
        check(self._lib.frehg_cg_converged_reason(self._h, C.byref(v)), "getConvergedReason")
        return v.value

    def setFusedIteration(self, on):
        """FP64 Jacobi-PCG: one cooperative launch per iteration (True), three kernels (False)
        or, None (the default), one launch up to 65,536 unknowns (not in reference)."""
        v = -1 if on is None else int(bool(on))
        check(self._lib.frehg_cg_set_fused_iteration(self._h, v), "setFusedIteration")


def makeLinearSolver(backend: str, cfg: SolverConfig):
    """LinearSolverFactory (src/linear/backends/LinearSolverFactory.cpp:9-16) with the gb300
    backend; unknown backends raise, as the reference does."""
    if backend in ("gb300", "gpu"):
        return GpuLinearSolver(cfg)
    raise RuntimeError(f"makeLinearSolver: unknown / not-built linear-solver backend '{backend}' "
                       "(only 'gb300' is built here)")
