"""The allocation-free CG entry point (frehg_cg_solve_noalloc).

It serves callers that may not allocate GPU memory themselves (a component under a framework
that owns the device memory budget, a time-critical loop that cannot take cudaMalloc's
synchronisation).  Checked here through the C ABI: two calls in a row, each against the
allocating entry point (frehg_cg_solve through the SparseSystem seam) on the same system, the
device memory left unchanged by a call, and the size limit refused with FREHG_ERR_BAD_ARG.
Kept in its own file so it runs after every other test."""
import ctypes as C

import numpy as np
import pytest

from frehg_gb300.abi import FREHG_ERR_BAD_ARG, FREHG_OK, SolverConfig

pytestmark = pytest.mark.gpu

TOL = 1e-12


def spd_owned(nx, ny, nz, seed):
    """symmetric diagonally dominant 7-point system in owned order (k fastest)"""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    idx = np.arange(n)
    k, i, j = idx % nz, (idx // nz) % nx, idx // (nz * nx)
    a_k = np.where(k < nz - 1, -rng.uniform(0.1, 2.0, n), 0.0)
    a_i = np.where(i < nx - 1, -rng.uniform(0.1, 2.0, n), 0.0)
    a_j = np.where(j < ny - 1, -rng.uniform(0.1, 2.0, n), 0.0)
    offsum = np.abs(a_k) + np.abs(a_i) + np.abs(a_j)
    offsum[1:] += np.abs(a_k[:-1])
    offsum[nz:] += np.abs(a_i[:-nz])
    offsum[nz * nx:] += np.abs(a_j[:-nz * nx])
    diag = offsum + rng.uniform(1e-3, 0.5, n)
    return diag, a_k, a_i, a_j


def reference_solve(nx, ny, nz, diag, a_k, a_i, a_j, b, cfg):
    """the allocating entry point: rows through addCOO, frehg_cg_solve in the three-kernel
    form of the iteration, which the allocation-free solve runs"""
    from frehg_gb300.linear import makeLinearSolver
    n = nx * ny * nz
    s = makeLinearSolver("gb300", cfg)
    s.setFusedIteration(False)
    A = s.createSystem(nx, ny, nz)
    A.zeroEntries()
    r = np.arange(n)
    rows, cols, vals = [r], [r], [diag]
    for a, off in ((a_k, 1), (a_i, nz), (a_j, nz * nx)):
        m = a != 0.0
        rows += [r[m], r[m] + off]
        cols += [r[m] + off, r[m]]
        vals += [a[m], a[m]]
    A.addCOO(np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))
    A.endAssembly()
    x = s.solve(A, b)
    return x, s.getIterationCount()


def test_noalloc_matches_allocating_solve(gpu_lib):
    torch = pytest.importorskip("torch")
    nx, ny, nz = 20, 16, 24
    cfg = SolverConfig("cg", "jacobi", rtol=1e-12)
    diag, a_k, a_i, a_j = spd_owned(nx, ny, nz, seed=11)
    rng = np.random.default_rng(5)
    rhs = [rng.standard_normal(nx * ny * nz), rng.standard_normal(nx * ny * nz)]
    dev = torch.device("cuda")
    t = {name: torch.from_numpy(v).to(dev) for name, v in
         dict(diag=diag, a_k=a_k, a_i=a_i, a_j=a_j).items()}
    tb = [torch.from_numpy(v).to(dev) for v in rhs]
    tx = [torch.empty_like(tb[0]) for _ in rhs]
    torch.cuda.synchronize()
    its = C.c_int()
    rn = C.c_double()
    for q in range(2):
        free0 = torch.cuda.mem_get_info()[0]
        rc = gpu_lib.frehg_cg_solve_noalloc(
            nx, ny, nz, t["diag"].data_ptr(), t["a_k"].data_ptr(), t["a_i"].data_ptr(),
            t["a_j"].data_ptr(), tb[q].data_ptr(), tx[q].data_ptr(), C.byref(cfg), None,
            C.byref(its), C.byref(rn))
        assert rc == FREHG_OK, gpu_lib.frehg_last_error()
        torch.cuda.synchronize()
        if q == 1:  # the first call may load the module that holds the work space
            assert torch.cuda.mem_get_info()[0] == free0
        x_ref, its_ref = reference_solve(nx, ny, nz, diag, a_k, a_i, a_j, rhs[q], cfg)
        x = tx[q].cpu().numpy()
        assert its.value == its_ref
        assert np.abs(x - x_ref).max() <= TOL * max(1.0, np.abs(x_ref).max())
    # the caller's operator arrays are left untouched
    assert np.array_equal(t["diag"].cpu().numpy(), diag)


def test_noalloc_refuses_oversized_systems(gpu_lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    cfg = SolverConfig("cg", "jacobi", rtol=1e-10)
    p = buf.data_ptr()
    rc = gpu_lib.frehg_cg_solve_noalloc(65, 65, 65, p, p, p, p, p, p, C.byref(cfg), None, None,
                                        None)
    assert rc == FREHG_ERR_BAD_ARG
    assert b"exceed" in gpu_lib.frehg_last_error()
