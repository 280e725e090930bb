"""Why the learned correction cannot pay on the three-layer soil: where line-PCG's error lives.

The learned-preconditioner configuration's hard systems come from the first time step: rain on
dry sand over loam and clay, Picard iterations that do not converge at dt = 60 s, and linear
systems whose FP64 Jacobi-PCG needs thousands of iterations.  This study takes such a system
from the oracle (8 Picard iterations into the first step of a 16 x 16 x 64 window), scales it
to unit diagonal as the solvers do, and compares preconditioners inside CG (numpy / scipy on
the CPU):

* the vertical-line (column tridiagonal) preconditioner removes most of Jacobi's iterations;
* two-level corrections with exact coarse solves over aggregates of 1x1 (whole columns), 2x2
  and 4x4 columns by 8 to all levels -- the smooth, domain-wide lateral modes a 3-level U-Net's
  receptive field could not represent -- change line-PCG's iteration count by a few percent
  only: the error is not smooth;
* after 30 line-PCG iterations more than 99 % of the error energy sits in the top sand layer
  (class 0), spread over individual cells (column means hold a few percent of it), while an
  incomplete LU factorisation (sequential, not a GPU method) needs a fraction of line-PCG's
  iterations.

So what remains after the line solve is local, cell-to-cell structure of the wetting front in
dry sand (conductivity contrasts of many orders of magnitude between neighbouring cells), which
depends on the current head field rather than on the soil's static lnK; a correction that pays
would have to remove it in fewer operations than the line-PCG iterations it saves."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W

sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")

NX = NY = 16
NZ = 64


@pytest.fixture(scope="module")
def hard_system(oracle_mod):
    w = W.config3("picard", nx=NX, ny=NY, nz=NZ, steps=1, precision=0, pc="jacobi")
    w.params.picard_max_it = 8
    w.params.picard_dt_adapt = 0
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    try:
        o.advance_step()  # stops after 8 Picard iterations without converging
    except RuntimeError:
        pass
    jacobi_its = o.last_ksp_its()
    coef, b = o.last_system()
    n = NX * NY * NZ
    r = np.arange(n)
    k, i, j = r % NZ, (r // NZ) % NX, r // (NZ * NX)
    rows, cols, vals = [r], [r], [coef[:, 0]]
    for slot, off, ok in ((2, NZ, i < NX - 1), (4, NZ * NX, j < NY - 1), (6, 1, k < NZ - 1)):
        rows += [r[ok], r[ok] + off]
        cols += [r[ok] + off, r[ok]]
        vals += [coef[ok, slot], coef[ok, slot]]
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    s = 1.0 / np.sqrt(A.diagonal())
    As = (sp.diags(s) @ A @ sp.diags(s)).tocsr()
    cls = np.asarray(w.class_index).reshape(NZ, NY, NX)[k, j, i]
    return dict(A=As, b=s * b, k=k, i=i, j=j, cls=cls, jacobi_its=jacobi_its)


def line_solver(hs):
    A, k = hs["A"], hs["k"]
    n = A.shape[0]
    d = A.diagonal()
    up = np.zeros(n)
    up[:-1] = A.diagonal(1)
    up[k == NZ - 1] = 0.0
    D, U = d.reshape(-1, NZ).T, up.reshape(-1, NZ).T
    c = np.zeros_like(D)
    m = np.zeros_like(D)
    m[0] = D[0]
    c[0] = U[0] / m[0]
    for q in range(1, NZ):
        m[q] = D[q] - U[q - 1] * c[q - 1]
        c[q] = U[q] / m[q]

    def solve(rv):
        R = rv.reshape(-1, NZ).T
        y = np.zeros_like(R)
        y[0] = R[0] / m[0]
        for q in range(1, NZ):
            y[q] = (R[q] - U[q - 1] * y[q - 1]) / m[q]
        for q in range(NZ - 2, -1, -1):
            y[q] -= c[q] * y[q + 1]
        return y.T.ravel()
    return solve


def pcg(A, b, M, maxit=4000, tol=1e-10, keep=None):
    """flexible CG (Polak-Ribiere beta); returns iterations (and the iterate after `keep`)"""
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    p = z.copy()
    rz = r @ z
    b0 = np.linalg.norm(b)
    snap = None
    for it in range(maxit):
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        rold = r.copy()
        r -= a * q
        if keep is not None and it + 1 == keep:
            snap = x.copy()
        if np.linalg.norm(r) <= tol * b0:
            return it + 1, snap
        zn = M(r)
        beta = (zn @ (r - rold)) / rz
        rz = zn @ r
        p = zn + beta * p
    return maxit, snap


def test_line_pcg_error_is_local_to_the_wet_sand(hard_system):
    hs = hard_system
    A, b = hs["A"], hs["b"]
    line = line_solver(hs)
    its_line, x30 = pcg(A, b, line, keep=30)
    print(f"\n  hard first-step system {NX}x{NY}x{NZ}: FP64 Jacobi-PCG {hs['jacobi_its']} "
          f"iterations (oracle), line-PCG {its_line}")
    assert its_line < hs["jacobi_its"] / 4
    # geometric two-level corrections (exact coarse solves) do not help
    for bx, bz in ((1, NZ), (2, 8), (4, 8), (4, NZ)):
        agg = ((hs["j"] // bx) * (NX // bx) + hs["i"] // bx) * (NZ // bz) + hs["k"] // bz
        P = sp.csr_matrix((np.ones(A.shape[0]), (np.arange(A.shape[0]), agg)))
        lu = spla.splu((P.T @ A @ P).tocsc())
        its2, _ = pcg(A, b, lambda rv, P=P, lu=lu: line(rv) + P @ lu.solve(P.T @ rv))
        print(f"  line + exact coarse solve on {bx}x{bx}x{bz} aggregates "
              f"({P.shape[1]} unknowns): {its2} iterations")
        assert its2 > 0.85 * its_line
    # where the error is after 30 line-PCG iterations
    x_ex = spla.spsolve(A.tocsc(), b)
    e = x_ex - x30
    e2 = e * e
    sand = e2[hs["cls"] == 0].sum() / e2.sum()
    col_mean = e.reshape(-1, NZ).mean(axis=1)
    smooth = (col_mean ** 2).sum() * NZ / e2.sum()
    print(f"  after 30 line-PCG iterations: {100 * sand:.2f} % of the error energy in the sand "
          f"layer, {100 * smooth:.1f} % in column means")
    assert sand > 0.99 and smooth < 0.2
    # a sequential incomplete factorisation removes it
    ilu = spla.spilu(A.tocsc(), drop_tol=1e-4, fill_factor=5)
    its_ilu, _ = pcg(A, b, ilu.solve)
    print(f"  incomplete LU (drop 1e-4, sequential): {its_ilu} iterations")
    assert its_ilu < its_line / 3
