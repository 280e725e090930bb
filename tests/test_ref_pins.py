"""The oracle against the reference's own code, compiled (oracle/_ref), on the same inputs.

oracle/ref.py compiles the reference's src/re/ReSolver.cpp (with VanGenuchten.hpp and
GwFields.hpp), src/linear/DomainDecomposition.cpp, src/core/{Grid,MpiComm}.cpp and
src/soil/SoilMap.cpp from the reference tree, against single-rank Kokkos/MPI shims; PETSc's
KSPSolve is the one part stood in for (by the oracle's restatement of it, pinned by
test_oracle_pins.py's manufactured-solution tests).  Every comparison here is bit for bit: all
nineteen halo fields the step writes, the dt sequence and the Krylov iteration counts.

These tests need the reference tree (present in the development container, absent on the GPU
machine); tests/golden/ carries the reference's outputs to the GPU tests.
"""
import numpy as np
import pytest

from frehg_gb300 import workloads as W
from frehg_gb300.abi import SoilParams

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("reference sources not present: oracle/_ref not built", allow_module_level=True)

FIELDS = ["h", "hn", "wc", "wcn", "wch", "hwc", "ch", "Kx", "Ky", "Kz", "qx", "qy", "qz",
          "Gct", "Grhs", "Gxp", "Gyp", "Gzp", "Gzm"]


def run_both(oracle_mod, w, steps=None, uniform_col=None, check_every=1):
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    r = ref.RefRe(w.nx, w.ny, w.nz, w.params)
    for s in (o, r):
        if uniform_col is not None:
            s.initialize_uniform_column(uniform_col)
            s.attach_solver(w.solver)
        else:
            w.apply(s)
    for f in FIELDS:
        assert np.array_equal(o.field(f), r.field(f)), f"initial state: field {f} differs"
    n = w.steps if steps is None else steps
    for step in range(n):
        o.advance_step()
        r.advance_step()
        assert o.dt_used() == r.dt_used() and o.dt() == r.dt(), f"step {step}: dt"
        assert o.last_ksp_its() == r.last_ksp_its(), f"step {step}: KSP iterations"
        if step % check_every == 0 or step == n - 1:
            for f in FIELDS:
                a, b = o.field(f), r.field(f)
                assert np.array_equal(a, b), (
                    f"step {step}: field {f} differs by {np.abs(a - b).max():.3e}")
    return o, r


SOILS = [
    SoilParams(alpha=1.43, n=1.56, theta_s=0.33, theta_r=0.0, Ks_z=2.89e-6, use_vg=1, air_entry=-0.02),
    W.soil(W.LOAM), W.soil(W.SAND), W.soil(W.CLAY),
    SoilParams(alpha=1.43, n=1.56, theta_s=0.33, theta_r=0.02, Ks_z=2.89e-6, use_vg=1, use_mvg=1,
               air_entry=-0.05),
]


@pytest.mark.parametrize("si", range(len(SOILS)))
def test_van_genuchten_bit_identical(oracle_mod, si):
    """VanGenuchten.hpp:31-136, every function over heads from -1000 m to +1 m."""
    s = SOILS[si]
    heads = np.concatenate([-np.logspace(-4, 3, 200), [0.0, 1e-3, 0.5, 1.0], [-0.02, -0.0199]])
    for h in heads:
        for fn in ("theta", "capacity"):
            assert oracle_mod.vg(fn, s, h) == ref.vg(fn, s, h), (fn, h)
        assert oracle_mod.vg("conductivity", s, h, s.Ks_z) == ref.vg("conductivity", s, h, s.Ks_z)
    for wc in np.linspace(s.theta_r + 1e-6, s.theta_s, 60):
        assert oracle_mod.vg("head", s, wc) == ref.vg("head", s, wc), wc
        assert oracle_mod.vg("dKdwc", s, wc, s.Ks_z) == ref.vg("dKdwc", s, wc, s.Ks_z), wc


def test_closed_box(oracle_mod):
    run_both(oracle_mod, W.small_box())


def test_closed_box_vertical_only(oracle_mod):
    run_both(oracle_mod, W.small_box(full3d=False))


def test_bottom_flux_box(oracle_mod):
    w = W.small_box()
    w.params.bc_type[4] = 2
    w.params.qbot = 1e-7
    run_both(oracle_mod, w)


def test_layered_map(oracle_mod):
    w = W.small_box(Ks=5e-5)
    slow = w.params.soil.copy(Ks_x=2e-6, Ks_y=2e-6, Ks_z=2e-6)
    idx = np.zeros((w.nz, w.ny, w.nx), np.int32)
    idx[w.nz // 2:] = 1
    w.classes, w.class_index = [w.params.soil, slow], idx.ravel()
    run_both(oracle_mod, w)


def test_column_map(oracle_mod):
    """Per-column (2D) class map (SoilMap::setClassIndex)."""
    w = W.config0("pca", nx=6, ny=5, nz=20, steps=10)
    w.classes = [W.soil(W.LOAM), W.soil(W.SAND)]
    w.class_index = (np.arange(w.nx * w.ny) % 3 == 0).astype(np.int32)
    w.class3d = False
    run_both(oracle_mod, w)


@pytest.mark.parametrize("pc", ["sor", "jacobi"])
def test_b2gw_adaptive_column(oracle_mod, pc):
    """benchmarks/b2-gw column: 400 adaptive steps (flux and Courant dt rules)."""
    w = W.b2gw_column(pc=pc, rtol=1e-10)
    run_both(oracle_mod, w, steps=400, uniform_col=0.033, check_every=25)


def test_config0_ponded_loam(oracle_mod):
    w = W.config0("pca", nx=10, ny=8, nz=40, steps=20)
    run_both(oracle_mod, w)


def test_config0_full_size_first_steps(oracle_mod):
    """40x40x100 loam, ponded top: the stated size, first 6 steps."""
    w = W.config0("pca")
    run_both(oracle_mod, w, steps=6, check_every=5)


def test_config1_grf_soil(oracle_mod):
    """Per-cell Ks / alpha fields as a fully heterogeneous 3D SoilMap; top flux, bottom
    Dirichlet with the first step's zero bottom ghost."""
    w = W.config1("pca", nx=16, ny=12, nz=24, steps=6)
    run_both(oracle_mod, w)


def test_layered_classes_with_grf(oracle_mod):
    w = W.config0("pca", nx=10, ny=9, nz=30, steps=15)
    classes, cls, Ks = W.layered_soil(w.nx, w.ny, w.nz, 5, 11)
    w.classes, w.class_index, w.Ks = classes, cls.ravel(), Ks
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.5)
    w.params.htop = 0.05
    run_both(oracle_mod, w)


def test_vertical_only_saturating_box(oracle_mod):
    w = W.config0("pca", nx=6, ny=5, nz=20, steps=30)
    w.params.use_full3d = 0
    w.h0 = np.full((w.nz, w.ny, w.nx), -0.05)
    w.h0[:3] = 0.02
    w.params.htop = 0.1
    run_both(oracle_mod, w)


def test_partial_recharge_field(oracle_mod):
    """Per-column top flux (ReSolver::setTopFluxField) on part of the top face."""
    w = W.config1("pca", nx=12, ny=10, nz=16, steps=6)
    q = np.zeros((w.ny, w.nx))
    q[2:7, 3:9] = -4e-6
    w.top_flux = q
    run_both(oracle_mod, w)


def test_adaptive_3d_grf(oracle_mod):
    w = W.config1("pca", nx=10, ny=8, nz=20, steps=25)
    w.params.adaptive_dt = 1
    w.params.dt, w.params.dt_min, w.params.dt_max = 5.0, 0.5, 120.0
    run_both(oracle_mod, w)


def test_b3_kirkland_first_steps(oracle_mod):
    """benchmarks/b3-kirkland (two-class 3D map from the layer files, partial recharge, adaptive
    dt, CG + SOR): the first 300 steps"""
    from tests.golden_util import b3_case, b3_setup
    _, inp = b3_case()
    o = oracle_mod.OracleRe(inp["nx"], inp["ny"], inp["nz"], inp["params"])
    r = ref.RefRe(inp["nx"], inp["ny"], inp["nz"], inp["params"])
    for s in (o, r):
        b3_setup(s, inp)
    for step in range(300):
        o.advance_step()
        r.advance_step()
        assert o.dt_used() == r.dt_used() and o.last_ksp_its() == r.last_ksp_its(), step
    for f in FIELDS:
        assert np.array_equal(o.field(f), r.field(f)), f
