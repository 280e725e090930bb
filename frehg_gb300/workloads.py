"""Synthetic workloads of the benchmark configurations (seeded; no external data).

Each builder returns a `Workload`: grid sizes, ReParams, SolverConfig, soil description
(class map and/or per-cell Ks / alpha) and the initial head.  `apply(solver)` configures any
object with the ReSolver method names (the GPU ReSolver or the CPU oracle) identically.

Loam / sand / clay parameters are the ones the benchmark configurations state.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .abi import ReParams, SoilParams, SolverConfig
from .grf import exponential_grf, lnk_lnalpha_fields

LOAM = dict(theta_s=0.43, theta_r=0.078, alpha=3.6, n=1.56, Ks=2.89e-6)
SAND = dict(theta_s=0.43, theta_r=0.045, alpha=14.5, n=2.68, Ks=8.25e-5)
CLAY = dict(theta_s=0.38, theta_r=0.068, alpha=0.8, n=1.09, Ks=5.56e-7)


def soil(d, Ss=1.0e-5, **kw) -> SoilParams:
    return SoilParams(alpha=d["alpha"], n=d["n"], theta_s=d["theta_s"], theta_r=d["theta_r"],
                      Ks_x=d["Ks"], Ks_y=d["Ks"], Ks_z=d["Ks"], Ss=Ss, use_vg=1, use_mvg=0,
                      air_entry=-0.02, **kw)


@dataclasses.dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    params: ReParams
    solver: SolverConfig
    steps: int
    h0: np.ndarray | None = None
    wc0: np.ndarray | None = None
    classes: list | None = None
    class_index: np.ndarray | None = None
    class3d: bool = True
    Ks: np.ndarray | None = None
    alpha: np.ndarray | None = None
    top_flux: np.ndarray | None = None

    @property
    def cells(self):
        return self.nx * self.ny * self.nz

    def apply(self, s):
        """Configure a solver (GPU ReSolver or oracle) following the reference call order."""
        if self.classes is not None:
            if hasattr(s, "set_soil_map") and s.__class__.__name__ in ("OracleRe", "RefRe"):
                s.set_soil_map(self.classes, self.class_index, self.class3d)
            else:
                from .re_solver import SoilMap
                m = SoilMap()
                m.setClasses(self.classes)
                if self.class3d:
                    m.setClassIndex3D(self.nx, self.ny, self.nz, self.class_index)
                else:
                    m.setClassIndex(self.nx, self.ny, self.class_index)
                s.set_soil_map(m)
        if self.Ks is not None or self.alpha is not None:
            s.set_cell_fields(self.Ks, self.alpha)
        s.initialize_geometry()
        if self.h0 is not None:
            s.set_initial_head(self.h0)
        else:
            s.set_initial_water_content(self.wc0)
        s.finalize_initial_state()
        s.attach_solver(self.solver)
        if self.top_flux is not None:
            s.set_top_flux_field(self.top_flux)
        return s


def hydrostatic_head(nz, dz, depth_table):
    zc = (np.arange(nz) + 0.5) * dz  # depth of the cell centre below the top
    return zc - depth_table


def config0(scheme="pca", nx=40, ny=40, nz=100, steps=120, rtol=1e-12) -> Workload:
    """40x40x100 loam infiltration, ponded top (+0.01 m), h0 = -2 m, dt = 30 s x 120.

    scheme "pca": the reference's PCA step with its bottom rule set (free drainage is not a
    reference boundary, so the bottom is no-flux); "picard": the mixed-form Picard step with the
    unit-gradient free-drainage bottom (bc 3)."""
    p = ReParams(soil=soil(LOAM), dx=0.1, dy=0.1, dz=0.01, botz=-0.01 * nz, dt=30.0, dt_min=30.0,
                 dt_max=30.0, adaptive_dt=0, use_corrector=1, use_full3d=1,
                 bc_type=[0, 0, 0, 0, 0, 1], htop=0.01)
    if scheme == "picard":
        p.scheme = 1
        p.bc_type[4] = 3
        p.picard_tol = 1.0e-6
        p.picard_max_it = 50
    h0 = np.full((nz, ny, nx), -2.0)
    return Workload(f"c0-{scheme}-{nx}x{ny}x{nz}", nx, ny, nz, p,
                    SolverConfig("cg", "jacobi", rtol=rtol, max_it=20000), steps, h0=h0)


def config1(scheme="pca", nx=256, ny=256, nz=128, steps=60, seed_k=1, seed_a=2, rtol=1e-12,
            precision=0) -> Workload:
    """256x256x128 heterogeneous loam: ln Ks GRF (sigma 1, exponential, 8x8x4 cells), ln alpha
    correlated (rho 0.7, sigma 0.3); hydrostatic start with the water table 4 m below the top;
    20 mm/h rain on top; bottom head fixed at its hydrostatic value; dt = 60 s x 60."""
    dz = 0.05
    ln_ks, ln_a = lnk_lnalpha_fields((nz, ny, nx), (4.0, 8.0, 8.0), seed_k, seed_a,
                                     math.log(LOAM["Ks"]), 1.0, math.log(LOAM["alpha"]), 0.3, 0.7)
    depth = nz * dz
    p = ReParams(soil=soil(LOAM), dx=1.0, dy=1.0, dz=dz, botz=-depth, dt=60.0, dt_min=60.0,
                 dt_max=60.0, adaptive_dt=0, use_corrector=1, use_full3d=1,
                 bc_type=[0, 0, 0, 0, 1, 2], qtop=-20.0e-3 / 3600.0, hbot=depth - 4.0)
    if scheme == "picard":
        p.scheme = 1
    h0 = np.broadcast_to(hydrostatic_head(nz, dz, 4.0)[:, None, None], (nz, ny, nx)).copy()
    return Workload(f"c1-{scheme}-{nx}x{ny}x{nz}", nx, ny, nz, p,
                    SolverConfig("cg", "jacobi", rtol=rtol, max_it=20000, precision=precision),
                    steps, h0=h0, Ks=np.exp(ln_ks), alpha=np.exp(ln_a))


def config2(scheme="pca", nx=512, ny=512, nz=128, steps=60) -> Workload:
    """config 1's generator at 512x512x128 with new seeds, FP32 Krylov under FP64 refinement."""
    w = config1(scheme, nx, ny, nz, steps, seed_k=3, seed_a=4, precision=1)
    w.name = f"c2-{scheme}-{nx}x{ny}x{nz}"
    w.solver.ir_rtol = 1e-10
    return w


def layered_soil(nx, ny, nz, seed_layers, seed_k, sigma=1.5, corr=(4.0, 8.0, 8.0)):
    """Sand / loam / clay layers at seeded random interface depths, each with an in-layer
    ln Ks GRF (sigma 1.5).  Returns (classes, class_index, Ks)."""
    rng = np.random.Generator(np.random.PCG64(seed_layers))
    k1 = int(rng.integers(nz // 6, nz // 3))
    k2 = int(rng.integers(nz // 2, (5 * nz) // 6))
    cls = np.zeros((nz, ny, nx), dtype=np.int32)
    cls[k1:k2] = 1
    cls[k2:] = 2
    classes = [soil(SAND), soil(LOAM), soil(CLAY)]
    base = np.array([SAND["Ks"], LOAM["Ks"], CLAY["Ks"]])
    xi = exponential_grf((nz, ny, nx), corr, seed_k)
    Ks = base[cls] * np.exp(sigma * xi)
    return classes, cls, Ks


def config3(scheme="pca", nx=256, ny=256, nz=128, steps=60, seed=5, precision=1,
            pc="unet-line", rtol=1e-12, ir_rtol=1e-12) -> Workload:
    """256x256x128 three-layer soil (sand / loam / clay at seeded interface depths, in-layer
    ln Ks GRF sigma 1.5, 8x8x4 cells) under config 1's forcing: hydrostatic start with the
    water table at 0.625 of the depth (4 m at 6.4 m), 20 mm/h rain on top, bottom head fixed,
    dt = 60 s.  The learned preconditioner's configuration (FCG under FP64 refinement)."""
    w = config1(scheme, nx=nx, ny=ny, nz=nz, steps=steps, rtol=rtol, precision=precision)
    classes, cls, Ks = layered_soil(nx, ny, nz, seed_layers=seed, seed_k=1000 + seed)
    w.classes, w.class_index, w.Ks, w.alpha = classes, cls.ravel(), Ks, None
    depth = nz * w.params.dz
    table = 0.625 * depth
    w.h0 = np.broadcast_to(hydrostatic_head(nz, w.params.dz, table)[:, None, None],
                           (nz, ny, nx)).copy()
    w.params.hbot = depth - table
    w.solver.pc_type = pc.encode() if precision == 1 else b"jacobi"
    w.solver.ir_rtol = ir_rtol
    if scheme == "picard":
        # across the sand / clay contrasts a 60 s Picard step does not converge in 50
        # iterations (nor in native FP64): a failed step is retried at half the time step and
        # the Picard count brings dt back towards 60 s
        p = w.params
        p.picard_dt_adapt = 1
        p.dt_min, p.dt_max = 5.0, 60.0
    w.name = f"c3-{scheme}-{nx}x{ny}x{nz}-seed{seed}"
    return w


def config4(nx=768, ny=768, nz=96, steps=200, seeds=(6, 7), precision=1, pc="unet-line",
            rtol=1e-12, ir_rtol=1e-12) -> Workload:
    """768x768x96 three-layer soil (config 3's generator, new seeds), dry start h = -5 m,
    50 mm/h rain for the first 1800 s then none (the surface does not pond: rain beyond what
    the top face admits at h = 0 runs off), free-drainage bottom, lateral no-flux, mixed-form
    Picard (|dh|_inf < 1e-6 m, at most 1 m head change per iteration) with the time step driven
    by the Picard count between 10 and 120 s, 200 steps."""
    dz = 0.05
    classes, cls, Ks = layered_soil(nx, ny, nz, seed_layers=seeds[0], seed_k=seeds[1])
    p = ReParams(soil=soil(LOAM), dx=1.0, dy=1.0, dz=dz, botz=-nz * dz, dt=10.0, dt_min=10.0,
                 dt_max=120.0, adaptive_dt=0, use_corrector=1, use_full3d=1,
                 bc_type=[0, 0, 0, 0, 3, 2], qtop=0.0)
    p.scheme = 1
    p.picard_tol = 1.0e-6
    p.picard_max_it = 50
    p.picard_dt_adapt = 1
    p.picard_dh_max = 1.0
    p.rain_rate = -50.0e-3 / 3600.0
    p.rain_until = 1800.0
    solver = SolverConfig("cg", pc if precision == 1 else "jacobi", rtol=rtol, max_it=20000,
                          precision=precision, ir_rtol=ir_rtol)
    return Workload(f"c4-picard-{nx}x{ny}x{nz}", nx, ny, nz, p, solver, steps,
                    h0=np.full((nz, ny, nx), -5.0), classes=classes, class_index=cls.ravel(),
                    Ks=Ks)


def small_box(nx=4, ny=4, nz=8, steps=40, full3d=True, Ks=1.0e-5) -> Workload:
    """tests/re/test_re_3d.cpp's closed heterogeneous box (dx=2, dy=1, dz=0.05, dt=5, Ss=0)."""
    s = SoilParams(alpha=2.0, n=1.6, theta_s=0.45, theta_r=0.05, Ks_x=Ks, Ks_y=Ks, Ks_z=Ks,
                   Ss=0.0, use_vg=1)
    p = ReParams(soil=s, dx=2.0, dy=1.0, dz=0.05, botz=-0.05 * nz, dt=5.0, adaptive_dt=0,
                 use_corrector=1, use_full3d=int(full3d), bc_type=[0] * 6)
    gi = np.arange(nx)[None, None, :]
    gj = np.arange(ny)[None, :, None]
    wc = (0.20 + 0.03 * np.sin(0.9 * gi) + 0.02 * np.cos(0.7 * gj)) * np.ones((nz, 1, 1))
    return Workload(f"box-{nx}x{ny}x{nz}", nx, ny, nz, p,
                    SolverConfig("cg", "jacobi", rtol=1e-13), steps, wc0=wc)


def b2gw_column(pc="jacobi", rtol=1e-10, adaptive=True) -> Workload:
    """benchmarks/b2-gw: 1x1x100 column, wc0 = 0.033, top head 0, adaptive dt from 1e-4 s."""
    s = SoilParams(alpha=1.43, n=1.56, theta_s=0.33, theta_r=0.0, Ks_x=0.0, Ks_y=0.0,
                   Ks_z=2.89e-6, Ss=1.0e-5, use_vg=1, air_entry=-0.02)
    p = ReParams(soil=s, dx=1.0, dy=1.0, dz=0.01, botz=-1.0, dt=1e-4, dt_min=1e-4, dt_max=2.0,
                 co_max=2.0, adaptive_dt=int(adaptive), use_corrector=1, use_full3d=0,
                 bc_type=[0, 0, 0, 0, 0, 1], htop=0.0)
    return Workload("b2-gw", 1, 1, 100, p, SolverConfig("cg", pc, rtol=rtol), 0,
                    wc0=np.full((100, 1, 1), 0.033))
