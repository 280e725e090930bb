"""Surface-water exchange through the top face (Coupling::exchange, src/coupling/Coupling.cpp:
25-166): the oracle's restatement conserves water between surface and subsurface and respects
the limits (CPU); the GPU entry point matches the oracle column by column and the steps after
it keep the 1e-8 m head parity (GPU)."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W


def surface(nx, ny, rng):
    bottom = rng.uniform(-0.2, 0.2, nx * ny)
    depth = np.where(rng.random(nx * ny) < 0.5, rng.uniform(0.0, 0.05, nx * ny),
                     -rng.uniform(0.0, 0.1, nx * ny))
    depth[::7] = 2e-5  # below min_depth: no infiltration
    return bottom + depth, bottom


def test_oracle_exchange_conserves_and_limits(oracle_mod):
    w = W.config1("pca", nx=12, ny=10, nz=16, steps=1)
    o = oracle_mod.OracleRe(w.nx, w.ny, w.nz, w.params)
    w.apply(o)
    o.advance_step()
    rng = np.random.default_rng(3)
    eta, bottom = surface(w.nx, w.ny, rng)
    wc0 = o.interior("wc")[0].ravel().copy()
    v0 = o.water_volume()
    dt, az = 60.0, w.params.dx * w.params.dy
    eta1, q, total = o.surface_exchange(eta, bottom, dt, visc=1.0, min_depth=1e-4)
    v1 = o.water_volume()
    # what left the surface entered the subsurface (no clamp is active in this case)
    assert abs((eta1 - eta).sum() * az - total) < 1e-12 * max(1.0, abs(total))
    assert abs((v1 - v0) + total) < 1e-9 * v0
    dept = np.maximum(eta - bottom, 0.0)
    assert np.all(q[dept <= 1e-4] >= 0.0)                 # no infiltration from dry columns
    assert np.all(-q * dt <= dept * az + 1e-15)           # infiltration <= ponded volume
    ths = w.params.soil.theta_s
    assert np.all(o.interior("wc")[0].ravel() <= ths + 1e-15)
    assert np.any(q != 0.0)


@pytest.mark.gpu
def test_gpu_exchange_matches_oracle(gpu_lib, oracle_mod):
    from tests.test_pca_parity_gpu import pair
    w = W.config1("pca", nx=16, ny=12, nz=24, steps=4)
    g, o = pair(w, oracle_mod)
    for _ in range(2):
        g.advance_step()
        o.advance_step()
    rng = np.random.default_rng(5)
    eta, bottom = surface(w.nx, w.ny, rng)
    eg, qg, tg = g.surface_exchange(eta, bottom, 60.0, visc=1.0, min_depth=1e-4)
    eo, qo, to = o.surface_exchange(eta, bottom, 60.0, visc=1.0, min_depth=1e-4)
    assert np.allclose(qg, qo, rtol=1e-12, atol=1e-20)
    assert np.allclose(eg, eo, rtol=0, atol=1e-14)
    assert abs(tg - to) <= 1e-12 * max(1.0, abs(to))
    assert np.abs(g.interior("h") - o.interior("h")).max() <= 1e-10
    assert np.abs(g.interior("wc") - o.interior("wc")).max() <= 1e-14
    for s in range(2):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        assert dh <= 1e-8, f"step {s} after the exchange: {dh:.3e} m"


@pytest.mark.gpu
def test_gpu_exchange_device_arrays(gpu_lib):
    """device pointers (on_device = 1) give the host path's result"""
    torch = pytest.importorskip("torch")
    import ctypes as C
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config1("pca", nx=8, ny=8, nz=8, steps=1)
    rng = np.random.default_rng(9)
    eta, bottom = surface(w.nx, w.ny, rng)
    out = []
    for dev in (False, True):
        g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
        w.apply(g)
        g.advance_step()
        if not dev:
            e, q, t = g.surface_exchange(eta, bottom, 30.0)
        else:
            de = torch.tensor(eta, device="cuda")
            db = torch.tensor(bottom, device="cuda")
            dq = torch.empty_like(de)
            tot = C.c_double()
            assert g._lib.frehg_re_surface_exchange(g._h, C.c_void_p(de.data_ptr()),
                                                    C.c_void_p(db.data_ptr()), 30.0, 1.0, 0.0,
                                                    C.c_void_p(dq.data_ptr()), C.byref(tot),
                                                    1) == 0
            e, q, t = de.cpu().numpy(), dq.cpu().numpy(), tot.value
        out.append((e, q, t, g.interior("h")))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
