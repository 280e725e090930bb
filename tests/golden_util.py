"""Loading the golden fixtures of tests/golden/ and rebuilding their inputs."""
import os

import numpy as np

from tests.golden.cases import CASES, input_digest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(HERE, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


def build_inputs(name):
    """(case, workload, fixture): the workload rebuilt from its seeds, with the fixture's stored
    per-cell fields; asserts that the other inputs hash to the fixture's digest."""
    case = CASES[name]
    fx = load(name)
    w = case.build()
    assert input_digest(w, case) == str(fx["input_sha"]), f"{name}: inputs differ from the fixture's"
    if "Ks" in fx:
        w.Ks = fx["Ks"]
    if "alpha" in fx:
        w.alpha = fx["alpha"]
    return case, w, fx


# ---- b3-kirkland (tests/golden/b3_kirkland.npz, written by tests/golden/gen_b3_kirkland.py) ----

def b3_case():
    """(fixture, inputs) of the b3-kirkland benchmark: inputs = dict of nx, ny, nz, params,
    classes, class_index, top_flux, solver, h0, t_end."""
    import ctypes as C
    from frehg_gb300.abi import ReParams, SoilParams, SolverConfig
    fx = load("b3_kirkland")
    nx, ny, nz = (int(v) for v in fx["shape"])
    p = ReParams.from_buffer_copy(fx["params"].tobytes())
    raw = fx["classes"].tobytes()
    size = C.sizeof(SoilParams)
    classes = [SoilParams.from_buffer_copy(raw[q * size:(q + 1) * size])
               for q in range(int(fx["nclass"]))]
    solver = SolverConfig.from_buffer_copy(fx["solver"].tobytes())
    inp = dict(nx=nx, ny=ny, nz=nz, params=p, classes=classes,
               class_index=fx["class_index"].astype(np.int32), top_flux=fx["top_flux"],
               solver=solver, h0=float(fx["h0"]), t_end=float(fx["t_end"]))
    return fx, inp


def b3_setup(s, inp, soil_map_obj=None):
    """configure a solver (GPU ReSolver, oracle or reference) the way the Orchestrator does"""
    n = inp["nx"] * inp["ny"] * inp["nz"]
    if soil_map_obj is not None:
        s.set_soil_map(soil_map_obj)
    else:
        s.set_soil_map(inp["classes"], inp["class_index"], True)
    s.initialize_geometry()
    s.set_initial_head(np.full(n, inp["h0"]))
    s.finalize_initial_state()
    s.attach_solver(inp["solver"])
    s.set_top_flux_field(inp["top_flux"])


def b3_run(s, inp):
    """steps until t_end (Orchestrator::runLoopSequential); returns the dt sequence"""
    eps = 1e-9 * max(1.0, inp["t_end"])
    t, dts = 0.0, []
    while t < inp["t_end"] - eps:
        s.advance_step()
        t += s.dt_used()
        dts.append(s.dt_used())
    return np.array(dts)


def b3_checks(h, wc, store0, fx, inp):
    """The reference test's checks (tests/integration/test_b3_kirkland.cpp:142-197): bounded
    state, the storage gain against the prescribed recharge (5 %), a saturated plume under the
    source, and the h = 0 / h = -400 fronts against the digitized Kirkland contours (RMS
    < 0.5 m).  h, wc are (nz, ny, nx) interior arrays; returns the measured figures."""
    nx, nz = inp["nx"], inp["nz"]
    p = inp["params"]
    cls = inp["class_index"].reshape(nz, inp["ny"], nx)
    ths = np.array([c.theta_s for c in inp["classes"]])[cls]
    thr = np.array([c.theta_r for c in inp["classes"]])[cls]
    assert np.isfinite(h).all() and np.isfinite(wc).all()
    assert (wc >= thr - 1e-9).all() and (wc <= ths + 1e-9).all()
    V = p.dx * p.dy * p.dz
    added = wc.sum() * V - store0
    cols = int((inp["top_flux"] != 0).sum())
    expect = abs(float(inp["top_flux"][inp["top_flux"] != 0][0])) * cols * p.dx * p.dy * inp["t_end"]
    assert 0.95 * expect < added < 1.05 * expect, (added, expect)
    hxz = h[:, 0, :]
    src = np.nonzero(inp["top_flux"].reshape(inp["ny"], nx)[0] != 0)[0]
    nsat = int((hxz[:, src] >= 0.0).sum())
    assert nsat > 20
    height = nz * p.dz

    def rms(ref, level):
        sse, used = 0.0, 0
        for x, z in ref:
            i = min(max(int(round(x / p.dx - 0.5)), 0), nx - 1)
            wet = np.nonzero(hxz[:, i] >= level)[0]
            if wet.size:
                zf = height - (wet.max() + 0.5) * p.dz
                sse += (zf - z) ** 2
                used += 1
        return (np.sqrt(sse / used) if used else float("nan")), used

    r0, n0 = rms(fx["kirkland_h0"], 0.0)
    r4, n4 = rms(fx["kirkland_h400"], -400.0)
    assert n0 >= 10 and n4 >= 8 and r0 < 0.5 and r4 < 0.5, (r0, n0, r4, n4)
    return dict(added=added, expected=expect, saturated=nsat, rms_h0=r0, rms_h400=r4)
