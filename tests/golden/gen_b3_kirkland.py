"""Write tests/golden/b3_kirkland.npz: the reference's b3-kirkland benchmark (2-D layered-soil
infiltration, benchmarks/b3-kirkland/b3-kirkland.yaml) run to t_end by the reference's own
ReSolver::advanceStep (compiled from its tree by oracle/ref.py), with every input the GPU test
needs (the YAML read through frehg_gb300.config: ReParams, soil classes, the per-cell class map
from the benchmark's layer files, the recharge field, the solver configuration) and the digitized
Kirkland head contours that the reference's test compares with
(tests/integration/test_b3_kirkland.cpp), read from that file.
Run from the repository root with the reference tree present:
    python tests/golden/gen_b3_kirkland.py
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REF = os.environ.get("FREHG_REFERENCE_DIR", "/root/reference")
BENCH = os.path.join(REF, "benchmarks", "b3-kirkland")
TEST = os.path.join(REF, "tests", "integration", "test_b3_kirkland.cpp")
SAVE_TIMES = (21600.0, 43200.0)  # head / water content kept at these times and at t_end


def contours():
    """kRef0 / kRef400 of the reference's test: (x, z above bottom) pairs"""
    text = open(TEST).read()
    out = {}
    for name in ("kRef0", "kRef400"):
        body = text[text.index(name):]
        body = body[body.index("{{"):body.index("}};")]
        nums = [float(v) for v in re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", body)]
        out[name] = np.array(nums).reshape(-1, 2)
    return out


def main():
    from frehg_gb300 import config as cf
    from oracle import ref
    d = cf.load_yaml(os.path.join(BENCH, "b3-kirkland.yaml"))
    scheme = cf.validate(d)
    nx, ny, nz = (int(cf.get(d, f"domain.{k}")) for k in ("nx", "ny", "nz"))
    p = cf.re_params(d, scheme)
    m = cf.soil_map(d, nx, ny, nz, BENCH)
    q = cf.recharge_field(d, nx, ny, p.dx, p.dy)
    solver = cf.solver_config(d)
    h0 = cf.constant_head_ic(cf.get(d, "initial_conditions.groundwater"))
    t_end = float(cf.get(d, "time.t_end"))
    idx = np.asarray(m.index, dtype=np.int32)
    r = ref.RefRe(nx, ny, nz, p)
    r.set_soil_map(m.classes, idx, m.is3d)
    r.initialize_geometry()
    r.set_initial_head(np.full(nx * ny * nz, h0))
    r.finalize_initial_state()
    r.attach_solver(solver)
    r.set_top_flux_field(q)
    out = {"shape": np.array([nx, ny, nz]), "params": np.frombuffer(bytes(p), np.uint8),
           "classes": np.frombuffer(b"".join(bytes(c) for c in m.classes), np.uint8),
           "nclass": np.array(len(m.classes)), "class_index": idx.astype(np.int8),
           "top_flux": q, "solver": np.frombuffer(bytes(solver), np.uint8), "h0": np.array(h0),
           "t_end": np.array(t_end), "save_times": np.array(SAVE_TIMES)}
    eps = 1e-9 * max(1.0, t_end)  # Orchestrator::runLoopSequential's end test
    t, dts, its, saved = 0.0, [], [], 0
    while t < t_end - eps:
        r.advance_step()
        t += r.dt_used()
        dts.append(r.dt_used())
        its.append(r.last_ksp_its())
        if saved < len(SAVE_TIMES) and t >= SAVE_TIMES[saved] - eps:
            out[f"h_{saved}"] = r.interior("h")
            out[f"wc_{saved}"] = r.interior("wc")
            out[f"step_{saved}"] = np.array(len(dts))
            saved += 1
    out["h_end"] = r.interior("h")
    out["wc_end"] = r.interior("wc")
    out["dt_used"] = np.array(dts)
    out["ksp_its"] = np.array(its, dtype=np.int32)
    c = contours()
    out["kirkland_h0"], out["kirkland_h400"] = c["kRef0"], c["kRef400"]
    path = os.path.join(HERE, "b3_kirkland.npz")
    np.savez_compressed(path, **out)
    print(f"b3-kirkland: {len(dts)} steps to t = {t:.1f} s, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
