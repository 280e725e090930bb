"""v2 YAML selection (frehg_gb300/config.py): the YAML subset reader, the groundwater capability
gate of Orchestrator::validateCapabilities (src/driver/Orchestrator.cpp:139-168) and the key
mapping of Orchestrator::buildGroundwater (:442-493).  CPU only, except the last test."""
import numpy as np
import pytest

from frehg_gb300 import config as cf

# a groundwater-only column in the reference's v2 layout (the b2-gw benchmark's physical values)
COLUMN = """
schema_version: '2.0'
simulation: {id: column, mode: groundwater}
domain:
  nx: 1
  ny: 1
  nz: 100
  dx: 1.0
  dy: 1.0
  dz: 0.01     # 1 m column
  botz: -1.0
  follow_terrain: false
time:
  dt: 0.0001
  max_steps: 100
modules:
  groundwater: true
groundwater:
  solver: pca
  full_3d: false
  adaptive_dt: true
  use_corrector: true
  use_vg: true
  air_entry_value: -0.02
  dt_max: 2.0
  dt_min: 0.0001
  co_max: 2
  specific_storage: 1.0e-05
  bc_type_gw: &gwbc
  - 0
  - 0
  - 0
  - 0
  - 0
  - 1
initial_conditions:
  groundwater:
    wc: 0.033
    h: 1.0
soil:
  map:
    from_file: false
  types:
  - id: 0
    theta_s: 0.33
    theta_r: 0.0
    vg:
      alpha: 1.43
      n: 1.56
    k_sat:
      x: 0.0
      y: 0.0
      z: 2.89e-06
legacy_raw:
  bctype_GW: *gwbc
  note: "a # inside quotes"
"""


def test_yaml_subset():
    d = cf.load_yaml_text(COLUMN)
    assert d["schema_version"] == "2.0"
    assert d["simulation"] == {"id": "column", "mode": "groundwater"}
    assert d["domain"]["nz"] == 100 and d["domain"]["dz"] == 0.01
    assert d["domain"]["follow_terrain"] is False
    assert d["groundwater"]["bc_type_gw"] == [0, 0, 0, 0, 0, 1]
    assert d["legacy_raw"]["bctype_GW"] == [0, 0, 0, 0, 0, 1]      # alias
    assert d["legacy_raw"]["note"] == "a # inside quotes"
    assert d["soil"]["types"][0]["vg"] == {"alpha": 1.43, "n": 1.56}
    assert d["soil"]["types"][0]["k_sat"]["z"] == 2.89e-6
    assert d["groundwater"]["specific_storage"] == 1e-5
    e = cf.load_yaml_text("a: [1, 2.5, x, 'y z']\nb:\n  - [1, 2]\n  - {p: 1, q: two}\nc: ~\n")
    assert e == {"a": [1, 2.5, "x", "y z"], "b": [[1, 2], {"p": 1, "q": "two"}], "c": None}
    with pytest.raises(cf.ConfigError):
        cf.load_yaml_text("a: *nothing\n")


def test_parameter_mapping():
    d = cf.load_yaml_text(COLUMN)
    scheme = cf.validate(d)
    assert scheme == "pca"
    p = cf.re_params(d, scheme)
    assert (p.dx, p.dy, p.dz, p.botz, p.dt) == (1.0, 1.0, 0.01, -1.0, 1e-4)
    assert (p.dt_min, p.dt_max, p.co_max) == (1e-4, 2.0, 2.0)
    assert p.adaptive_dt == 1 and p.use_corrector == 1 and p.use_full3d == 0
    assert list(p.bc_type) == [0, 0, 0, 0, 0, 1]
    assert (p.soil.alpha, p.soil.n, p.soil.theta_s, p.soil.Ks_z) == (1.43, 1.56, 0.33, 2.89e-6)
    assert p.soil.Ss == 1e-5 and p.soil.use_vg == 1 and p.soil.air_entry == -0.02
    assert p.scheme == 0 and p.face_mean == 0
    k = cf.solver_config(d)
    # an unset pc_type is PCSOR, the reference default (Orchestrator.cpp:489)
    assert (k.ksp_type, k.pc_type, k.rtol, k.precision) == (b"cg", b"sor", 1e-10, 0)
    # mapping form of groundwater.solver (Orchestrator.cpp:487-490) + precision extension
    d["groundwater"]["solver"] = {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-8}
    d["groundwater"]["solver_options"] = {"precision": "mixed", "ir_rtol": 1e-12}
    assert cf.validate(d) == "pca"
    k = cf.solver_config(d)
    assert k.rtol == 1e-8 and k.precision == 1 and k.ir_rtol == 1e-12
    # per-class overrides win over the groundwater-level keys (src/soil/SoilConfig.cpp:22-29)
    d["soil"]["types"][0]["specific_storage"] = 2e-5
    assert cf.soil_classes(d)[0].Ss == 2e-5
    # Picard kernel precision: unset follows the solve (-1), true FP64 (1), false float-float
    assert p.picard_fp64 == -1
    for v, want in ((True, 1), (False, 0)):
        d["groundwater"]["picard_fp64"] = v
        assert cf.re_params(d, scheme).picard_fp64 == want


def test_capability_gate():
    base = cf.load_yaml_text(COLUMN)

    def bad(mut, msg):
        d = cf.load_yaml_text(COLUMN)
        mut(d)
        with pytest.raises((cf.ConfigError, RuntimeError), match=msg):
            cf.validate(d)

    bad(lambda d: d.update(schema_version="1.0"), "schema_version")
    bad(lambda d: d["groundwater"].update(solver="newton"), "groundwater.solver")
    bad(lambda d: d["groundwater"].update(iter_solve=1), "iter_solve")
    for face in range(4):
        def lateral(d, face=face):
            d["groundwater"]["bc_type_gw"] = [0] * 6
            d["groundwater"]["bc_type_gw"][face] = 1
        bad(lateral, r"bc_type_gw\[%d\]" % face)
    bad(lambda d: d["groundwater"].update(bc_type_gw=[0, 0, 0, 0, 3, 1]), r"bc_type_gw\[4\]")
    bad(lambda d: d["groundwater"].update(bc_type_gw=[0, 0, 0, 0, 0, 3]), r"bc_type_gw\[5\]")
    bad(lambda d: d.update(solver={"backend": "petsc"}), "backend")
    # free drainage (3) at the bottom is accepted with the Picard scheme only
    d = cf.load_yaml_text(COLUMN)
    d["groundwater"].update(solver="picard", bc_type_gw=[0, 0, 0, 0, 3, 1])
    assert cf.validate(d) == "picard"
    assert cf.re_params(d, "picard").scheme == 1
    assert cf.validate(base) == "pca"
    d = cf.load_yaml_text(COLUMN)
    d["groundwater"]["solver_options"] = {"precision": "fp16"}
    with pytest.raises(cf.ConfigError, match="precision"):
        cf.solver_config(d)


def test_soil_map_files(tmp_path):
    d = cf.load_yaml_text(COLUMN)
    d["domain"].update(nx=3, ny=2, nz=2)
    d["soil"]["types"].append(dict(d["soil"]["types"][0], theta_s=0.4))
    d["soil"]["map"] = {"from_file": True, "layers": ["l0.txt", "l1.txt"]}
    (tmp_path / "l0.txt").write_text("0 1 0\n1 0 1\n")
    (tmp_path / "l1.txt").write_text("1,1,1,0,0,0\n")
    m = cf.soil_map(d, 3, 2, 2, str(tmp_path))
    assert m.is3d and list(m.index) == [0, 1, 0, 1, 0, 1, 1, 1, 1, 0, 0, 0]
    assert m.classes[1].theta_s == 0.4
    (tmp_path / "l1.txt").write_text("1 2 1 0 0 0\n")
    with pytest.raises(cf.ConfigError, match="out of range"):
        cf.soil_map(d, 3, 2, 2, str(tmp_path))
    d["soil"]["map"] = {"from_file": True, "file": "l0.txt"}
    m = cf.soil_map(d, 3, 2, 2, str(tmp_path))
    assert not m.is3d and list(m.index) == [0, 1, 0, 1, 0, 1]


@pytest.mark.gpu
def test_yaml_column_matches_oracle(gpu_lib, oracle_mod):
    """The YAML-built GPU solver steps the 1 m column like the oracle given the same values."""
    d = cf.load_yaml_text(COLUMN)
    g = cf.build_groundwater(d)
    p = cf.re_params(d, "pca")
    o = oracle_mod.OracleRe(1, 1, 100, p)
    o.initialize_geometry()
    o.set_initial_water_content(np.full(100, 0.033))
    o.finalize_initial_state()
    o.attach_solver(cf.solver_config(d))
    for s in range(200):
        g.advance_step()
        o.advance_step()
        dh = np.abs(g.interior("h") - o.interior("h")).max()
        assert dh <= 1e-8, f"step {s}: head differs by {dh:.3e} m"
        assert abs(g.dt() - o.dt()) <= 1e-12 * o.dt()


def test_recharge_polygon():
    """groundwater.recharge: columns whose centre lies in the ring get the rate (even-odd rule,
    concave ring), the rest 0; without a ring the whole top gets it."""
    d = cf.load_yaml_text(COLUMN)
    # L-shaped ring on a 6 x 4 grid of 1 m columns: the notch [3,6] x [2,4] is outside
    d["groundwater"]["recharge"] = {"rate": -1e-6,
                                    "polygon": [[0, 0], [6, 0], [6, 2], [3, 2], [3, 4], [0, 4]]}
    q = cf.recharge_field(d, 6, 4, 1.0, 1.0).reshape(4, 6)
    expect = np.zeros((4, 6))
    expect[:2, :] = -1e-6
    expect[2:, :3] = -1e-6
    assert np.array_equal(q, expect)
    d["domain"]["x0"] = 2.0  # shifted origin moves the columns, not the ring
    q = cf.recharge_field(d, 6, 4, 1.0, 1.0).reshape(4, 6)
    assert np.array_equal(q[:, 4:], np.zeros((4, 2)))
    d["groundwater"]["recharge"] = {"rate": 2e-7}
    assert np.all(cf.recharge_field(d, 6, 4, 1.0, 1.0) == 2e-7)
    del d["groundwater"]["recharge"]
    assert cf.recharge_field(d, 6, 4, 1.0, 1.0) is None


def test_constant_formula_head_ic():
    """initial_conditions.groundwater.h as a formula that is a number is a uniform head (the
    reference dispatches formula ICs as head fields); other forms are not constant heads."""
    assert cf.constant_head_ic({"h": {"type": "formula", "formula": "-500"}}) == -500.0
    assert cf.constant_head_ic({"h": {"type": "formula", "formula": "-2*z"}}) is None
    assert cf.constant_head_ic({"wc": 0.1}) is None
