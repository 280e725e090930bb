"""v2 YAML selection of the groundwater step (mirror of Orchestrator::buildGroundwater and the
groundwater part of validateCapabilities, src/driver/Orchestrator.cpp:106-173, 442-493).

yaml-cpp / PyYAML are not available, so `load_yaml` reads the subset the reference's configs use:
block mappings and sequences by indentation, `- key: value` sequence items, flow sequences
`[a, b]`, anchors `&name` and aliases `*name`, comments, plain / quoted scalars
(int, float, bool, null, string).

Keys read (reference names; "not in reference" marks the extensions):
  schema_version '2.0'; domain.{nx, ny, nz, dx, dy, dz, botz}; time.dt;
  groundwater.{solver (pca | picard*), iter_solve, full_3d, adaptive_dt, use_corrector,
               dt_min, dt_max, co_max, specific_storage, use_vg, use_mvg, air_entry_value,
               bc_type_gw[6], htop, hbot, qtop, qbot, face_mean*, picard_tol*,
               picard_max_it*, solver_options*{ksp_type, pc_type, rtol, atol, max_it,
               precision, ir_rtol, inner_rtol}};
  groundwater.solver.{ksp_type, pc_type, rtol} when groundwater.solver is a mapping
  (Orchestrator.cpp:487-490); solver.backend (must be "gb300" here);
  soil.types[]{theta_s, theta_r, vg{alpha, n}, k_sat{x, y, z}, specific_storage, use_vg,
               use_mvg, air_entry_value}, soil.map.{from_file, file, layers, format};
  initial_conditions.groundwater.{h | wc} (uniform values);
  groundwater.recharge.{rate, polygon} and domain.{x0, y0} (partial-width top recharge).
"""
from __future__ import annotations

import os
import re

from .abi import ReParams, SoilParams, SolverConfig


class ConfigError(RuntimeError):
    pass


# ------------------------------------------------------------------------------------------
# YAML subset


def _scalar(tok: str):
    t = tok.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if (t[0] == t[-1]) and t[0] in "'\"" and len(t) >= 2:
        return t[1:-1]
    if t in ("true", "True", "TRUE", "yes", "on"):
        return True
    if t in ("false", "False", "FALSE", "no", "off"):
        return False
    if re.fullmatch(r"[-+]?\d+", t):
        return int(t)
    if re.fullmatch(r"[-+]?(\d+\.\d*|\.\d+|\d+)([eE][-+]?\d+)?", t) or t in (".inf", "-.inf"):
        return float(t.replace(".inf", "inf"))
    return t


def _strip_comment(line: str) -> str:
    out, q = [], None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _flow(text: str, anchors):
    text = text.strip()
    if text.startswith("[") and text.endswith("]"):
        inner = text[1:-1].strip()
        if not inner:
            return []
        return [_value(x, anchors) for x in _split_top(inner)]
    if text.startswith("{") and text.endswith("}"):
        inner = text[1:-1].strip()
        d = {}
        for item in _split_top(inner):
            k, _, v = item.partition(":")
            d[_scalar(k)] = _value(v, anchors)
        return d
    return _scalar(text)


def _split_top(s):
    parts, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur))
    return parts


def _value(tok: str, anchors):
    t = tok.strip()
    if t.startswith("*"):
        name = t[1:].strip()
        if name not in anchors:
            raise ConfigError(f"unknown YAML alias *{name}")
        return anchors[name]
    return _flow(t, anchors)


def load_yaml_text(text: str):
    lines = []
    for raw in text.splitlines():
        s = _strip_comment(raw)
        if not s.strip() or s.strip() in ("---", "..."):
            continue
        ind = len(s) - len(s.lstrip(" "))
        lines.append((ind, s.strip()))
    anchors = {}
    pos = [0]

    def take_anchor(v: str):
        m = re.match(r"&(\S+)\s*(.*)$", v)
        if m:
            return m.group(1), m.group(2)
        return None, v

    def parse_block(ind):
        if pos[0] >= len(lines):
            return None
        if lines[pos[0]][1].startswith("- ") or lines[pos[0]][1] == "-":
            return parse_seq(lines[pos[0]][0])
        return parse_map(lines[pos[0]][0])

    def parse_map(ind):
        d = {}
        while pos[0] < len(lines):
            li, s = lines[pos[0]]
            if li < ind or s.startswith("- ") or s == "-":
                break
            if li > ind:
                raise ConfigError(f"bad indentation at '{s}'")
            key, sep, rest = s.partition(":")
            if not sep:
                raise ConfigError(f"expected 'key: value' at '{s}'")
            key = _scalar(key)
            pos[0] += 1
            anchor, rest = take_anchor(rest.strip())
            if rest.strip():
                val = _value(rest, anchors)
            elif pos[0] < len(lines) and (lines[pos[0]][0] > li or
                                          (lines[pos[0]][0] == li and
                                           lines[pos[0]][1].startswith("-"))):
                val = parse_block(lines[pos[0]][0])
            else:
                val = None
            if anchor:
                anchors[anchor] = val
            d[key] = val
        return d

    def parse_seq(ind):
        out = []
        while pos[0] < len(lines):
            li, s = lines[pos[0]]
            if li != ind or not (s.startswith("- ") or s == "-"):
                break
            item = s[1:].strip()
            anchor, item = take_anchor(item)
            if not item:
                pos[0] += 1
                val = parse_block(lines[pos[0]][0]) if pos[0] < len(lines) else None
            elif re.match(r"^[^\[\{'\"]*?:(\s|$)", item):
                # "- key: value" starts a mapping whose keys sit at indent ind + 2
                lines[pos[0]] = (ind + 2, item)
                val = parse_map(ind + 2)
            else:
                pos[0] += 1
                val = _value(item, anchors)
            if anchor:
                anchors[anchor] = val
            out.append(val)
        return out

    if not lines:
        return {}
    root = parse_block(lines[0][0])
    if pos[0] != len(lines):
        raise ConfigError(f"unparsed YAML from '{lines[pos[0]][1]}'")
    return root


def load_yaml(path: str):
    with open(path) as f:
        return load_yaml_text(f.read())


# ------------------------------------------------------------------------------------------
# dotted-path access with the reference's fail-loud semantics (src/io/Config.hpp:28-53)


def get(cfg, dotted, default=KeyError):
    cur = cfg
    for part in dotted.split("."):
        if isinstance(cur, dict) and part in cur:
            cur = cur[part]
        else:
            if default is KeyError:
                raise ConfigError(f"config key '{dotted}' missing")
            return default
    return cur


# ------------------------------------------------------------------------------------------


def validate(cfg):
    """schema version and the groundwater capability gate (Orchestrator.cpp:106-173)."""
    if str(cfg.get("schema_version", "")) != "2.0":
        raise ConfigError("schema error: schema_version must be '2.0'")
    scheme = get(cfg, "groundwater.solver", "pca")
    if isinstance(scheme, dict):
        # the mapping form carries the head-solver options; the scheme then defaults to PCA
        # unless the extension key groundwater.scheme names it
        scheme = get(cfg, "groundwater.scheme", "pca")
    if scheme not in ("pca", "picard"):
        raise ConfigError(f"unsupported configuration: 'groundwater.solver' '{scheme}' is not "
                          "implemented (pca, picard)")
    if scheme == "pca" and int(get(cfg, "groundwater.iter_solve", 0) or 0) != 0:
        raise ConfigError("unsupported configuration: 'groundwater.iter_solve' must be 0 with "
                          "the PCA scheme")
    bc = get(cfg, "groundwater.bc_type_gw", None)
    if bc is not None:
        for i, mode in enumerate(bc[:6]):
            if i < 4 and int(mode) != 0:
                raise ConfigError(f"unsupported configuration: 'groundwater.bc_type_gw[{i}]' "
                                  "lateral Dirichlet/fixed-flux GW boundaries are not "
                                  "implemented")
            top = 3 if (scheme == "picard" and i == 4) else 2
            if i >= 4 and not (0 <= int(mode) <= top):
                raise ConfigError(f"unsupported configuration: 'groundwater.bc_type_gw[{i}]' "
                                  f"must be in [0, {top}]")
    backend = get(cfg, "solver.backend", "gb300")
    if backend != "gb300":
        raise RuntimeError(f"makeLinearSolver: unknown / not-built linear-solver backend "
                           f"'{backend}' (only 'gb300' is built here)")
    return scheme


def soil_classes(cfg):
    """parseSoilClasses (src/soil/SoilConfig.cpp:10-43)"""
    types = get(cfg, "soil.types", None)
    if not types:
        raise ConfigError("parseSoilClasses: soil.types is missing or empty")
    out = []
    for st in types:
        for k in ("theta_s", "theta_r", "vg", "k_sat"):
            if k not in st:
                raise ConfigError("parseSoilClasses: a soil.types entry is missing "
                                  "theta_s/theta_r/vg/k_sat")
        sp = SoilParams(theta_s=float(st["theta_s"]), theta_r=float(st["theta_r"]),
                        alpha=float(st["vg"]["alpha"]), n=float(st["vg"]["n"]),
                        Ks_x=float(st["k_sat"]["x"]), Ks_y=float(st["k_sat"]["y"]),
                        Ks_z=float(st["k_sat"]["z"]),
                        Ss=float(get(cfg, "groundwater.specific_storage", 1e-5)),
                        use_vg=int(bool(get(cfg, "groundwater.use_vg", True))),
                        use_mvg=int(bool(get(cfg, "groundwater.use_mvg", False))),
                        air_entry=float(get(cfg, "groundwater.air_entry_value", -0.02)))
        if "specific_storage" in st:
            sp.Ss = float(st["specific_storage"])
        if "use_vg" in st:
            sp.use_vg = int(bool(st["use_vg"]))
        if "use_mvg" in st:
            sp.use_mvg = int(bool(st["use_mvg"]))
        if "air_entry_value" in st:
            sp.air_entry = float(st["air_entry_value"])
        out.append(sp)
    return out


def re_params(cfg, scheme):
    """ReParams from the v2 keys (Orchestrator.cpp:452-472)"""
    p = ReParams(soil=soil_classes(cfg)[0])
    p.dx = float(get(cfg, "domain.dx"))
    p.dy = float(get(cfg, "domain.dy"))
    p.dz = float(get(cfg, "domain.dz"))
    p.botz = float(get(cfg, "domain.botz", -1.0))
    p.dt = float(get(cfg, "time.dt"))
    p.dt_min = float(get(cfg, "groundwater.dt_min", 1e-4))
    p.dt_max = float(get(cfg, "groundwater.dt_max", 2.0))
    p.co_max = float(get(cfg, "groundwater.co_max", 2.0))
    p.adaptive_dt = int(bool(get(cfg, "groundwater.adaptive_dt", True)))
    p.use_corrector = int(bool(get(cfg, "groundwater.use_corrector", True)))
    p.use_full3d = int(bool(get(cfg, "groundwater.full_3d", False)))
    p.follow_terrain = int(bool(get(cfg, "domain.follow_terrain", False)))
    for k in ("htop", "hbot", "qtop", "qbot"):
        setattr(p, k, float(get(cfg, f"groundwater.{k}", 0.0)))
    bc = get(cfg, "groundwater.bc_type_gw", None)
    if bc is not None:
        p.bc_type[:] = [int(v) for v in bc[:6]] + [0, 0, 0, 0, 0, 1][len(bc[:6]):]
    p.scheme = 1 if scheme == "picard" else 0
    fm = get(cfg, "groundwater.face_mean", "arithmetic")
    if fm not in ("arithmetic", "harmonic"):
        raise ConfigError(f"groundwater.face_mean '{fm}' (arithmetic, harmonic)")
    p.face_mean = 1 if fm == "harmonic" else 0
    p.picard_tol = float(get(cfg, "groundwater.picard_tol", 1e-6))
    p.picard_max_it = int(get(cfg, "groundwater.picard_max_it", 50))
    p.picard_dt_adapt = int(bool(get(cfg, "groundwater.picard_dt_adapt", False)))
    p.picard_dh_max = float(get(cfg, "groundwater.picard_dh_max", 0.0))
    # constitutive relations, assembly and final update of the Picard scheme in native FP64
    # (true) or in float-float arithmetic on the FP32 pipe (false); unset: float-float with
    # the mixed-precision solve, FP64 with the FP64 solve (-1)
    pf = get(cfg, "groundwater.picard_fp64", None)
    p.picard_fp64 = -1 if pf is None else int(bool(pf))
    p.rain_rate = float(get(cfg, "groundwater.rain.rate", 0.0))
    p.rain_until = float(get(cfg, "groundwater.rain.until", 0.0))
    return p


def solver_config(cfg):
    """SolverConfig of the head solve (Orchestrator.cpp:487-490) plus the precision keys"""
    sol = get(cfg, "groundwater.solver", None)
    opts = dict(sol) if isinstance(sol, dict) else {}
    opts.update(get(cfg, "groundwater.solver_options", {}) or {})
    prec = opts.get("precision", "fp64")
    if prec not in ("fp64", "mixed"):
        raise ConfigError(f"precision '{prec}' (fp64, mixed)")
    # An unset pc_type is "sor" (PETSc PCSOR, local symmetric sweep), the reference's
    # groundwater default (Orchestrator.cpp:489); the GPU realises it in FP64.
    return SolverConfig(ksp_type=str(opts.get("ksp_type", "cg")),
                        pc_type=str(opts.get("pc_type", "sor")),
                        rtol=float(opts.get("rtol", 1e-10)),
                        atol=float(opts.get("atol", 1e-50)),
                        max_it=int(opts.get("max_it", 10000)),
                        precision=1 if prec == "mixed" else 0,
                        ir_rtol=float(opts.get("ir_rtol", 1e-10)),
                        inner_rtol=float(opts.get("inner_rtol", 1e-4)))


def soil_map(cfg, nx, ny, nz, base_dir):
    """buildSoilMap (Orchestrator.cpp:495-591), list-file formats"""
    if not get(cfg, "soil.map.from_file", False):
        return None
    from .re_solver import SoilMap
    import numpy as np
    classes = soil_classes(cfg)

    def layer(path):
        p = path if os.path.isabs(path) else os.path.join(base_dir, path)
        vals = np.loadtxt(p, delimiter=None if open(p).read().find(",") < 0 else ",").ravel()
        ids = np.rint(vals).astype(np.int32)
        if ids.size != nx * ny:
            raise ConfigError(f"soil class file '{p}' has {ids.size} values; expected nx*ny")
        if ids.min() < 0 or ids.max() >= len(classes):
            raise ConfigError(f"soil class id out of range in '{p}'")
        return ids

    m = SoilMap()
    m.setClasses(classes)
    layers = get(cfg, "soil.map.layers", None)
    if layers:
        if len(layers) != nz:
            raise ConfigError(f"soil.map.layers has {len(layers)} layers but domain nz={nz}")
        m.setClassIndex3D(nx, ny, nz, np.concatenate([layer(f) for f in layers]))
    else:
        m.setClassIndex(nx, ny, layer(get(cfg, "soil.map.file", "soil_class")))
    return m


def polygon_contains(vertices, x, y):
    """Even-odd ray casting (a +x ray from each point counts edge crossings; the ring closes
    itself), with a bounding-box reject: the membership rule of the reference's polygon regions
    (src/bc/Polygon.hpp:27-55).  x, y: arrays of points; returns a boolean array."""
    import numpy as np
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    inside = np.zeros(np.broadcast(x, y).shape, dtype=bool)
    v = [(float(a), float(b)) for a, b in vertices]
    if len(v) < 3:
        return inside
    xs, ys = [p[0] for p in v], [p[1] for p in v]
    box = (x >= min(xs)) & (x <= max(xs)) & (y >= min(ys)) & (y <= max(ys))
    for q in range(len(v)):
        xi, yi = v[q]
        xj, yj = v[q - 1]
        straddles = (yi > y) != (yj > y)
        with np.errstate(divide="ignore", invalid="ignore"):
            x_cross = xj + (y - yj) * (xi - xj) / (yi - yj)
        inside ^= straddles & (x < x_cross)
    return inside & box


def recharge_field(cfg, nx, ny, dx, dy):
    """Orchestrator::buildRecharge (src/driver/Orchestrator.cpp:593-628): groundwater.recharge
    {rate, polygon}: columns whose centre (x0 + (i + 1/2) dx, y0 + (j + 1/2) dy) lies inside the
    ring get the rate [m/s, < 0 downward], the others 0; no ring (< 3 vertices) = the whole top.
    Returns the per-column top flux (index i + j*nx), or None without the section."""
    import numpy as np
    rech = get(cfg, "groundwater.recharge", None)
    if not isinstance(rech, dict):
        return None
    rate = float(rech.get("rate", 0.0) or 0.0)
    verts = [p for p in (rech.get("polygon") or []) if isinstance(p, list) and len(p) >= 2]
    x0 = float(get(cfg, "domain.x0", 0.0))
    y0 = float(get(cfg, "domain.y0", 0.0))
    xc = x0 + (np.arange(nx) + 0.5) * dx
    yc = y0 + (np.arange(ny) + 0.5) * dy
    X, Y = np.meshgrid(xc, yc)  # (ny, nx): index i + j*nx when raveled
    inside = np.ones_like(X, dtype=bool) if len(verts) < 3 else polygon_contains(verts, X, Y)
    return np.where(inside, rate, 0.0).ravel()


def constant_head_ic(ic):
    """A head IC given as a formula that is a plain number (`h: {type: formula, formula: "-500"}`,
    dispatched as a head field like the reference's formula ICs, src/ic/ICApply.cpp:211-224);
    None for any other form."""
    h = ic.get("h") if isinstance(ic, dict) else None
    if isinstance(h, dict) and h.get("type") == "formula":
        try:
            return float(str(h.get("formula")).strip())
        except ValueError:
            return None
    return None


def build_groundwater(cfg, base_dir="."):
    """Validate, then build and initialise a GPU ReSolver from a parsed v2 config."""
    import numpy as np
    from .re_solver import Grid, ReSolver
    scheme = validate(cfg)
    nx, ny, nz = (int(get(cfg, f"domain.{k}")) for k in ("nx", "ny", "nz"))
    p = re_params(cfg, scheme)
    s = ReSolver(Grid(nx, ny, nz, p.dx, p.dy, p.dz), p)
    m = soil_map(cfg, nx, ny, nz, base_dir)
    if m is not None:
        s.set_soil_map(m)
    q = recharge_field(cfg, nx, ny, p.dx, p.dy)
    if q is not None:
        s.set_top_flux_field(q)
    s.initialize_geometry()
    # setupInitialConditions / applyInitialConditions (src/ic/ICConfig.cpp:121-124,
    # src/ic/ICApply.cpp:211-224): a spatial head field wins, otherwise the (constant) water
    # content initialises every cell; its default is theta_r of soil class 0; a constant head
    # is not used.
    ic = get(cfg, "initial_conditions.groundwater", {}) or {}
    h0 = constant_head_ic(ic)
    if h0 is not None:
        s.set_initial_head(np.full(nx * ny * nz, h0))
    else:
        if ic.get("h_from_file") or ic.get("wc_from_file") or isinstance(ic.get("h"), dict) or \
                isinstance(ic.get("wc"), dict):
            raise ConfigError("raster / polygon / non-constant formula initial conditions belong "
                              "to the IC builder, which is not built here (constant wc or head)")
        wc0 = ic.get("wc")
        wc0 = p.soil.theta_r if wc0 is None else float(wc0)
        s.set_initial_water_content(np.full(nx * ny * nz, wc0))
    s.finalize_initial_state()
    s.attach_solver(solver_config(cfg))
    return s
