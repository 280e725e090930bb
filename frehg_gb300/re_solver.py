"""Host-side mirror of the reference's ReSolver (src/re/ReSolver.hpp:48-156) over the C ABI.

Method names follow the reference (camelCase aliases included) so callers and tests read like
the reference's own.  Every call goes to libfrehg_gb300.so; when the library is missing the
constructor raises -- there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import (CHECKPOINT_SCALARS, KernelStat, ReCounters, ReParams, SoilParams,
                  SolverConfig, check, dptr, load_library)


class Grid:
    """Grid (src/core/Grid.hpp:153-231): sizes and the halo-padded index."""

    def __init__(self, nx, ny, nz, dx=1.0, dy=1.0, dz=1.0, dz_incre=1.0):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.dx, self.dy, self.dz, self.dz_incre = dx, dy, dz, dz_incre

    def nCell(self):
        return (self.nx + 2) * (self.ny + 2) * (self.nz + 2)

    def nActiveCell(self):
        return self.nx * self.ny * self.nz

    def getIndex(self, i, j, k):
        return (i + 1) + (j + 1) * (self.nx + 2) + (k + 1) * (self.nx + 2) * (self.ny + 2)


class SoilMap:
    """SoilMap (src/soil/SoilMap.hpp:28-92): class table + per-column or per-cell class ids."""

    def __init__(self):
        self.classes: list[SoilParams] = []
        self.index = None
        self.is3d = False

    def setClasses(self, classes):
        if not classes:
            raise ValueError("SoilMap::setClasses: empty class table")
        self.classes = list(classes)

    def setClassIndex(self, nx, ny, idx):
        idx = np.asarray(idx, dtype=np.int32).ravel()
        if idx.size != nx * ny:
            raise ValueError("SoilMap::setClassIndex: size mismatch")
        self.index, self.is3d = idx, False

    def setClassIndex3D(self, nx, ny, nz, idx):
        idx = np.asarray(idx, dtype=np.int32).ravel()
        if idx.size != nx * ny * nz:
            raise ValueError("SoilMap::setClassIndex3D: size mismatch")
        self.index, self.is3d = idx, True


# GwFields arrays in a checkpoint record (those frehg_re_get_field materialises)
GW_RECORD_FIELDS = ("h", "hn", "wc", "wcn", "wch", "hwc", "ch", "Kx", "Ky", "Kz", "qx", "qy",
                    "qz", "room", "bot3d", "dz3d", "actv")


class Fields:
    """Lazy view of GwFields (src/re/GwFields.hpp:52-59): fields['h'] is the halo array as a
    (nz+2, ny+2, nx+2) numpy array copied from the device on access."""

    def __init__(self, solver: "ReSolver"):
        self._s = solver

    def __getitem__(self, name):
        return self._s.field(name)

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        return self._s.field(name)


class ReSolver:
    def __init__(self, grid: Grid, params: ReParams | None = None):
        self._lib = load_library()
        self.grid = grid
        self._params = params.copy() if params is not None else ReParams()
        h = C.c_void_p()
        check(self._lib.frehg_re_create(grid.nx, grid.ny, grid.nz, C.byref(self._params),
                                        C.byref(h)), "ReSolver")
        self._h = h
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.frehg_re_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration ---------------------------------------------------------------------
    def set_params(self, p: ReParams):
        self._params = p.copy()
        check(self._lib.frehg_re_set_params(self._h, C.byref(self._params)), "setParams")

    def params(self) -> ReParams:
        p = ReParams()
        check(self._lib.frehg_re_get_params(self._h, C.byref(p)), "params")
        return p

    def set_soil_map(self, m: SoilMap):
        arr = (SoilParams * len(m.classes))(*m.classes)
        idx = np.ascontiguousarray(m.index, dtype=np.int32)
        check(self._lib.frehg_re_set_soil_map(self._h, arr, len(m.classes),
                                              idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                              int(m.is3d)), "setSoilMap")

    def set_cell_fields(self, Ks=None, alpha=None):
        ks = None if Ks is None else np.ascontiguousarray(Ks, dtype=np.float64).ravel()
        al = None if alpha is None else np.ascontiguousarray(alpha, dtype=np.float64).ravel()
        n = self.grid.nActiveCell()
        for a in (ks, al):
            if a is not None and a.size != n:
                raise ValueError("per-cell field must have nx*ny*nz values")
        check(self._lib.frehg_re_set_cell_fields(self._h, dptr(ks), dptr(al)), "setCellFields")

    def attach_solver(self, cfg):
        if hasattr(cfg, "config"):
            cfg = cfg.config
        check(self._lib.frehg_re_attach_solver(self._h, C.byref(cfg)), "attachSolver")

    # -- initial state ---------------------------------------------------------------------
    def _interior(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        if a.size != self.grid.nActiveCell():
            raise ValueError("expected nx*ny*nz values")
        return a

    def initialize_geometry(self):
        check(self._lib.frehg_re_initialize_geometry(self._h), "initializeGeometry")

    def set_initial_head(self, h):
        a = self._interior(h)
        check(self._lib.frehg_re_set_initial_head(self._h, dptr(a)), "setInitialHead")

    def set_initial_water_content(self, wc):
        a = self._interior(wc)
        check(self._lib.frehg_re_set_initial_water_content(self._h, dptr(a)),
              "setInitialWaterContent")

    def finalize_initial_state(self):
        check(self._lib.frehg_re_finalize_initial_state(self._h), "finalizeInitialState")

    def initialize_uniform_column(self, wc0):
        check(self._lib.frehg_re_initialize_uniform_column(self._h, float(wc0)),
              "initializeUniformColumn")

    def set_top_flux_field(self, q):
        a = np.ascontiguousarray(q, dtype=np.float64).ravel()
        if a.size != self.grid.nx * self.grid.ny:
            raise ValueError(f"ReSolver::setTopFluxField: expected nx*ny={self.grid.nx * self.grid.ny}"
                             f" values, got {a.size}")
        check(self._lib.frehg_re_set_top_flux_field(self._h, dptr(a)), "setTopFluxField")

    # -- stepping --------------------------------------------------------------------------
    def advance_step(self):
        check(self._lib.frehg_re_advance_step(self._h), "advanceStep")

    def advance_steps(self, n):
        check(self._lib.frehg_re_advance_steps(self._h, int(n)), "advanceSteps")

    def dt(self):
        v = C.c_double()
        check(self._lib.frehg_re_dt(self._h, C.byref(v)), "dt")
        return v.value

    def dt_used(self):
        v = C.c_double()
        check(self._lib.frehg_re_dt_used(self._h, C.byref(v)), "dtUsed")
        return v.value

    def time(self):
        v = C.c_double()
        check(self._lib.frehg_re_time(self._h, C.byref(v)), "time")
        return v.value

    def set_dt(self, dt):
        check(self._lib.frehg_re_set_dt(self._h, float(dt)), "setDt")

    def prime_adaptive_dt(self, dt):
        check(self._lib.frehg_re_prime_adaptive_dt(self._h, float(dt)), "primeAdaptiveDt")

    def surface_exchange(self, eta, bottom, dt, visc=1.0, min_depth=0.0):
        """Coupling::exchange through the top face (surface level eta, bed level bottom per
        column, i + j*nx); returns (eta after, limited rates q [m^3/s], total sum q dt)."""
        eta = np.array(eta, dtype=np.float64).ravel().copy()
        bottom = np.ascontiguousarray(bottom, dtype=np.float64).ravel()
        if eta.size != self.grid.nx * self.grid.ny or bottom.size != eta.size:
            raise ValueError("surface_exchange: one value per column required")
        q = np.empty_like(eta)
        tot = C.c_double()
        check(self._lib.frehg_re_surface_exchange(self._h, dptr(eta), dptr(bottom), float(dt),
                                                  float(visc), float(min_depth), dptr(q),
                                                  C.byref(tot), 0), "surface_exchange")
        return eta, q, tot.value

    def checkpoint(self) -> dict:
        """The step state (h, wc in interior order, time, dt state, budgets, ghost flag)."""
        n = self.grid.nx * self.grid.ny * self.grid.nz
        h, wc, st = np.empty(n), np.empty(n), np.empty(CHECKPOINT_SCALARS)
        check(self._lib.frehg_re_checkpoint(self._h, dptr(h), dptr(wc), dptr(st)), "checkpoint")
        return {"h": h, "wc": wc, "state": st}

    def restart(self, cp: dict):
        """Continue from a checkpoint: the parameters, soil, solver and top flux field are the
        caller's (as a reference restart rebuilds them from the configuration)."""
        h = np.ascontiguousarray(cp["h"], dtype=np.float64)
        wc = np.ascontiguousarray(cp["wc"], dtype=np.float64)
        st = np.ascontiguousarray(cp["state"], dtype=np.float64)
        check(self._lib.frehg_re_restart(self._h, dptr(h), dptr(wc), dptr(st)), "restart")

    def checkpoint_record(self) -> dict:
        """The groundwater part of the reference's checkpoint record (Orchestrator::
        writeCheckpointNow, src/driver/Orchestrator.cpp:1461-1502): cp.h, cp.hn, cp.wc, cp.wcn
        and, under "gw_<name>", every GwFields array (src/re/GwFields.hpp:62-74) that
        frehg_re_get_field materialises, each flattened in the halo layout
        ((nx+2)(ny+2)(nz+2) doubles, Grid::getIndex order), with time, dt and the layout tag
        "internal-with-halo".  The matrix and density arrays of namedViews (G*, r_*) are
        rewritten by every step before they are read and are not part of it.  The names and
        layout are the HDF5 checkpoint's (np.savez(path, **record) keeps them on disk here,
        where no HDF5 library is present)."""
        rec = {"time": np.float64(self.time()), "dt": np.float64(self.dt()),
               "storage_layout": "internal-with-halo", "has_gw": True}
        for name in GW_RECORD_FIELDS:
            rec["gw_" + name] = self.field(name).ravel().copy()
        for name in ("h", "hn", "wc", "wcn"):
            rec[name] = rec["gw_" + name]
        return rec

    def restart_from_record(self, rec):
        """Continue from a checkpoint record in the reference's layout (the groundwater part of
        Orchestrator::loadCheckpointState, Orchestrator.cpp:688-747): the head and water content
        from gw_h and gw_wc (the arrays the next step reads; it recomputes the rest), then
        primeAdaptiveDt(dt) and the record's time.  A missing field or a size mismatch raises,
        as the reference does.  The head's ghost layer tells whether a step has run (its
        enforceHeadBc wrote it; the first step after an initial state reads zero ghosts)."""
        g = self.grid
        shape = (g.nz + 2, g.ny + 2, g.nx + 2)
        arrays = {}
        for name in ("h", "wc"):
            key = "gw_" + name
            if key not in rec:
                raise RuntimeError(f"checkpoint load: missing field '{key}'")
            a = np.asarray(rec[key], dtype=np.float64)
            if a.size != shape[0] * shape[1] * shape[2]:
                raise RuntimeError(f"checkpoint load: field '{key}' size mismatch (grid differs "
                                   "from checkpoint)")
            arrays[name] = a.reshape(shape)
        h = arrays["h"]
        shell = np.ones(shape, dtype=bool)
        shell[1:-1, 1:-1, 1:-1] = False
        ghosts = bool(np.any(h[shell] != 0.0))
        dt = float(rec["dt"])
        st = np.zeros(CHECKPOINT_SCALARS)
        st[0] = float(rec.get("time", 0.0))
        st[1:4] = dt  # dt, dtn (primeAdaptiveDt) and the last step's dt
        st[7] = 1.0 if ghosts else 0.0
        self.restart({"h": np.ascontiguousarray(h[1:-1, 1:-1, 1:-1]).ravel(),
                      "wc": np.ascontiguousarray(arrays["wc"][1:-1, 1:-1, 1:-1]).ravel(),
                      "state": st})

    # -- outputs ---------------------------------------------------------------------------
    def field(self, name) -> np.ndarray:
        g = self.grid
        out = np.empty((g.nz + 2) * (g.ny + 2) * (g.nx + 2), dtype=np.float64)
        check(self._lib.frehg_re_get_field(self._h, name.encode(), dptr(out)), f"fields.{name}")
        return out.reshape(g.nz + 2, g.ny + 2, g.nx + 2)

    def fields(self) -> Fields:
        return Fields(self)

    def interior(self, name, out=None) -> np.ndarray:
        g = self.grid
        if out is None:
            out = np.empty((g.nz, g.ny, g.nx), dtype=np.float64)
        check(self._lib.frehg_re_get_interior(self._h, name.encode(), dptr(out), 0), name)
        return out

    def interior_async(self, name, out: np.ndarray) -> np.ndarray:
        """Start the copy of an interior field (h, wc, hn, wcn) into `out` (C-contiguous float64,
        page-locked for an asynchronous copy) and return at once; the values are there after
        sync().  The copy overlaps the next step (not in reference)."""
        g = self.grid
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != g.nx * g.ny * g.nz:
            raise ValueError("interior_async: out must be a C-contiguous float64 array of the grid")
        check(self._lib.frehg_re_get_interior_async(self._h, name.encode(), dptr(out)), name)
        return out

    def interior_to_device(self, name, dev_ptr: int):
        check(self._lib.frehg_re_get_interior(self._h, name.encode(),
                                              C.cast(C.c_void_p(dev_ptr), C.POINTER(C.c_double)),
                                              1), name)

    def counters(self) -> ReCounters:
        c = ReCounters()
        check(self._lib.frehg_re_get_counters(self._h, C.byref(c)), "counters")
        return c

    def water_volume(self):
        v = C.c_double()
        check(self._lib.frehg_re_water_volume(self._h, C.byref(v)), "waterVolume")
        return v.value

    def boundary_volumes(self):
        t, b = C.c_double(), C.c_double()
        check(self._lib.frehg_re_boundary_volumes(self._h, C.byref(t), C.byref(b)),
              "boundaryVolumes")
        return t.value, b.value

    def elastic_volume(self):
        """Cumulative specific-storage volume of the Picard step (not in reference)."""
        return self.counters().elastic_volume

    def set_assembly_staging(self, on: bool):
        """Stage the Picard assembly's inputs through the Tensor Memory Accelerator (same bits;
        not in reference)."""
        check(self._lib.frehg_re_set_assembly_staging(self._h, int(bool(on))), "setAssemblyStaging")

    def set_fused_iteration(self, on):
        """FP64 Jacobi-PCG solves as one cooperative launch per iteration (True), three kernels
        (False) or, None (the default), one launch up to 65,536 unknowns (not in reference)."""
        v = -1 if on is None else int(bool(on))
        check(self._lib.frehg_re_set_fused_iteration(self._h, v), "setFusedIteration")

    def set_profiling(self, on: bool):
        check(self._lib.frehg_re_set_profiling(self._h, int(bool(on))), "setProfiling")

    def kernel_stats(self) -> list[dict]:
        n = C.c_int()
        check(self._lib.frehg_re_kernel_stats(self._h, None, 0, C.byref(n)), "kernelStats")
        arr = (KernelStat * max(n.value, 1))()
        check(self._lib.frehg_re_kernel_stats(self._h, arr, n.value, C.byref(n)), "kernelStats")
        return [dict(name=a.name.decode(), launches=a.launches, total_ms=a.total_ms,
                     bytes_per_launch=a.bytes_per_launch, idle_launches=a.idle_launches)
                for a in arr[:n.value]]

    def set_stream(self, cuda_stream: int | None):
        check(self._lib.frehg_re_set_stream(self._h, C.c_void_p(cuda_stream or 0)), "setStream")

    def sync(self):
        check(self._lib.frehg_re_sync(self._h), "sync")

    # reference spellings
    setParams = set_params
    setSoilMap = set_soil_map
    attachSolver = attach_solver
    initializeGeometry = initialize_geometry
    setInitialHead = set_initial_head
    setInitialWaterContent = set_initial_water_content
    finalizeInitialState = finalize_initial_state
    initializeUniformColumn = initialize_uniform_column
    setTopFluxField = set_top_flux_field
    advanceStep = advance_step
    dtUsed = dt_used
    setDt = set_dt
    primeAdaptiveDt = prime_adaptive_dt
