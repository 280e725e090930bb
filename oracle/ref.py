"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: the reference's own groundwater step, compiled.

``build()`` compiles the reference's src/re/ReSolver.cpp, src/core/Grid.cpp,
src/core/MpiComm.cpp, src/linear/DomainDecomposition.cpp, src/soil/SoilMap.cpp and
src/perf/{PerfRecorder,Timer}.cpp where they lie in the reference tree (read-only; nothing is
copied), against the Kokkos / MPI shims in oracle/ref_shim/ and the harness
oracle/ref_harness.cpp, into oracle/_ref/libfrehg_ref.so (git-ignored).  The reference tree is
at /root/reference in the development container, or wherever FREHG_REFERENCE_DIR points; where
it is absent (the GPU machine) ``available()`` is False and the tests that need it skip.  The
golden fixtures under tests/golden/ carry its outputs there.

``RefRe`` mirrors ``oracle.oracle.OracleRe`` for the PCA step, so a test can run both on the
same inputs and compare every field bit for bit.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from frehg_gb300.abi import ReParams, SoilParams, SolverConfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("FREHG_REFERENCE_DIR", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT_DIR, "libfrehg_ref.so")
REF_SOURCES = [
    "src/re/ReSolver.cpp",
    "src/core/Grid.cpp",
    "src/core/MpiComm.cpp",
    "src/linear/DomainDecomposition.cpp",
    "src/soil/SoilMap.cpp",
    "src/perf/PerfRecorder.cpp",
    "src/perf/Timer.cpp",
]
OWN = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_shim", "Kokkos_Core.hpp"),
       os.path.join(HERE, "ref_shim", "mpi.h"), os.path.join(HERE, "frehg_oracle.c"),
       os.path.join(HERE, "frehg_oracle.h")]


def sources_present() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, s)) for s in REF_SOURCES)


def build(force: bool = False) -> str | None:
    """Compile oracle/_ref/libfrehg_ref.so; returns its path, or None without the reference."""
    if not sources_present():
        return LIB_PATH if os.path.exists(LIB_PATH) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(REF_DIR, s) for s in REF_SOURCES] + OWN
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB_PATH
    # The reference builds with C++20 and no special floating-point flags (CMakeLists.txt:12);
    # contraction is switched off so no fused multiply-add changes a rounding on any host.
    flags = ["-O2", "-fPIC", "-ffp-contract=off"]
    inc = ["-I" + os.path.join(HERE, "ref_shim"), "-I" + os.path.join(REF_DIR, "include"),
           "-I" + os.path.join(REF_DIR, "src"), "-I" + HERE]
    objs = []
    oracle_obj = os.path.join(OUT_DIR, "frehg_oracle.o")
    subprocess.run(["gcc", "-std=c11", "-fopenmp", *flags, "-c", os.path.join(HERE, "frehg_oracle.c"),
                    "-o", oracle_obj], check=True)
    objs.append(oracle_obj)
    for src in REF_SOURCES + [None]:
        path = os.path.join(HERE, "ref_harness.cpp") if src is None else os.path.join(REF_DIR, src)
        obj = os.path.join(OUT_DIR, os.path.basename(path).replace(".cpp", ".o"))
        subprocess.run(["g++", "-std=c++20", *flags, *inc, "-c", path, "-o", obj], check=True)
        objs.append(obj)
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", LIB_PATH, *objs, "-lm"], check=True)
    for o in objs:
        os.remove(o)
    return LIB_PATH


def available() -> bool:
    try:
        return build() is not None
    except (OSError, subprocess.CalledProcessError):
        return False


_lib = None
_PD = C.POINTER(C.c_double)
_VP = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise FileNotFoundError("reference sources not present: oracle/_ref cannot be built")
        L = C.CDLL(path)
        sig = {
            "ref_re_create": (_VP, [C.c_int, C.c_int, C.c_int, C.POINTER(ReParams)]),
            "ref_re_destroy": (None, [_VP]),
            "ref_re_last_error": (C.c_char_p, [_VP]),
            "ref_re_set_soil_map": (C.c_int, [_VP, C.POINTER(SoilParams), C.c_int,
                                              C.POINTER(C.c_int32), C.c_int]),
            "ref_re_set_cell_fields": (C.c_int, [_VP, _PD, _PD]),
            "ref_re_attach_solver": (C.c_int, [_VP, C.POINTER(SolverConfig)]),
            "ref_re_initialize_geometry": (None, [_VP]),
            "ref_re_set_initial_head": (C.c_int, [_VP, _PD]),
            "ref_re_set_initial_water_content": (C.c_int, [_VP, _PD]),
            "ref_re_finalize_initial_state": (None, [_VP]),
            "ref_re_initialize_uniform_column": (None, [_VP, C.c_double]),
            "ref_re_set_top_flux_field": (C.c_int, [_VP, _PD]),
            "ref_re_advance_step": (C.c_int, [_VP]),
            "ref_re_dt": (C.c_double, [_VP]),
            "ref_re_dt_used": (C.c_double, [_VP]),
            "ref_re_set_dt": (None, [_VP, C.c_double]),
            "ref_re_prime_adaptive_dt": (None, [_VP, C.c_double]),
            "ref_re_last_ksp_its": (C.c_int, [_VP]),
            "ref_re_total_ksp_its": (C.c_longlong, [_VP]),
            "ref_re_get_field": (C.c_int, [_VP, C.c_char_p, _PD]),
            "ref_vg_theta": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "ref_vg_head": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "ref_vg_capacity": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "ref_vg_conductivity": (C.c_double, [C.POINTER(SoilParams), C.c_double, C.c_double]),
            "ref_vg_dKdwc": (C.c_double, [C.POINTER(SoilParams), C.c_double, C.c_double]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_PD)


class RefRe:
    """The reference's ReSolver behind the same methods as ``OracleRe``."""

    def __init__(self, nx, ny, nz, params: ReParams):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = lib().ref_re_create(nx, ny, nz, C.byref(params))
        if not self.h:
            raise ValueError("ref_re_create failed (PCA scheme and bc types 0-2 only)")

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_re_destroy(self.h)
            self.h = None

    def _check(self, rc, what):
        if rc:
            raise RuntimeError(f"{what}: {lib().ref_re_last_error(self.h).decode()}")

    def set_soil_map(self, classes, index, is3d):
        arr = (SoilParams * len(classes))(*classes)
        idx = np.ascontiguousarray(index, dtype=np.int32)
        self._check(lib().ref_re_set_soil_map(self.h, arr, len(classes),
                                              idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                              int(is3d)), "setSoilMap")

    def set_cell_fields(self, Ks=None, alpha=None):
        ks = None if Ks is None else np.ascontiguousarray(Ks, dtype=np.float64).ravel()
        al = None if alpha is None else np.ascontiguousarray(alpha, dtype=np.float64).ravel()
        self._check(lib().ref_re_set_cell_fields(self.h, _d(ks), _d(al)), "setSoilMap")

    def attach_solver(self, cfg: SolverConfig):
        self._check(lib().ref_re_attach_solver(self.h, C.byref(cfg)), "attachSolver")

    def initialize_geometry(self):
        lib().ref_re_initialize_geometry(self.h)

    def set_initial_head(self, h):
        a = np.ascontiguousarray(h, dtype=np.float64).ravel()
        self._check(lib().ref_re_set_initial_head(self.h, _d(a)), "setInitialHead")

    def set_initial_water_content(self, wc):
        a = np.ascontiguousarray(wc, dtype=np.float64).ravel()
        self._check(lib().ref_re_set_initial_water_content(self.h, _d(a)),
                    "setInitialWaterContent")

    def finalize_initial_state(self):
        lib().ref_re_finalize_initial_state(self.h)

    def initialize_uniform_column(self, wc0):
        lib().ref_re_initialize_uniform_column(self.h, wc0)

    def set_top_flux_field(self, q):
        a = np.ascontiguousarray(q, dtype=np.float64).ravel()
        self._check(lib().ref_re_set_top_flux_field(self.h, _d(a)), "setTopFluxField")

    def advance_step(self):
        self._check(lib().ref_re_advance_step(self.h), "advanceStep")

    def dt(self):
        return lib().ref_re_dt(self.h)

    def dt_used(self):
        return lib().ref_re_dt_used(self.h)

    def set_dt(self, dt):
        lib().ref_re_set_dt(self.h, dt)

    def prime_adaptive_dt(self, dt):
        lib().ref_re_prime_adaptive_dt(self.h, dt)

    def last_ksp_its(self):
        return lib().ref_re_last_ksp_its(self.h)

    def total_ksp_its(self):
        return lib().ref_re_total_ksp_its(self.h)

    def field(self, name):
        """Halo array reshaped (nz+2, ny+2, nx+2)."""
        out = np.empty((self.nz + 2) * (self.ny + 2) * (self.nx + 2))
        if lib().ref_re_get_field(self.h, name.encode(), out.ctypes.data_as(_PD)):
            raise KeyError(name)
        return out.reshape(self.nz + 2, self.ny + 2, self.nx + 2)

    def interior(self, name):
        return np.ascontiguousarray(self.field(name)[1:-1, 1:-1, 1:-1])


def vg(fn, soil, *args):
    return getattr(lib(), "ref_vg_" + fn)(C.byref(soil), *args)
