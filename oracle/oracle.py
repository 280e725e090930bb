"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: ctypes wrapper of the C oracle (oracle/frehg_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs import
this module; the product package never does.  ``build()`` compiles the restatement with gcc.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from frehg_gb300.abi import ReParams, SoilParams, SolverConfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libfrehg_oracle.so")
SOURCES = [os.path.join(HERE, "frehg_oracle.c")]
DEPS = SOURCES + [os.path.join(HERE, "frehg_oracle.h"), os.path.join(HERE, "frehg_oracle_picard.inc")]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/libfrehg_oracle.so (gcc, OpenMP, -O2)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB_PATH
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall", "-o", LIB_PATH] + SOURCES + ["-lm"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


_lib = None
_PD = C.POINTER(C.c_double)
_VP = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        sig = {
            "or_re_create": (_VP, [C.c_int, C.c_int, C.c_int, C.POINTER(ReParams)]),
            "or_re_destroy": (None, [_VP]),
            "or_re_set_params": (C.c_int, [_VP, C.POINTER(ReParams)]),
            "or_re_set_soil_map": (C.c_int, [_VP, C.POINTER(SoilParams), C.c_int,
                                             C.POINTER(C.c_int32), C.c_int]),
            "or_re_set_cell_fields": (C.c_int, [_VP, _PD, _PD]),
            "or_re_attach_solver": (C.c_int, [_VP, C.POINTER(SolverConfig)]),
            "or_re_initialize_geometry": (None, [_VP]),
            "or_re_set_initial_head": (C.c_int, [_VP, _PD]),
            "or_re_set_initial_water_content": (C.c_int, [_VP, _PD]),
            "or_re_finalize_initial_state": (None, [_VP]),
            "or_re_initialize_uniform_column": (None, [_VP, C.c_double]),
            "or_re_set_top_flux_field": (C.c_int, [_VP, _PD]),
            "or_re_advance_step": (C.c_int, [_VP]),
            "or_re_dt": (C.c_double, [_VP]),
            "or_re_dt_used": (C.c_double, [_VP]),
            "or_re_time": (C.c_double, [_VP]),
            "or_re_set_dt": (None, [_VP, C.c_double]),
            "or_re_prime_adaptive_dt": (None, [_VP, C.c_double]),
            "or_re_get_field": (C.c_int, [_VP, C.c_char_p, _PD]),
            "or_re_last_ksp_its": (C.c_int, [_VP]),
            "or_re_last_system": (None, [_VP, _PD, _PD]),
            "or_re_last_picard_its": (C.c_int, [_VP]),
            "or_re_last_rnorm": (C.c_double, [_VP]),
            "or_re_total_ksp_its": (C.c_longlong, [_VP]),
            "or_re_water_volume": (C.c_double, [_VP]),
            "or_re_surface_exchange": (C.c_int, [_VP, _PD, _PD, C.c_double, C.c_double,
                                                 C.c_double, _PD, _PD]),
            "or_re_boundary_volumes": (None, [_VP, _PD, _PD]),
            "or_re_elastic_volume": (C.c_double, [_VP]),
            "or_vg_theta": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "or_vg_head": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "or_vg_capacity": (C.c_double, [C.POINTER(SoilParams), C.c_double]),
            "or_vg_conductivity": (C.c_double, [C.POINTER(SoilParams), C.c_double, C.c_double]),
            "or_vg_dKdwc": (C.c_double, [C.POINTER(SoilParams), C.c_double, C.c_double]),
            "or_ksp_solve_stencil": (C.c_int, [C.c_int, C.c_int, C.c_int, _PD, _PD, _PD,
                                               C.c_char_p, C.c_char_p, C.c_double, C.c_double,
                                               C.c_int, C.POINTER(C.c_int), _PD]),
            "or_num_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_PD)


class OracleRe:
    """CPU restatement of ReSolver with the reference's method names."""

    def __init__(self, nx, ny, nz, params: ReParams):
        self.nx, self.ny, self.nz = nx, ny, nz
        self._keep = []
        self.h = lib().or_re_create(nx, ny, nz, C.byref(params))
        if not self.h:
            raise ValueError("or_re_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_re_destroy(self.h)
            self.h = None

    def set_params(self, p):
        lib().or_re_set_params(self.h, C.byref(p))

    def set_soil_map(self, classes, index, is3d):
        arr = (SoilParams * len(classes))(*classes)
        idx = np.ascontiguousarray(index, dtype=np.int32)
        rc = lib().or_re_set_soil_map(self.h, arr, len(classes),
                                      idx.ctypes.data_as(C.POINTER(C.c_int32)), int(is3d))
        if rc:
            raise ValueError("bad soil map")

    def set_cell_fields(self, Ks=None, alpha=None):
        ks = None if Ks is None else np.ascontiguousarray(Ks, dtype=np.float64).ravel()
        al = None if alpha is None else np.ascontiguousarray(alpha, dtype=np.float64).ravel()
        lib().or_re_set_cell_fields(self.h, _d(ks), _d(al))

    def attach_solver(self, cfg: SolverConfig):
        lib().or_re_attach_solver(self.h, C.byref(cfg))

    def initialize_geometry(self):
        lib().or_re_initialize_geometry(self.h)

    def set_initial_head(self, h):
        a = np.ascontiguousarray(h, dtype=np.float64).ravel()
        lib().or_re_set_initial_head(self.h, _d(a))

    def set_initial_water_content(self, wc):
        a = np.ascontiguousarray(wc, dtype=np.float64).ravel()
        lib().or_re_set_initial_water_content(self.h, _d(a))

    def finalize_initial_state(self):
        lib().or_re_finalize_initial_state(self.h)

    def initialize_uniform_column(self, wc0):
        lib().or_re_initialize_uniform_column(self.h, wc0)

    def set_top_flux_field(self, q):
        a = np.ascontiguousarray(q, dtype=np.float64).ravel()
        lib().or_re_set_top_flux_field(self.h, _d(a))

    def advance_step(self):
        rc = lib().or_re_advance_step(self.h)
        if rc:
            raise RuntimeError(f"oracle advance_step failed ({rc})")

    def dt(self):
        return lib().or_re_dt(self.h)

    def dt_used(self):
        return lib().or_re_dt_used(self.h)

    def time(self):
        return lib().or_re_time(self.h)

    def set_dt(self, dt):
        lib().or_re_set_dt(self.h, dt)

    def field(self, name):
        """Halo array reshaped (nz+2, ny+2, nx+2)."""
        out = np.empty((self.nz + 2) * (self.ny + 2) * (self.nx + 2))
        rc = lib().or_re_get_field(self.h, name.encode(), _d(out) if False else out.ctypes.data_as(_PD))
        if rc:
            raise KeyError(name)
        return out.reshape(self.nz + 2, self.ny + 2, self.nx + 2)

    def interior(self, name):
        """Interior array (nz, ny, nx)."""
        return np.ascontiguousarray(self.field(name)[1:-1, 1:-1, 1:-1])

    def last_ksp_its(self):
        return lib().or_re_last_ksp_its(self.h)

    def last_system(self):
        """(coef (n, 7) in owned order with slots C W E S N Up Down, b (n,)) of the last
        assembled linear system"""
        n = self.nx * self.ny * self.nz
        coef, b = np.empty(7 * n), np.empty(n)
        lib().or_re_last_system(self.h, coef.ctypes.data_as(_PD), b.ctypes.data_as(_PD))
        return coef.reshape(n, 7), b

    def last_picard_its(self):
        return lib().or_re_last_picard_its(self.h)

    def total_ksp_its(self):
        return lib().or_re_total_ksp_its(self.h)

    def water_volume(self):
        return lib().or_re_water_volume(self.h)

    def surface_exchange(self, eta, bottom, dt, visc=1.0, min_depth=0.0):
        """Coupling::exchange on the oracle state; returns (eta after, q, total)"""
        eta = np.array(eta, dtype=np.float64).ravel().copy()
        bottom = np.ascontiguousarray(bottom, dtype=np.float64).ravel()
        q = np.empty_like(eta)
        tot = C.c_double()
        rc = lib().or_re_surface_exchange(self.h, _d(eta), _d(bottom), float(dt), float(visc),
                                          float(min_depth), _d(q), C.byref(tot))
        if rc != 0:
            raise RuntimeError(f"oracle surface_exchange failed ({rc})")
        return eta, q, tot.value

    def boundary_volumes(self):
        t, b = C.c_double(), C.c_double()
        lib().or_re_boundary_volumes(self.h, C.byref(t), C.byref(b))
        return t.value, b.value

    def elastic_volume(self):
        return lib().or_re_elastic_volume(self.h)


def vg(fn, soil, *args):
    return getattr(lib(), "or_vg_" + fn)(C.byref(soil), *args)


def ksp_solve_stencil(nx, ny, nz, coef, b, ksp="cg", pc="jacobi", rtol=1e-8, atol=1e-50,
                      max_it=10000):
    """PETSc-semantics solve of a 7-point owned-order system; returns (x, reason, its, rnorm)."""
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    its = C.c_int()
    rn = C.c_double()
    reason = lib().or_ksp_solve_stencil(nx, ny, nz, coef.ctypes.data_as(_PD), b.ctypes.data_as(_PD),
                                        x.ctypes.data_as(_PD), ksp.encode(), pc.encode(), rtol,
                                        atol, max_it, C.byref(its), C.byref(rn))
    return x, reason, its.value, rn.value


def num_threads():
    return lib().or_num_threads()
