"""ctypes mirror of include/frehg_gb300.h (structs, status codes) and the loader of the CUDA
library ``frehg_gb300/_lib/libfrehg_gb300.so``.

The loader fails loudly: when the shared library is missing or cannot be loaded it raises
``RuntimeError`` -- there is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libfrehg_gb300.so")

FREHG_OK = 0
FREHG_ERR_BAD_ARG = 1
FREHG_ERR_CUDA = 2
FREHG_ERR_NOT_CONVERGED = 3
FREHG_ERR_NONFINITE = 4
FREHG_ERR_STATE = 5
FREHG_ERR_UNSUPPORTED = 6
FREHG_ERR_NO_DEVICE = 7
# doubles of a checkpoint's state block (frehg_re_checkpoint, include/frehg_gb300.h)
CHECKPOINT_SCALARS = 10

STATUS_NAMES = {
    0: "FREHG_OK",
    1: "FREHG_ERR_BAD_ARG",
    2: "FREHG_ERR_CUDA",
    3: "FREHG_ERR_NOT_CONVERGED",
    4: "FREHG_ERR_NONFINITE",
    5: "FREHG_ERR_STATE",
    6: "FREHG_ERR_UNSUPPORTED",
    7: "FREHG_ERR_NO_DEVICE",
}


class SoilParams(C.Structure):
    """struct SoilParams (include/frehg2/re/SoilParams.hpp:13-25)."""

    _fields_ = [
        ("alpha", C.c_double),
        ("n", C.c_double),
        ("theta_s", C.c_double),
        ("theta_r", C.c_double),
        ("Ks_x", C.c_double),
        ("Ks_y", C.c_double),
        ("Ks_z", C.c_double),
        ("Ss", C.c_double),
        ("use_vg", C.c_int32),
        ("use_mvg", C.c_int32),
        ("air_entry", C.c_double),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.alpha, self.n, self.theta_s, self.theta_r = 1.43, 1.56, 0.33, 0.0
        self.Ks_x, self.Ks_y, self.Ks_z, self.Ss = 0.0, 0.0, 2.89e-6, 1.0e-5
        self.use_vg, self.use_mvg, self.air_entry = 1, 0, -0.02
        for k, v in kw.items():
            setattr(self, k, v)

    def copy(self, **kw):
        s = SoilParams()
        C.pointer(s)[0] = self
        for k, v in kw.items():
            setattr(s, k, v)
        return s


class ReParams(C.Structure):
    """struct ReParams (src/re/ReSolver.hpp:24-46) plus the spec extension keys."""

    _fields_ = [
        ("soil", SoilParams),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("dz", C.c_double),
        ("botz", C.c_double),
        ("dt", C.c_double),
        ("dt_min", C.c_double),
        ("dt_max", C.c_double),
        ("co_max", C.c_double),
        ("adaptive_dt", C.c_int32),
        ("use_corrector", C.c_int32),
        ("use_full3d", C.c_int32),
        ("follow_terrain", C.c_int32),
        ("sim_shallowwater", C.c_int32),
        ("baroclinic", C.c_int32),
        ("bc_type", C.c_int32 * 6),
        ("htop", C.c_double),
        ("hbot", C.c_double),
        ("qtop", C.c_double),
        ("qbot", C.c_double),
        ("scheme", C.c_int32),
        ("face_mean", C.c_int32),
        ("picard_max_it", C.c_int32),
        ("picard_tol", C.c_double),
        ("rain_rate", C.c_double),
        ("rain_until", C.c_double),
        ("picard_dt_adapt", C.c_int32),
        ("picard_fp64", C.c_int32),
        ("picard_dh_max", C.c_double),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.soil = SoilParams()
        self.dx, self.dy, self.dz, self.botz = 1.0, 1.0, 0.01, -1.0
        self.dt, self.dt_min, self.dt_max, self.co_max = 1.0e-4, 1.0e-4, 2.0, 2.0
        self.adaptive_dt, self.use_corrector, self.use_full3d = 1, 1, 0
        self.follow_terrain, self.sim_shallowwater, self.baroclinic = 0, 0, 0
        self.bc_type[:] = [0, 0, 0, 0, 0, 1]
        self.htop = self.hbot = self.qtop = self.qbot = 0.0
        self.scheme, self.face_mean, self.picard_max_it, self.picard_tol = 0, 0, 50, 1.0e-6
        self.rain_rate, self.rain_until, self.picard_dt_adapt = 0.0, 0.0, 0
        self.picard_dh_max = 0.0
        self.picard_fp64 = -1  # float-float with the mixed-precision solve, else FP64
        for k, v in kw.items():
            if k == "bc_type":
                self.bc_type[:] = list(v)
            else:
                setattr(self, k, v)

    def copy(self, **kw):
        p = ReParams()
        C.pointer(p)[0] = self
        for k, v in kw.items():
            if k == "bc_type":
                p.bc_type[:] = list(v)
            else:
                setattr(p, k, v)
        return p


class SolverConfig(C.Structure):
    """struct SolverConfig (include/frehg2/linear/SolverConfig.hpp:14-20) plus precision keys."""

    _fields_ = [
        ("ksp_type", C.c_char * 16),
        ("pc_type", C.c_char * 16),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("max_it", C.c_int32),
        ("precision", C.c_int32),
        ("ir_rtol", C.c_double),
        ("inner_rtol", C.c_double),
    ]

    def __init__(self, ksp_type="cg", pc_type="jacobi", rtol=1e-8, atol=1e-50, max_it=10000,
                 precision=0, ir_rtol=1e-10, inner_rtol=1e-4):
        super().__init__()
        self.ksp_type = ksp_type.encode()
        self.pc_type = pc_type.encode()
        self.rtol, self.atol, self.max_it = rtol, atol, max_it
        self.precision, self.ir_rtol, self.inner_rtol = precision, ir_rtol, inner_rtol


class ReCounters(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("cells_touched", C.c_int64),
        ("ksp_iterations", C.c_int64),
        ("picard_iterations", C.c_int64),
        ("realloc_sweeps", C.c_int64),
        ("last_ksp_iterations", C.c_int32),
        ("last_picard_iterations", C.c_int32),
        ("last_residual_norm", C.c_double),
        ("kernel_launches", C.c_int64),
        ("ir_sweeps", C.c_int64),
        ("fcg_fallbacks", C.c_int64),
        ("elastic_volume", C.c_double),
        ("net_solves", C.c_int64),
        ("net_skipped", C.c_int64),
        ("net_ms", C.c_double),
        ("plain_ms", C.c_double),
    ]


class KernelStat(C.Structure):
    _fields_ = [
        ("name", C.c_char * 32),
        ("launches", C.c_int64),
        ("total_ms", C.c_double),
        ("bytes_per_launch", C.c_double),
        ("idle_launches", C.c_int64),
    ]


# ---------------------------------------------------------------------------------------------
# library loading

_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)
_PI32 = C.POINTER(C.c_int32)
_VP = C.c_void_p

# name -> (restype, argtypes); the exact list of symbols include/frehg_gb300.h declares
SIGNATURES = {
    "frehg_last_error": (C.c_char_p, []),
    "frehg_soil_params_default": (None, [C.POINTER(SoilParams)]),
    "frehg_re_params_default": (None, [C.POINTER(ReParams)]),
    "frehg_solver_config_default": (None, [C.POINTER(SolverConfig)]),
    "frehg_re_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(ReParams), C.POINTER(_VP)]),
    "frehg_re_destroy": (C.c_int, [_VP]),
    "frehg_re_set_params": (C.c_int, [_VP, C.POINTER(ReParams)]),
    "frehg_re_get_params": (C.c_int, [_VP, C.POINTER(ReParams)]),
    "frehg_re_set_soil_map": (C.c_int, [_VP, C.POINTER(SoilParams), C.c_int, _PI32, C.c_int]),
    "frehg_re_set_cell_fields": (C.c_int, [_VP, _PD, _PD]),
    "frehg_re_attach_solver": (C.c_int, [_VP, C.POINTER(SolverConfig)]),
    "frehg_re_initialize_geometry": (C.c_int, [_VP]),
    "frehg_re_set_initial_head": (C.c_int, [_VP, _PD]),
    "frehg_re_set_initial_water_content": (C.c_int, [_VP, _PD]),
    "frehg_re_finalize_initial_state": (C.c_int, [_VP]),
    "frehg_re_initialize_uniform_column": (C.c_int, [_VP, C.c_double]),
    "frehg_re_set_top_flux_field": (C.c_int, [_VP, _PD]),
    "frehg_re_advance_step": (C.c_int, [_VP]),
    "frehg_re_advance_steps": (C.c_int, [_VP, C.c_int]),
    "frehg_re_dt": (C.c_int, [_VP, _PD]),
    "frehg_re_dt_used": (C.c_int, [_VP, _PD]),
    "frehg_re_set_dt": (C.c_int, [_VP, C.c_double]),
    "frehg_re_prime_adaptive_dt": (C.c_int, [_VP, C.c_double]),
    "frehg_re_time": (C.c_int, [_VP, _PD]),
    "frehg_re_get_field": (C.c_int, [_VP, C.c_char_p, _PD]),
    "frehg_re_get_interior": (C.c_int, [_VP, C.c_char_p, _PD, C.c_int]),
    "frehg_re_get_interior_async": (C.c_int, [_VP, C.c_char_p, _PD]),
    "frehg_re_get_counters": (C.c_int, [_VP, C.POINTER(ReCounters)]),
    "frehg_re_water_volume": (C.c_int, [_VP, _PD]),
    "frehg_re_boundary_volumes": (C.c_int, [_VP, _PD, _PD]),
    "frehg_re_set_profiling": (C.c_int, [_VP, C.c_int]),
    "frehg_re_kernel_stats": (C.c_int, [_VP, C.POINTER(KernelStat), C.c_int, _PI]),
    "frehg_re_set_stream": (C.c_int, [_VP, _VP]),
    "frehg_re_sync": (C.c_int, [_VP]),
    "frehg_cg_create": (C.c_int, [C.POINTER(SolverConfig), C.POINTER(_VP)]),
    "frehg_cg_destroy": (C.c_int, [_VP]),
    "frehg_system_create": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.POINTER(_VP)]),
    "frehg_system_destroy": (C.c_int, [_VP]),
    "frehg_system_zero_entries": (C.c_int, [_VP]),
    "frehg_system_begin_assembly": (C.c_int, [_VP]),
    "frehg_system_end_assembly": (C.c_int, [_VP]),
    "frehg_system_add_row": (C.c_int, [_VP, C.c_int, C.c_int, _PI, _PD]),
    "frehg_system_add_coo": (C.c_int, [_VP, _PI, _PI, _PD, C.c_int64, C.c_int]),
    "frehg_system_set_rhs": (C.c_int, [_VP, _PD, C.c_int]),
    "frehg_system_get_solution": (C.c_int, [_VP, _PD, C.c_int]),
    "frehg_cg_setup": (C.c_int, [_VP, _VP]),
    "frehg_cg_solve": (C.c_int, [_VP, _VP, _PD, _PD, C.c_int]),
    "frehg_cg_iteration_count": (C.c_int, [_VP, _PI]),
    "frehg_cg_residual_norm": (C.c_int, [_VP, _PD]),
    "frehg_cg_converged_reason": (C.c_int, [_VP, _PI]),
    "frehg_cg_set_fused_iteration": (C.c_int, [_VP, C.c_int]),
    "frehg_check_grid_barrier": (C.c_int, [C.c_int, C.c_longlong, _PI]),
    "frehg_cg_solve_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, _VP, _VP, _VP, _VP, _VP,
                                         _VP, C.POINTER(SolverConfig), _VP, _PI, _PD]),
    "frehg_unet_create": (C.c_int, [C.c_uint64, C.POINTER(_VP)]),
    "frehg_unet_destroy": (C.c_int, [_VP]),
    "frehg_unet_num_params": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "frehg_unet_get_params": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "frehg_unet_set_params": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "frehg_unet_set_input_scaling": (C.c_int, [_VP, C.c_float, C.c_float, C.c_float]),
    "frehg_unet_forward": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, _VP, _VP, _VP, _VP, _VP]),
    "frehg_unet_loss_grad": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, _VP, _VP, _VP, _VP, _PD,
                                       C.POINTER(C.c_float), _VP]),
    "frehg_unet_set_loss_weight": (C.c_int, [_VP, C.c_float]),
    "frehg_unet_adam_step": (C.c_int, [_VP, C.c_float, C.c_float, C.c_float, C.c_float, _VP]),
    "frehg_unet_flops": (C.c_int, [C.c_int, C.c_int, C.c_int, _PD]),
    "frehg_re_attach_unet": (C.c_int, [_VP, _VP]),
    "frehg_re_set_learned_policy": (C.c_int, [_VP, C.c_int, C.c_double]),
    "frehg_re_set_assembly_staging": (C.c_int, [_VP, C.c_int]),
    "frehg_re_set_fused_iteration": (C.c_int, [_VP, C.c_int]),
    "frehg_re_training_pairs": (C.c_int, [_VP, C.c_int, _PI, C.c_int, _VP, _VP, _VP, _VP]),
    "frehg_build_arch": (C.c_int, []),
    "frehg_re_checkpoint": (C.c_int, [_VP, _VP, _VP, _VP]),
    "frehg_re_surface_exchange": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_double, C.c_double,
                                            _VP, _VP, C.c_int]),
    "frehg_re_restart": (C.c_int, [_VP, _VP, _VP, _VP]),
    "frehg_fastmath_eval": (C.c_int, [C.c_int, _VP, _VP, C.c_int64]),
    "frehg_constit_eval": (C.c_int, [_VP, C.c_int, C.c_int, _VP, C.c_int64, _VP, _VP, _VP]),
    "frehg_re_check_staged_assembly": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "frehg_re_check_staged_wait": (C.c_int, [_VP, _PI]),
    "frehg_unet_conv_check": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}

_lib = None


def load_library(path: str | None = None):
    """Load (once) and return the CUDA library with every declared symbol bound.

    Raises RuntimeError when the library has not been built or cannot be loaded: the package
    has no CPU path to fall back on.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"frehg_gb300 CUDA library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    try:
        lib = C.CDLL(p, mode=C.RTLD_GLOBAL)
    except OSError as e:  # pragma: no cover - depends on the machine
        raise RuntimeError(f"cannot load {p}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError = a declared symbol is not exported
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class FrehgError(RuntimeError):
    """Non-zero status from the C ABI (the reference throws std::runtime_error)."""

    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(code: int, where: str):
    if code != FREHG_OK:
        lib = load_library()
        msg = lib.frehg_last_error() or b""
        raise FrehgError(code, where, msg.decode(errors="replace"))


def dptr(a):
    """double* of a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_PD)
