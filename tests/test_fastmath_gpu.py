"""The library's FP64 exp / log / log1p / expm1 (table-driven, used by the van Genuchten
kernels) against the CUDA math library on the same GPU and against the host's libm (numpy):
at most 2 ulp apart over wide argument ranges and special values (zero, subnormals, infinities,
NaN, arguments next to 1 and to the overflow / underflow limits)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ["exp", "log", "log1p", "expm1"]


def ulp_diff(a, b):
    """distance in units in the last place between doubles of equal sign (NaN == NaN)"""
    with np.errstate(over="ignore"):
        d = np.abs(a.view(np.int64) - b.view(np.int64)).astype(np.float64)  # exact in int64
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    d[same] = 0.0
    d[(np.signbit(a) != np.signbit(b)) & ~same] = np.inf
    return d


def samples(name, rng):
    n = 400_000
    if name == "exp":
        x = np.concatenate([rng.uniform(-745.2, 709.8, n), rng.uniform(-1, 1, n) * 1e-3,
                            rng.uniform(-40, 5, n)])
        sp = [0.0, -0.0, 1e-300, -1e-20, 709.78, 709.79, -708.5, -720.0, -745.1, -746.0,
              np.inf, -np.inf, np.nan, 0.5 * np.log(2), -np.log(2)]
    elif name == "log":
        x = np.concatenate([10.0 ** rng.uniform(-323, 308, n), 1.0 + rng.uniform(-0.02, 0.02, n),
                            rng.uniform(0.5, 2.0, n)])
        sp = [0.0, 5e-324, 1e-310, 1.0, 1.0 + 2**-52, 1.0 - 2**-53, 2.0, 0.5, np.inf, np.nan,
              -1.0, 1.7976931348623157e308]
    elif name == "log1p":
        x = np.concatenate([10.0 ** rng.uniform(-20, 300, n), -rng.uniform(0, 0.99, n),
                            rng.uniform(-0.02, 0.02, n)])
        sp = [0.0, 1e-300, 2**-6, -2**-6, 1e300, 1e305, np.inf, np.nan]
    else:
        x = np.concatenate([rng.uniform(-50, 50, n), rng.uniform(-0.02, 0.02, n),
                            -(10.0 ** rng.uniform(-16, 1, n)), rng.uniform(-1, 1, n)])
        sp = [0.0, 1e-300, -1e-300, 2**-6, -2**-6, np.log(2), -np.log(2), 700.0, -800.0,
              np.inf, -np.inf, np.nan]
    return np.ascontiguousarray(np.concatenate([x, np.array(sp)]), dtype=np.float64)


@pytest.mark.parametrize("fn", range(4))
def test_fastmath_against_cuda_and_libm(gpu_lib, fn):
    rng = np.random.default_rng(7 + fn)
    x = samples(NAMES[fn], rng)
    ours = np.empty_like(x)
    cuda = np.empty_like(x)
    P = C.c_void_p
    assert gpu_lib.frehg_fastmath_eval(fn, P(x.ctypes.data), P(ours.ctypes.data), x.size) == 0
    assert gpu_lib.frehg_fastmath_eval(fn + 4, P(x.ctypes.data), P(cuda.ctypes.data),
                                       x.size) == 0
    with np.errstate(all="ignore"):
        host = getattr(np, NAMES[fn])(x)
    d_cuda = ulp_diff(ours, cuda)
    d_host = ulp_diff(ours, host)
    print(f"\n  {NAMES[fn]}: max ulp vs CUDA {d_cuda.max():.0f}, vs libm {d_host.max():.0f}, "
          f"mean vs libm {d_host.mean():.3f} over {x.size} arguments")
    worst = np.argmax(d_cuda)
    assert d_cuda.max() <= 2, (x[worst], ours[worst], cuda[worst])
    assert d_host.max() <= 2
