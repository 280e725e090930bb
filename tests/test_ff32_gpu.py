"""Float-float arithmetic on the FP32 pipe (frehg_gb300/csrc/ff32.cuh) and the Picard
constitutive relations built on it (vg_constit_ff), on the GPU.

The float-float functions are compared with the host's libm (numpy, FP64) over the argument
ranges the van Genuchten kernels produce and their edges; the constitutive relations with the
library's FP64 forms (themselves within 2 ulp of libm, tests/test_fastmath_gpu.py) at heads
from -1e3 m to saturation for the benchmark soils.  Bounds are in units of 2^-48 (u^2, the
precision of a float-float value) and stated per check."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U2 = 2.0 ** -48


def ff_eval(lib, fn, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    assert lib.frehg_fastmath_eval(fn, C.c_void_p(x.ctypes.data), C.c_void_p(y.ctypes.data),
                                   x.size) == 0
    return y


def rel(a, b):
    with np.errstate(all="ignore"):
        return np.abs(a - b) / np.abs(b)


def test_split_and_reciprocal(gpu_lib):
    rng = np.random.default_rng(3)
    x = np.concatenate([10.0 ** rng.uniform(-29, 37, 200_000), -(10.0 ** rng.uniform(-29, 37, 1000)),
                        [1.0, -1.0, 2.0 ** -100, 3.0e38]])
    back = ff_eval(gpu_lib, 12, x)
    e = rel(back, x).max()
    print(f"\n  double -> float-float -> double: max rel {e:.2e} ({e / U2:.2f} u^2)")
    assert e <= 2.0 * U2
    # outside the integer-split range: zero, tiny, huge, inf, NaN take the conversions
    sp = np.array([0.0, -0.0, 1e-35, 1e-300, np.inf, -np.inf, np.nan])
    got = ff_eval(gpu_lib, 12, sp)
    assert got[0] == 0.0 and got[1] == 0.0 and np.isinf(got[4]) and np.isinf(got[5])
    assert np.isnan(got[6]) and abs(got[2] - 1e-35) <= 1e-35 * 1e-6
    # reciprocal, results above 2^-100 (the low part of smaller results goes subnormal)
    x = x[(np.abs(x) < 1e29) & (np.abs(x) > 1e-29)]
    r = ff_eval(gpu_lib, 13, x)
    e = rel(r, 1.0 / ff_eval(gpu_lib, 12, x)).max()
    print(f"  float-float reciprocal: max rel {e:.2e} ({e / U2:.2f} u^2)")
    assert e <= 16.0 * U2


def test_elementary_functions(gpu_lib):
    """Each function against libm at the float-float value of its argument (the argument's split
    from a double rounds it to ~48 bits, which exp amplifies by |x|)."""
    rng = np.random.default_rng(11)
    n = 300_000

    def run(fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return ff_eval(gpu_lib, fn, x), ff_eval(gpu_lib, 12, x)

    # exp: relative error while the result's low part is a normal float (x >= -70)
    y, xs = run(8, np.concatenate([rng.uniform(-70, 88, n), rng.uniform(-0.01, 0.01, n),
                                   rng.uniform(-60, 10, n), [0.0, -70.0, 88.0,
                                                             np.log(2) / 256]]))
    e_exp = rel(y, np.exp(xs)).max()
    # below, the low part goes subnormal: the float-float value degrades towards a float's
    y, xs = run(8, rng.uniform(-87, -70, n))
    e_exp_tail = rel(y, np.exp(xs)).max()
    # log: absolute error (the kernels feed every logarithm into an exponential)
    y, xs = run(9, np.concatenate([10.0 ** rng.uniform(-30, 30, n), 1.0 + rng.uniform(-0.01, 0.01, n),
                                   rng.uniform(0.5, 2.0, n), [1.0, 2.0, 0.5, 1.0 + 2.0 ** -30]]))
    e_log = (np.abs(y - np.log(xs)) / np.maximum(1.0, np.abs(np.log(xs)))).max()
    # log1p: absolute error
    y, xs = run(10, np.concatenate([10.0 ** rng.uniform(-30, 30, n), rng.uniform(0, 0.01, n),
                                    [0.0, 2.0 ** -9, 2.0 ** -9 * (1 + 2.0 ** -20)]]))
    e_l1p = (np.abs(y - np.log1p(xs)) / np.maximum(1.0, np.log1p(xs))).max()
    # expm1: relative error
    y, xs = run(11, np.concatenate([-(10.0 ** rng.uniform(-20, 1.7, n)), rng.uniform(-1, 0.69, n),
                                    rng.uniform(-0.01, 0.01, n),
                                    [0.0027, -0.0027, 0.6931, -0.6931, -50.0]]))
    with np.errstate(all="ignore"):
        r_em1 = rel(y, np.expm1(xs))
        e_em1 = np.nanmax(r_em1)
    w = np.nanargmax(r_em1)
    print(f"\n  expm1 worst at x = {xs[w]!r}: {y[w]!r} vs {np.expm1(xs[w])!r}")
    print(f"\n  float-float exp {e_exp / U2:.1f} u^2 (rel; x in [-87, -70]: {e_exp_tail:.1e}), "
          f"log {e_log / U2:.1f} u^2 (abs), log1p {e_l1p / U2:.1f} u^2 (abs), "
          f"expm1 {e_em1 / U2:.1f} u^2 (rel)")
    assert e_exp <= 16 * U2
    assert e_exp_tail <= 2.0 ** -20
    assert e_log <= 16 * U2
    assert e_l1p <= 16 * U2
    assert e_em1 <= 16 * U2
    # special values
    sp = ff_eval(gpu_lib, 9, np.array([0.0, np.inf, np.nan, -1.0]))
    assert sp[0] == -np.inf and sp[1] == np.inf and np.isnan(sp[2]) and np.isnan(sp[3])
    sp = ff_eval(gpu_lib, 8, np.array([-200.0, 100.0, np.nan, -np.inf]))
    assert sp[0] == 0.0 and sp[1] == np.inf and np.isnan(sp[2]) and sp[3] == 0.0


def vg_reference(s, h):
    """K/Ks, theta, C of the continuous-theta van Genuchten relations in host FP64 (numpy), with
    (1 - se^{1/m})^m from ln(1 + 1/t) for t > 1 so that dry cells keep their relative accuracy"""
    m = 1.0 - 1.0 / s.n
    with np.errstate(all="ignore"):
        ah = np.abs(s.alpha * h)
        nL = s.n * np.log(ah)
        t = np.exp(nL)
        v = np.log1p(1.0 / t)
        dry = t > 1.0
        u = np.where(dry, nL + v, np.log1p(t))
        y = np.where(dry, -m * v, m * (nL - u))
        se_half = np.exp(-0.5 * m * u)
        kr = np.minimum(se_half * np.expm1(y) ** 2, 1.0)
        se = se_half * se_half
        wc = s.theta_r + (s.theta_s - s.theta_r) * se
        cap = s.alpha * s.n * m * (s.theta_s - s.theta_r) * t * se / (ah * (1.0 + t))
    sat = h >= 0
    kr[sat], wc[sat], cap[sat] = 1.0, s.theta_s, 0.0
    return kr, np.minimum(wc, s.theta_s), cap


@pytest.mark.parametrize("name", ["loam", "sand", "clay"])
def test_constitutive_ff(gpu_lib, name):
    """The float-float relations against a host FP64 statement of the same relations (relative
    accuracy of K kept in dry cells), and against the library's FP64 forms (which agree with
    the oracle to a few ulp and lose about log10(t) digits of K in dry cells)."""
    from frehg_gb300 import workloads as W
    s = W.soil(getattr(W, name.upper()))
    rng = np.random.default_rng(5)
    h = np.concatenate([-(10.0 ** rng.uniform(-12, 3, 400_000)), [0.0, 1e-3, 2.0, -1e-300],
                        -np.linspace(0, 0.05, 1001)])
    out = {}
    for arith in (0, 1):
        kr, wc, cap = (np.empty_like(h) for _ in range(3))
        P = C.c_void_p
        assert gpu_lib.frehg_constit_eval(C.byref(s), arith, 1, P(h.ctypes.data), h.size,
                                          P(kr.ctypes.data), P(wc.ctypes.data),
                                          P(cap.ctypes.data)) == 0
        out[arith] = (kr, wc, cap)
    (k0, w0, c0), (k1, w1, c1) = out[0], out[1]
    kref, wref, cref = vg_reference(s, h)
    live = kref > 1e-300
    e_kr = rel(k1[live], kref[live]).max()
    e_wc = np.abs(w1 - wref).max()
    cb = cref > 1e-30
    e_c = rel(c1[cb], cref[cb]).max()
    wet = live & (np.abs(s.alpha * h) < 1.0)
    e_kr64 = rel(k0[live], kref[live]).max()
    print(f"\n  {name}: float-float vs host FP64: K {e_kr:.2e} (rel), theta {e_wc:.2e} (abs), "
          f"C {e_c:.2e} (rel); FP64 forms: K {e_kr64:.2e} (rel; wet cells "
          f"{rel(k0[wet], kref[wet]).max():.2e}), theta {np.abs(w0 - wref).max():.2e}")
    # saturated and h >= 0 branches are exact
    sat = h >= 0
    assert np.all(k1[sat] == 1.0) and np.all(w1[sat] == w0[sat]) and np.all(c1[sat] == 0.0)
    assert np.all(w1 <= s.theta_s) and np.all(w1 >= s.theta_r)
    assert e_wc <= 64 * U2
    # t = e^{n ln|alpha h|} carries the argument's absolute error |n ln|alpha h|| u^2 as a
    # relative error; K inherits it (about 1e-12 at |alpha h| = 1e3).  C is formed in FP32
    # (it enters only the FP32 matrix diagonal of the float-float Picard path).
    assert e_kr <= 1e-11
    assert e_c <= 1e-6
    # in wet cells the two device forms agree to float-float precision
    assert rel(k1[wet], k0[wet]).max() <= 1e-12
