"""The seeded Gaussian-random-field generator of the heterogeneous workloads (frehg_gb300/grf.py):
standardised realisations whose empirical correlation along each axis follows the exponential
covariance exp(-lag / l) of the stated correlation lengths, and ln Ks / ln alpha fields with the
stated standard deviations and cross-correlation (rho 0.7)."""
import math

import numpy as np

from frehg_gb300.grf import exponential_grf, lnk_lnalpha_fields

SHAPE = (64, 128, 128)  # (nz, ny, nx)
CORR = (4.0, 8.0, 8.0)  # (lz, ly, lx) cells, the workloads' lengths


def axis_correlation(f, axis, lag):
    a = np.moveaxis(f, axis, 0)
    return float(np.mean(a[:-lag] * a[lag:]))


def test_moments_and_seeding():
    f = exponential_grf(SHAPE, CORR, seed=1)
    assert abs(f.mean()) < 1e-12 and abs(f.std() - 1.0) < 1e-12
    assert np.array_equal(f, exponential_grf(SHAPE, CORR, seed=1))
    assert not np.array_equal(f, exponential_grf(SHAPE, CORR, seed=2))


def test_exponential_correlation_lengths():
    fields = [exponential_grf(SHAPE, CORR, seed=s) for s in (11, 12, 13, 14)]
    for axis, l in zip((0, 1, 2), CORR):
        for lag in (1, int(l), int(2 * l)):
            rho = np.mean([axis_correlation(f, axis, lag) for f in fields])
            expect = math.exp(-lag / l)
            assert abs(rho - expect) < 0.06, (axis, lag, rho, expect)


def test_lnk_lnalpha_statistics():
    ln_ks, ln_a = lnk_lnalpha_fields(SHAPE, CORR, 1, 2, math.log(2.89e-6), 1.0, math.log(3.6),
                                     0.3, 0.7)
    assert abs(ln_ks.mean() - math.log(2.89e-6)) < 1e-9 and abs(ln_ks.std() - 1.0) < 1e-9
    assert abs(ln_a.mean() - math.log(3.6)) < 0.02
    assert abs(ln_a.std() - 0.3) < 0.02
    rho = np.corrcoef(ln_ks.ravel(), ln_a.ravel())[0, 1]
    assert abs(rho - 0.7) < 0.05, rho
