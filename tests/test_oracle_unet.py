"""The numpy statement of the U-Net (oracle/unet_ref.py) against finite differences, so that it
can serve as the reference for the GPU gradients."""
import numpy as np

from oracle import unet_ref as U


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    shape = (4, 8, 4)
    r = rng.standard_normal(shape)
    lnk = rng.standard_normal(shape)
    cap = rng.uniform(0, 1, shape)
    tgt = rng.standard_normal(shape)
    p = U.init_params(7).astype(np.float64)
    loss, g = U.loss_grad(p, r, lnk, cap, tgt, use_bf16=False)
    woff, boff, ooff, ntot = U.layout()
    picks = [woff[0] + 5, woff[2] + 123, woff[5] + 4000, woff[6] + 77, boff[8] + 3,
             woff[9] + 999, ooff + 4, ooff + 16]
    for k in picks:
        h = 1e-6 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp, _ = U.loss_grad(pp, r, lnk, cap, tgt, use_bf16=False)
        lm, _ = U.loss_grad(pm, r, lnk, cap, tgt, use_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1e-8, abs(fd)) + 1e-10, (k, fd, g[k])


def test_parameter_count():
    woff, boff, ooff, ntot = U.layout()
    live = sum(27 * live * cout + cout for cin, cout, _, live in U.CONVS) + 17
    assert live == 354145
