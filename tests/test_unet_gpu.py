"""The U-Net kernels on the GPU against the numpy statement (oracle/unet_ref.py): forward output,
loss and every parameter gradient, with BF16 rounding emulated at the GPU's storage points.
Also: Adam steps lower the loss, and the FLOP count of one application."""
import ctypes as C

import numpy as np
import pytest

from oracle import unet_ref as U

pytestmark = pytest.mark.gpu


def net_with(lib, params):
    h = C.c_void_p()
    assert lib.frehg_unet_create(1, C.byref(h)) == 0
    n = C.c_int64()
    lib.frehg_unet_num_params(h, C.byref(n))
    assert n.value == params.size
    p32 = np.ascontiguousarray(params, dtype=np.float32)
    assert lib.frehg_unet_set_params(h, p32.ctypes.data_as(C.POINTER(C.c_float))) == 0
    return h


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("shape", [(8, 8, 8), (4, 12, 16)])
def test_forward_and_gradients_match_reference(gpu_lib, shape):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    r = rng.standard_normal(shape).astype(np.float32)
    lnk = rng.standard_normal(shape).astype(np.float32)
    cap = rng.uniform(0, 1, shape).astype(np.float32)
    tgt = rng.standard_normal(shape).astype(np.float32)
    params = U.init_params(5)
    h = net_with(gpu_lib, params)
    nz, ny, nx = shape
    tr, tk, tc, tt = dev(torch, r), dev(torch, lnk), dev(torch, cap), dev(torch, tgt)
    y = torch.empty_like(tr)
    assert gpu_lib.frehg_unet_forward(h, nx, ny, nz, tr.data_ptr(), tk.data_ptr(), tc.data_ptr(),
                                      y.data_ptr(), None) == 0
    yref, _, rms = U.forward(params, r, lnk, cap)
    yg = y.cpu().numpy()
    err = np.abs(yg - yref * rms).max() / np.abs(yref * rms).max()
    print(f"\n  forward {shape}: max error {err:.2e} of the output's maximum")
    # the statement rounds to BF16 where the GPU stores BF16; what remains is the order of the
    # FP32 accumulations and BF16 ties (a few BF16 ulps, 2^-8 each, of a layer's inputs)
    assert err <= 8e-3
    loss = C.c_double()
    g = np.zeros(params.size, dtype=np.float32)
    assert gpu_lib.frehg_unet_loss_grad(h, nx, ny, nz, tr.data_ptr(), tk.data_ptr(),
                                        tc.data_ptr(), tt.data_ptr(), C.byref(loss),
                                        g.ctypes.data_as(C.POINTER(C.c_float)), None) == 0
    lref, gref = U.loss_grad(params, r, lnk, cap, tgt)
    assert abs(loss.value - lref) <= 1e-3 * abs(lref)
    woff, boff, ooff, ntot = U.layout()
    cos = float(g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)))
    assert cos > 0.999, cos
    for l in range(10):
        a = g[woff[l]:boff[l]]
        b = gref[woff[l]:boff[l]]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-12, l
    gpu_lib.frehg_unet_destroy(h)


# (cin, cout, in_stride, in_off, out_stride, out_off): every convolution shape of the network,
# forward and data gradient, with the channel slices of its concatenations
CONV_SHAPES = [(16, 16, 16, 0, 16, 0), (16, 16, 48, 32, 48, 32), (16, 32, 16, 0, 32, 0),
               (32, 32, 96, 64, 96, 64), (32, 64, 32, 0, 64, 0), (64, 64, 64, 0, 64, 0),
               (96, 32, 96, 0, 32, 0), (48, 16, 48, 0, 16, 0), (16, 48, 16, 0, 48, 0),
               (32, 96, 32, 0, 96, 0), (64, 32, 64, 0, 32, 0), (32, 16, 32, 0, 16, 0)]


@pytest.mark.parametrize("grid", [(136, 3, 2), (20, 5, 4), (256, 2, 1), (40, 3, 37)])
@pytest.mark.parametrize("shape", CONV_SHAPES)
def test_tensor_core_conv_matches_mma_sync(gpu_lib, shape, grid):
    """The tcgen05 convolution (TMEM accumulators, shared-memory operand descriptors) against
    the warp-level mma.sync one on the same BF16 inputs: the FP32 sums differ only in order, so
    the BF16 outputs agree to a rounding step (2^-8 relative) of the output scale.  Grids with a
    partial 128-pixel tile, rows shorter than a tile and single planes."""
    cin, cout, ins, ino, outs, outo = shape
    nx, ny, nz = grid
    diff, ref = C.c_double(), C.c_double()
    rc = gpu_lib.frehg_unet_conv_check(cin, cout, ins, ino, outs, outo, nx, ny, nz, 1, 17,
                                       C.byref(diff), C.byref(ref))
    assert rc == 0, gpu_lib.frehg_last_error()
    assert ref.value > 0.0
    assert diff.value <= 2.0 ** -7 * ref.value, (diff.value, ref.value)


def test_adam_lowers_the_loss(gpu_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    shape = (8, 16, 16)
    r = rng.standard_normal(shape).astype(np.float32)
    lnk = np.zeros(shape, np.float32)
    cap = np.zeros(shape, np.float32)
    tgt = (0.5 * r + 0.1).astype(np.float32)
    h = C.c_void_p()
    assert gpu_lib.frehg_unet_create(3, C.byref(h)) == 0
    tr, tk, tc, tt = dev(torch, r), dev(torch, lnk), dev(torch, cap), dev(torch, tgt)
    losses = []
    for it in range(60):
        loss = C.c_double()
        assert gpu_lib.frehg_unet_loss_grad(h, 16, 16, 8, tr.data_ptr(), tk.data_ptr(),
                                            tc.data_ptr(), tt.data_ptr(), C.byref(loss), None,
                                            None) == 0
        losses.append(loss.value)
        assert gpu_lib.frehg_unet_adam_step(h, 1e-3, 0.9, 0.999, 1e-8, None) == 0
    assert losses[-1] < 0.5 * losses[0], losses[::10]
    gpu_lib.frehg_unet_destroy(h)


def test_adam_matches_numpy(gpu_lib):
    """Three Adam steps on the GPU's own gradients against the same update in numpy (FP32):
    m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2, w -= lr (m/(1-b1^t)) / (sqrt(v/(1-b2^t)) + eps)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    shape = (8, 16, 16)
    r = rng.standard_normal(shape).astype(np.float32)
    lnk = rng.standard_normal(shape).astype(np.float32)
    cap = rng.uniform(0, 1, shape).astype(np.float32)
    tgt = rng.standard_normal(shape).astype(np.float32)
    params = U.init_params(8).astype(np.float32)
    h = net_with(gpu_lib, params)
    tr, tk, tc, tt = dev(torch, r), dev(torch, lnk), dev(torch, cap), dev(torch, tgt)
    lr, b1, b2, eps = np.float32(1e-3), np.float32(0.9), np.float32(0.999), np.float32(1e-8)
    w = params.copy()
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    for t in range(1, 4):
        loss = C.c_double()
        g = np.zeros(w.size, dtype=np.float32)
        assert gpu_lib.frehg_unet_loss_grad(h, 16, 16, 8, tr.data_ptr(), tk.data_ptr(),
                                            tc.data_ptr(), tt.data_ptr(), C.byref(loss),
                                            g.ctypes.data_as(C.POINTER(C.c_float)), None) == 0
        assert gpu_lib.frehg_unet_adam_step(h, float(lr), float(b1), float(b2), float(eps),
                                            None) == 0
        m = b1 * m + (np.float32(1) - b1) * g
        v = b2 * v + (np.float32(1) - b2) * g * g
        c1 = np.float32(1) - np.float32(b1 ** t)
        c2 = np.float32(1) - np.float32(b2 ** t)
        w = w - lr * (m / c1) / (np.sqrt(v / c2) + eps)
        got = np.empty_like(w)
        assert gpu_lib.frehg_unet_get_params(h, got.ctypes.data_as(C.POINTER(C.c_float))) == 0
        step = np.abs(w - params).max()
        assert np.abs(got - w).max() <= 1e-3 * step + 1e-9, (t, np.abs(got - w).max(), step)
    gpu_lib.frehg_unet_destroy(h)


def test_flop_count(gpu_lib):
    f = C.c_double()
    assert gpu_lib.frehg_unet_flops(256, 256, 128, C.byref(f)) == 0
    n = 256 * 256 * 128
    per_cell = f.value / n
    assert 1.0e5 < per_cell < 2.0e5
