"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: numpy statement of the learned preconditioner's U-Net
(forward, loss, backward) used to check the GPU kernels' outputs and gradients.

Same architecture, parameter layout and data flow as frehg_gb300/csrc/unet.cu.  With
`bf16=True` every tensor the GPU stores in BF16 (input, activations, weights, data gradients) is
rounded to BF16 (round to nearest even) at the same points, sums are carried in FP64; with
`bf16=False` everything is FP64 (used for the finite-difference check of the backward pass).
"""
from __future__ import annotations

import numpy as np

# (cin, cout, level, live input channels): c1a c1b c2a c2b c3a c3b d2a d2b d1a d1b
CONVS = [(16, 16, 0, 3), (16, 16, 0, 16), (16, 32, 1, 16), (32, 32, 1, 32), (32, 64, 2, 32),
         (64, 64, 2, 64), (96, 32, 1, 96), (32, 32, 1, 32), (48, 16, 0, 48), (16, 16, 0, 16)]


def layout():
    off, woff, boff = 0, [], []
    for cin, cout, _, _ in CONVS:
        woff.append(off)
        off += 27 * cin * cout
        boff.append(off)
        off += cout
    return woff, boff, off, off + 17


def bf16(x):
    """round float array to bfloat16 (nearest even), returned as float64"""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, q):
    woff, boff, ooff, _ = layout()
    Ws, bs = [], []
    for l, (cin, cout, _, _) in enumerate(CONVS):
        W = params[woff[l]:woff[l] + 27 * cin * cout].reshape(27, cout, cin).astype(np.float64)
        Ws.append(q(W))
        bs.append(params[boff[l]:boff[l] + cout].astype(np.float64))
    wo = params[ooff:ooff + 17].astype(np.float64)
    return Ws, bs, wo


def shift(a, dz, dy, dx):
    """b[z,y,x] = a[z+dz, y+dy, x+dx] with zero padding; a is (nz, ny, nx, c)"""
    nz, ny, nx = a.shape[:3]
    b = np.zeros_like(a)
    zs, ze = max(0, -dz), min(nz, nz - dz)
    ys, ye = max(0, -dy), min(ny, ny - dy)
    xs, xe = max(0, -dx), min(nx, nx - dx)
    b[zs:ze, ys:ye, xs:xe] = a[zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return b


TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def conv(x, W, b):
    out = np.zeros(x.shape[:3] + (W.shape[1],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += shift(x, dz, dy, dx) @ W[t].T
    if b is not None:
        out += b
    return out


def conv_data_grad(g, W):
    """d/dx of sum(g * conv(x, W)) = sum_t shift(g, -d_t) @ W[t]"""
    out = np.zeros(g.shape[:3] + (W.shape[2],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += shift(g, -dz, -dy, -dx) @ W[t]
    return out


def conv_weight_grad(x, g):
    cin, cout = x.shape[3], g.shape[3]
    dW = np.zeros((27, cout, cin))
    gf = g.reshape(-1, cout)
    for t, (dz, dy, dx) in enumerate(TAPS):
        dW[t] = gf.T @ shift(x, dz, dy, dx).reshape(-1, cin)
    return dW


def pool(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def up(x):
    return x.repeat(2, 0).repeat(2, 1).repeat(2, 2)


def up_grad(g):
    nz, ny, nx, c = g.shape
    return g.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def pool_grad(g):
    return up(g) / 8.0


def forward(params, r, lnk, cap, kmean=0.0, kscale=1.0, cscale=1.0, use_bf16=True):
    """r, lnk, cap: (nz, ny, nx) arrays.  Returns (y_normalised, cache, rms)."""
    q = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs, wo = unpack(params, q)
    r = np.asarray(r, dtype=np.float64)
    rms = np.sqrt(np.mean(r * r))
    rs = 1.0 / rms if rms > 0 else 1.0
    if use_bf16:
        rs = float(np.float32(rs))
    x0 = np.zeros(r.shape + (16,))
    x0[..., 0] = r * rs
    x0[..., 1] = (lnk - kmean) * kscale
    x0[..., 2] = cap * cscale
    x0 = q(x0)
    relu = lambda a: q(np.maximum(a, 0.0))
    a1 = relu(conv(x0, Ws[0], bs[0]))
    e1 = relu(conv(a1, Ws[1], bs[1]))
    p1 = q(pool(e1))
    a2 = relu(conv(p1, Ws[2], bs[2]))
    e2 = relu(conv(a2, Ws[3], bs[3]))
    p2 = q(pool(e2))
    a3 = relu(conv(p2, Ws[4], bs[4]))
    e3 = relu(conv(a3, Ws[5], bs[5]))
    cat2 = np.concatenate([up(e3), e2], axis=3)
    d2a = relu(conv(cat2, Ws[6], bs[6]))
    d2 = relu(conv(d2a, Ws[7], bs[7]))
    cat1 = np.concatenate([up(d2), e1], axis=3)
    d1a = relu(conv(cat1, Ws[8], bs[8]))
    d1 = relu(conv(d1a, Ws[9], bs[9]))
    y = d1 @ wo[:16] + wo[16]
    cache = dict(x0=x0, a1=a1, e1=e1, p1=p1, a2=a2, e2=e2, p2=p2, a3=a3, e3=e3, cat2=cat2,
                 d2a=d2a, d2=d2, cat1=cat1, d1a=d1a, d1=d1, Ws=Ws, wo=wo, rs=rs, q=q)
    return y, cache, rms


def loss_grad(params, r, lnk, cap, target, use_bf16=True, **scaling):
    """loss = mean((y - target * rs)^2) and the gradient in the flat parameter layout"""
    y, c, _ = forward(params, r, lnk, cap, use_bf16=use_bf16, **scaling)
    q = c["q"]
    n = y.size
    e = y - np.asarray(target, dtype=np.float64) * c["rs"]
    loss = float(np.mean(e * e))
    gy = 2.0 * e / n
    woff, boff, ooff, ntot = layout()
    grad = np.zeros(ntot)
    grad[ooff:ooff + 16] = np.tensordot(gy, c["d1"], axes=3)
    grad[ooff + 16] = gy.sum()
    Ws = c["Ws"]

    def layer(l, x, g, act):
        g = g * (act > 0)
        cin, cout = x.shape[3], g.shape[3]
        grad[woff[l]:woff[l] + 27 * cin * cout] = conv_weight_grad(x, g).ravel()
        grad[boff[l]:boff[l] + cout] = g.sum(axis=(0, 1, 2))
        return g

    g_d1 = q(gy[..., None] * c["wo"][:16])
    g = layer(9, c["d1a"], g_d1, c["d1"])
    g_d1a = q(conv_data_grad(g, Ws[9]))
    g = layer(8, c["cat1"], g_d1a, c["d1a"])
    g_cat1 = q(conv_data_grad(g, Ws[8]))
    g_d2 = q(up_grad(g_cat1[..., :32]))
    g = layer(7, c["d2a"], g_d2, c["d2"])
    g_d2a = q(conv_data_grad(g, Ws[7]))
    g = layer(6, c["cat2"], g_d2a, c["d2a"])
    g_cat2 = q(conv_data_grad(g, Ws[6]))
    g_e3 = q(up_grad(g_cat2[..., :64]))
    g = layer(5, c["a3"], g_e3, c["e3"])
    g_a3 = q(conv_data_grad(g, Ws[5]))
    g = layer(4, c["p2"], g_a3, c["a3"])
    g_p2 = q(conv_data_grad(g, Ws[4]))
    g_e2 = q(g_cat2[..., 64:] + pool_grad(g_p2))
    g = layer(3, c["a2"], g_e2, c["e2"])
    g_a2 = q(conv_data_grad(g, Ws[3]))
    g = layer(2, c["p1"], g_a2, c["a2"])
    g_p1 = q(conv_data_grad(g, Ws[2]))
    g_e1 = q(g_cat1[..., 32:] + pool_grad(g_p1))
    g = layer(1, c["a1"], g_e1, c["e1"])
    g_a1 = q(conv_data_grad(g, Ws[1]))
    layer(0, c["x0"], g_a1, c["a1"])
    # the input layer's padding channels are not trained
    cin, cout = 16, 16
    wg = grad[woff[0]:woff[0] + 27 * cin * cout].reshape(27, cout, cin)
    wg[:, :, 3:] = 0.0
    return loss, grad


def init_params(seed):
    """He-normal weights (numpy generator; independent of the GPU's initialiser)"""
    rng = np.random.default_rng(seed)
    woff, boff, ooff, ntot = layout()
    p = np.zeros(ntot, dtype=np.float32)
    for l, (cin, cout, _, live) in enumerate(CONVS):
        W = rng.standard_normal((27, cout, cin)) * np.sqrt(2.0 / (27 * live))
        W[:, :, live:] = 0.0
        p[woff[l]:woff[l] + W.size] = W.ravel()
        p[boff[l]:boff[l] + cout] = 0.01 * rng.standard_normal(cout)
    p[ooff:ooff + 16] = 0.1 * rng.standard_normal(16)
    p[ooff + 16] = 0.01
    return p
