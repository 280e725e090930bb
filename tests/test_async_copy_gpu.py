"""Asynchronous copies of the step's result (frehg_re_get_interior_async, not in reference): each
copy lands the state of the step it follows, bit for bit, although the next steps run while it
is in flight (they write the other state buffer; a call that writes the copied buffer waits for
the copy), and sync() completes them."""
import numpy as np
import pytest

from frehg_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def new(w):
    from frehg_gb300.re_solver import Grid, ReSolver
    g = ReSolver(Grid(w.nx, w.ny, w.nz, w.params.dx, w.params.dy, w.params.dz), w.params)
    w.apply(g)
    return g


def pinned(torch, n, count):
    return [torch.empty(n, dtype=torch.float64).pin_memory().numpy() for _ in range(count)]


@pytest.mark.parametrize("scheme", ["picard", "pca"])
def test_async_copies_hold_each_steps_result(gpu_lib, scheme):
    torch = pytest.importorskip("torch")
    w = W.config1(scheme, nx=24, ny=20, nz=32, steps=6, precision=1)
    w.solver.pc_type = b"line"
    a, b = new(w), new(w)
    n = w.nx * w.ny * w.nz
    hs, ws = pinned(torch, n, w.steps), pinned(torch, n, w.steps)
    ref_h, ref_w = [], []
    for s in range(w.steps):
        a.advance_step()
        ref_h.append(a.interior("h").ravel().copy())
        ref_w.append(a.interior("wc").ravel().copy())
        b.advance_step()
        b.interior_async("h", hs[s])
        b.interior_async("wc", ws[s])
    b.sync()
    for s in range(w.steps):
        assert np.array_equal(hs[s], ref_h[s]), f"step {s}: head copy"
        assert np.array_equal(ws[s], ref_w[s]), f"step {s}: water-content copy"


def test_async_copy_of_previous_state_and_overwrite_order(gpu_lib):
    """hn (the buffer the next step writes) and a copy followed at once by the next step: the
    step waits for the copy of the buffer it overwrites"""
    torch = pytest.importorskip("torch")
    w = W.config1("picard", nx=16, ny=16, nz=24, steps=4, precision=1)
    w.solver.pc_type = b"line"
    a, b = new(w), new(w)
    n = w.nx * w.ny * w.nz
    (hn,), (h2,) = pinned(torch, n, 1), pinned(torch, n, 1)
    for _ in range(2):
        a.advance_step()
        b.advance_step()
    ref_hn = a.interior("hn").ravel().copy()
    b.interior_async("hn", hn)
    a.advance_step()
    a.advance_step()
    b.advance_step()  # writes the buffer hn was copied from: waits for that copy
    b.interior_async("h", h2)
    b.advance_step()
    b.sync()
    assert np.array_equal(hn, ref_hn)
    assert np.array_equal(b.interior("h"), a.interior("h"))
    from frehg_gb300.abi import FrehgError
    with pytest.raises(FrehgError, match="asynchronous"):
        b.interior_async("kr", h2)
