"""The learned preconditioner end to end on the GPU: pairs from the plain solver, training with
the library's own forward/backward/Adam kernels, and flexible CG under FP64 refinement.

What the trained network gains over the method without it is measured, not assumed: the test
prints the held-out loss before and after training and the inner iterations and solve times of
line-PCG (the same refinement without the network) and of network-preconditioned FCG
(z = M_line^-1 r + NN(r)).  It checks that the training kernels fit a pair (the loss of a single
pair falls under repeated Adam steps), that both solvers reach the heads of the plain FP64
Jacobi-PCG run (the network changes the iteration count, not the accuracy), that the iteration
fallback bounds a solve, and that the time policy runs the network only on its probe solves
when it does not pay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)


@pytest.fixture(scope="module")
def trained():
    pytest.importorskip("torch")
    from frehg_gb300 import learned as Lr
    data = Lr.generate_pairs(list(range(100, 106)), *SHAPE, snapshots=(0, 2),
                             iters=(0, 2, 5, 10, 20), pc="unet-line")
    held = Lr.generate_pairs([99], *SHAPE, snapshots=(1,), iters=(0, 2, 5, 10, 20),
                             pc="unet-line")
    net = Lr.UNet(0)
    net.set_scaling(*Lr.input_scaling(data))

    def held_loss():
        return sum(Lr.pair_loss(net, held, q) for q in range(held["r"].shape[0])) / \
            held["r"].shape[0]

    before = held_loss()
    Lr.train(net, data, steps=300, lr=1e-3)
    after = held_loss()
    return net, before, after


def run(pc, net=None, precision=1, steps=3, policy=None):
    """3 steps of the 32^3 heterogeneous-loam infiltration (the benchmark's GRF generator);
    its conditioning lets FP64 Jacobi-PCG at rtol 1e-12 serve as the 1e-8 m head reference"""
    from frehg_gb300 import workloads as W
    from frehg_gb300.abi import SolverConfig, check
    from frehg_gb300.re_solver import Grid, ReSolver
    w = W.config1("pca", *SHAPE, steps=steps)
    w.solver = SolverConfig("cg", pc, rtol=1e-12, max_it=20000, precision=precision,
                            ir_rtol=1e-12)
    g = ReSolver(Grid(*SHAPE, 1.0, 1.0, 0.05), w.params)
    w.apply(g)
    if net is not None:
        check(g._lib.frehg_re_attach_unet(g._h, net.handle), "attach_unet")
        if policy is not None:
            check(g._lib.frehg_re_set_learned_policy(g._h, *policy), "policy")
    its, heads, falls = [], [], []
    for _ in range(steps):
        c0 = g.counters()
        g.advance_step()
        c1 = g.counters()
        its.append(c1.ksp_iterations - c0.ksp_iterations)
        falls.append(c1.fcg_fallbacks - c0.fcg_fallbacks)
        heads.append(g.interior("h").copy())
    run.fallbacks = falls
    return its, heads, g.counters()


def test_training_fits_a_pair(gpu_lib, trained):
    """Repeated Adam steps on one pair drive its relative loss down (the forward, backward and
    Adam kernels learn); the held-out loss of the trained network is reported."""
    from frehg_gb300 import learned as Lr
    net, before, after = trained
    print(f"\n  held-out relative loss {before:.3e} -> {after:.3e} after 300 Adam steps")
    data = Lr.generate_pairs([100], *SHAPE, snapshots=(0,), iters=(5,), pc="unet-line")
    one = Lr.UNet(3)
    one.set_scaling(*Lr.input_scaling(data))
    l0 = Lr.pair_loss(one, data, 0)
    hist = Lr.train(one, data, steps=200, lr=1e-3)
    l1 = Lr.pair_loss(one, data, 0)
    print(f"  single-pair relative loss {l0:.3e} -> {l1:.3e}")
    assert l1 < 0.5 * l0


def test_learned_fcg_accuracy_and_iterations(gpu_lib, trained):
    net, before, after = trained
    _, h64, _ = run("jacobi", precision=0)
    line, hl, cl = run("line")
    lrn, hn, cn = run("unet-line", net=net, policy=(0, 1.0))
    print(f"\n  inner iterations per step  line-PCG {line}  learned FCG {lrn}  "
          f"(held-out loss {before:.3e} -> {after:.3e}); solve ms: line {cl.plain_ms:.1f}, "
          f"learned {cn.net_ms + cn.plain_ms:.1f} ({cn.net_solves} network solves, "
          f"{cn.fcg_fallbacks} fallbacks)")
    for s, (a, b, c) in enumerate(zip(h64, hl, hn)):
        assert np.abs(a - b).max() <= 1e-8, f"step {s}: line-PCG head {np.abs(a - b).max():.3e}"
        assert np.abs(a - c).max() <= 1e-8, f"step {s}: learned head {np.abs(a - c).max():.3e}"
    # the first solve of the learned handle is its network-free reference solve
    assert lrn[0] == line[0], (lrn, line)
    assert cn.net_solves == len(lrn) - 1, (cn.net_solves, lrn)
    # the switching rule: a network solve whose inner count passes twice the reference count
    # (checked every 4 network iterations and at the start of every refinement sweep) ends its
    # network sweep there and finishes with line-PCG sweeps from that iterate, so a solve either
    # stays within 2 * ref + 3 inner iterations or records a fallback (its total then depends
    # on how far the network got)
    falls = run.fallbacks
    for a, f in zip(lrn[1:], falls[1:]):
        assert a <= 2 * lrn[0] + 3 or f > 0, (lrn, falls)


def test_time_policy(gpu_lib, trained):
    """A ratio nothing can meet keeps the network off (one application already costs more than
    the ratio allows, so not even a probe runs); a ratio everything meets keeps it on after the
    first probe."""
    net, _, _ = trained
    its, _, c = run("unet-line", net=net, steps=6, policy=(4, 1e-9))
    assert c.net_solves == 0
    assert c.net_skipped == len(its) - 1
    its, _, c = run("unet-line", net=net, steps=6, policy=(4, 1e9))
    assert c.net_solves == len(its) - 1
    assert c.net_skipped == 0
