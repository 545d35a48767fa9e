"""The learned two-level preconditioner (XF_PRECOND_UNET2): the U-Net on the
coarse grid of 4 x 4 x 4 blocks is the coarse solver, the FP32 Chebyshev
passes smooth, and the flexible CG drives both.

Bars: every solve, FP64 or mixed precision (FP32 vectors, FP64 dots),
reaches a true 1e-8 relative residual, recomputed in FP64 by the oracle, and
repeats its iteration count on a second solve; the two-level preconditioner
needs far fewer iterations than
plain and Jacobi FCG; a network trained on another geometry's coarse system
needs under half the iterations of the untrained one and fewer than the
Chebyshev smoother alone; bad networks fall back to plain CG; training is
bit-reproducible; grids that are not block coarsenings of each other are
refused.
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import capi
from xflow_gb300 import workloads as wl

F = 4


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def fine_and_coarse(ctx, n, nsph, seed):
    codes, nrm, _, sep, _ = wl.spheres_grid(n, nsph, 0.02, 0.06, seed)
    b = wl.divergence_rhs(codes, (sep, sep, sep), seed + 1)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    cc, s1, s2, s3 = wl.coarse_grid(codes, sep, F)
    gc = xf.Grid(ctx, cc, s1, s2, s3, None)
    return codes, sep, g, xf.Operator(g), b, gc, xf.Operator(gc)


def test_coarse_grid_is_the_any_active_pooling():
    codes, _, _, sep, _ = wl.spheres_grid(32, 6, 0.02, 0.08, 3)
    cc, s1, _, _ = wl.coarse_grid(codes, sep, F)
    assert cc.shape == (10, 10, 10) and np.allclose(s1, sep[0] * F)
    act = wl.space_mask(codes)[1:-1, 1:-1, 1:-1].astype(bool)
    for I, J, K in [(1, 1, 1), (4, 5, 6), (8, 8, 8), (2, 7, 3)]:
        blk = act[(I - 1) * F:I * F, (J - 1) * F:J * F, (K - 1) * F:K * F]
        assert (cc[I, J, K] == wl.ACTUAL) == blk.any()
    assert not cc[0].any() and not cc[:, -1].any()
    with pytest.raises(ValueError):
        wl.coarse_grid(codes, sep, 5)


@pytest.mark.gpu
def test_two_level_fcg_converges_with_fewer_iterations(ctx):
    # train on the coarse system of one geometry, pairs from plain CG's own iterates
    _, _, _, _, _, gt, At = fine_and_coarse(ctx, 64, 12, 11)
    net = xf.UNet(gt, seed=1)
    rs, es = [], []
    for s in range(3):
        bs = wl.divergence_rhs(np.asarray(gt.codes), (np.full(gt.shape[0] - 1, 1 / 16),) * 3, 300 + s)
        r_, e_ = xf.harvest_pairs(At, gt.vec(bs), iters=(2, 4, 8, 16, 30, 50))
        rs += r_
        es += e_
    for step in range(300):
        q = step % len(rs)
        net.train_step(rs[q], es[q], lr=2e-3, op=At)
    # a fresh geometry at 64^3: the network on its coarse grid
    codes, sep, g, A, b, gc, _ = fine_and_coarse(ctx, 64, 12, 29)
    trained = xf.UNet(gc, net.params())
    fresh = xf.UNet(gc, seed=1)
    bv = g.vec(b)
    og = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
    sm = og.smask.astype(bool)
    its = {}
    for name, kw in (("plain", {}), ("jacobi", {"precond": capi.XF_PRECOND_JACOBI}),
                     ("two_level_untrained", {"unet": fresh, "precond": capi.XF_PRECOND_UNET2}),
                     ("two_level", {"unet": trained, "precond": capi.XF_PRECOND_UNET2}),
                     ("two_level_w2", {"unet": trained, "precond": capi.XF_PRECOND_UNET2, "window": 2}),
                     ("two_level_mixed", {"unet": trained, "precond": capi.XF_PRECOND_UNET2, "window": 2,
                                          "precision": xf.XF_PREC_MIXED}),
                     ("two_level_mixed_deg4", {"unet": trained, "precond": capi.XF_PRECOND_UNET2, "window": 2,
                                               "precision": xf.XF_PREC_MIXED, "degree": 4, "ratio": 30})):
        for rep in range(2):   # a second solve in a row starts from the same state
            x = g.vec(np.zeros(g.shape))
            st = xf.solve_fcg(A, x, bv, rtol=1e-8, **kw)
            assert st.status == capi.XF_OK and st.rel_resid <= 1e-8, (name, st.status, st.rel_resid)
            r = O.apply(O.LAPLACE, og, x.download(), b, -1)
            rel = np.linalg.norm(r[sm]) / np.linalg.norm(b[sm])
            assert rel <= 1.01e-8, (name, rel)
            if rep == 0:
                its[name] = st.iterations
            else:
                assert st.iterations == its[name], (name, st.iterations, its[name])
    # the same smoother without the network: the Chebyshev-preconditioned mixed CG (degree 8, the two-level
    # default's degree)
    x = g.vec(np.zeros(g.shape))
    st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-8, precond=capi.XF_PRECOND_CHEB,
                  cheb_degree=8)
    assert st.status == capi.XF_OK
    its["chebyshev_pcg"] = st.iterations
    print("FCG iterations at 64^3:", its)
    assert its["two_level"] < 0.25 * its["plain"], its
    assert its["two_level"] < 0.5 * its["jacobi"], its
    # what training buys: well under half the iterations of the untrained network, and fewer than the smoother alone
    assert its["two_level"] < 0.5 * its["two_level_untrained"], its
    assert its["two_level"] < its["chebyshev_pcg"], its
    assert its["two_level_mixed"] <= 1.3 * its["two_level_w2"] + 3, its   # FP32 vectors cost few iterations


@pytest.mark.gpu
def test_training_is_deterministic(ctx):
    # the reductions of the training step (sums of squares, weight and bias gradients) are fixed-order:
    # two networks trained alike end bit-identical, so a trained solver's iteration count is reproducible
    _, _, _, _, _, gt, At = fine_and_coarse(ctx, 64, 12, 11)
    bs = wl.divergence_rhs(np.asarray(gt.codes), (np.full(gt.shape[0] - 1, 1 / 16),) * 3, 300)
    rs, es = xf.harvest_pairs(At, gt.vec(bs), iters=(2, 8, 30))
    out = []
    for _ in range(2):
        net = xf.UNet(gt, seed=1)
        for step in range(30):
            net.train_step(rs[step % 3], es[step % 3], lr=2e-3, op=At)
        out.append(net.params())
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
def test_two_level_refuses_grids_that_are_not_block_coarsenings(ctx):
    codes, sep, g, A, b, gc, _ = fine_and_coarse(ctx, 32, 4, 5)
    wrong = xf.UNet(g, seed=1)   # the fine grid itself: F = 1
    x = g.vec(np.zeros(g.shape))
    with pytest.raises(xf.XFError):
        xf.solve_fcg(A, x, g.vec(b), unet=wrong, precond=capi.XF_PRECOND_UNET2)
    cc, s1, s2, s3 = wl.coarse_grid(codes, sep, 2)
    half = xf.Grid(ctx, cc[:-4], s1[:-4], s2, s3, None)   # F = 2 on two axes only
    wrong2 = xf.UNet(half, seed=1)
    with pytest.raises(xf.XFError):
        xf.solve_fcg(A, x, g.vec(b), unet=wrong2, precond=capi.XF_PRECOND_UNET2)


def _flip_output_layer(p):
    """The same network with its output layer's weights and bias negated: its
    output is exactly the negated output (round-to-nearest is symmetric)."""
    q = p.copy()
    name, ci, co = xf.UNET_LAYERS[-1]
    n_last = 27 * co * ci + co
    q[-n_last:] = -q[-n_last:]
    return q


def _oracle_rel(codes, sep, x, b):
    og = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
    sm = og.smask.astype(bool)
    r = O.apply(O.LAPLACE, og, x, b, -1)
    return np.linalg.norm(r[sm]) / np.linalg.norm(b[sm])


@pytest.mark.gpu
def test_learned_preconditioners_fall_back_to_plain_cg_on_bad_networks(ctx):
    """Plain CG stays the fallback: a network whose output is no descent
    direction (the full-resolution preconditioner with its output layer
    negated) or not finite (weights of magnitude 1e30: the BF16 activations
    overflow) is replaced by z = r, the third time for the rest of the solve,
    and every solve still reaches the true 1e-8 residual (recomputed by the
    oracle) in about plain CG's iterations, counting its fallbacks."""
    codes, sep, g, A, b, gc, _ = fine_and_coarse(ctx, 32, 4, 41)
    bv = g.vec(b)
    plain = None
    cases = []
    good_fine = xf.UNet(g, seed=3).params()
    cases.append(("unet, negated output", xf.UNet(g, _flip_output_layer(good_fine)), capi.XF_PRECOND_UNET, {}))
    huge = np.where(good_fine != 0, 1e30, 0.0)
    cases.append(("unet, huge weights", xf.UNet(g, huge), capi.XF_PRECOND_UNET, {}))
    good_coarse = xf.UNet(gc, seed=3).params()
    huge_c = np.where(good_coarse != 0, 1e30, 0.0)
    for prec in (xf.XF_PREC_FP64, xf.XF_PREC_MIXED):
        cases.append((f"two-level {prec}, huge weights", xf.UNet(gc, huge_c), capi.XF_PRECOND_UNET2,
                      {"precision": prec, "window": 1 if prec == xf.XF_PREC_MIXED else 2}))
    x = g.vec(np.zeros(g.shape))
    plain = xf.solve_fcg(A, x, bv, rtol=1e-8).iterations
    for name, net, pre, kw in cases:
        x = g.vec(np.zeros(g.shape))
        st = xf.solve_fcg(A, x, bv, unet=net, precond=pre, rtol=1e-8, **kw)
        assert st.status == capi.XF_OK, (name, st.status)
        assert st.fallbacks >= 1, (name, st.fallbacks)
        assert _oracle_rel(codes, sep, x.download(), b) <= 1.01e-8, name
        # the fallback is plain CG (the third bad direction switches the network off): close to its count
        assert st.iterations <= 1.3 * plain + 10, (name, st.iterations, plain)


@pytest.mark.gpu
def test_two_level_is_invariant_to_the_sign_of_the_network(ctx):
    """omega = (y, r) / (y, A y) absorbs the network's output scale and sign:
    the two-level preconditioner with the output layer negated takes the same
    iterations to the same bits, with no fallback."""
    codes, sep, g, A, b, gc, _ = fine_and_coarse(ctx, 32, 4, 41)
    bv = g.vec(b)
    p = xf.UNet(gc, seed=3).params()
    out = []
    for params in (p, _flip_output_layer(p)):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve_fcg(A, x, bv, unet=xf.UNet(gc, params), precond=capi.XF_PRECOND_UNET2, rtol=1e-8, window=1,
                          precision=xf.XF_PREC_MIXED)
        assert st.status == capi.XF_OK and st.fallbacks == 0
        out.append((st.iterations, x.download()))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
