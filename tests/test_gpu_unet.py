"""The learned preconditioner: the U-Net's forward pass and gradients (run by
the tensor-core convolutions and this library's backward pass) against the
numpy FP64 restatement in oracle/unet_ref.py, and what training buys.

Bars (the GPU keeps BF16 weights and activations through 11 layers): the
network output within 3e-2 relative L2 of the oracle's, the loss within 3e-2
relative, the full gradient within 6e-2 relative L2 (each layer within 0.2),
for both losses (MSE against the scaled error, and the A-norm angle).
Training on (residual, error) pairs harvested from plain CG's own iterates
lowers the loss, and the trained network, used by the flexible CG on a fresh
geometry, needs fewer iterations than plain CG to the same true 1e-8
relative residual.
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from oracle import unet_ref as U
from xflow_gb300 import capi
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def spheres(ctx, n, nsph, seed):
    codes, nrm, nodes, sep, _ = wl.spheres_grid(n, nsph, 1.5 / n, 3.0 / n, seed)
    b = wl.divergence_rhs(codes, (sep, sep, sep), seed + 1)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    return g, xf.Operator(g), b


def test_unet_forward_and_gradients_match_oracle(ctx):
    g, A, b = spheres(ctx, 16, 3, 31)
    m0 = g.space_mask().astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(3))
    r = rng.standard_normal(g.shape) * m0
    e = rng.standard_normal(g.shape) * m0
    params = xf.unet_init_params(seed=5)
    net = xf.UNet(g, params)
    # forward
    z = net.apply(g.vec(r), g.vec(None)).download()
    zo, _ = U.forward(params, r, m0)
    zo = zo * m0
    assert np.linalg.norm(z - zo) <= 3e-2 * np.linalg.norm(zo)
    # loss and gradients (no update)
    loss = net.train_step(g.vec(r), g.vec(e), update=False)
    grads = net.grads()
    lo, go, _ = U.loss_and_grads(params, r, e, m0)
    assert abs(loss - lo) <= 3e-2 * lo
    assert np.linalg.norm(grads - go) <= 6e-2 * np.linalg.norm(go)
    o = 0
    for name, ci, co in U.LAYERS:
        k = 27 * co * ci + co
        gl, ol = grads[o:o + k], go[o:o + k]
        o += k
        if np.linalg.norm(ol) > 0:
            assert np.linalg.norm(gl - ol) <= 0.2 * np.linalg.norm(ol), name
    # the parameters round-trip
    np.testing.assert_array_equal(net.params(), params)
    # the A-norm loss on a consistent pair (r = A e)
    og = O.Grid(np.asarray(g.codes), np.zeros(g.shape + (3,)), *(np.full(n - 1, 1 / 16) for n in g.shape))
    apply_A = lambda x: O.apply(O.LAPLACE, og, x)  # noqa: E731
    r2 = apply_A(e) * m0
    loss = net.train_step(g.vec(r2), g.vec(e), update=False, op=A)
    grads = net.grads()
    lo, go, _ = U.loss_and_grads(params, r2, e, m0, apply_A)
    assert abs(loss - lo) <= 3e-2 * max(lo, 1e-2)
    assert np.linalg.norm(grads - go) <= 6e-2 * np.linalg.norm(go)


def test_training_lowers_loss_and_iterations(ctx):
    # train on one geometry: (r_k, e_k) from plain CG's own iterates for 4 right-hand sides
    g, A, b = spheres(ctx, 32, 6, 41)
    net = xf.UNet(g, seed=1)
    rs, es = [], []
    for s in range(4):
        bs = wl.divergence_rhs(np.asarray(g.codes), (np.full(33, 1 / 32),) * 3, 100 + s)
        r_, e_ = xf.harvest_pairs(A, g.vec(bs), iters=(2, 5, 10, 20, 40, 80, 120, 160))
        rs += r_
        es += e_
    first = np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)])
    for step in range(400):
        q = step % len(rs)
        net.train_step(rs[q], es[q], lr=2e-3, op=A)
    last = np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)])
    print("A-norm loss on the training pairs before / after:", first, last)
    assert last < 0.5 * first, (first, last)
    # fresh geometry: held-out pairs, and flexible CG vs plain CG and Jacobi
    g2, A2, b2 = spheres(ctx, 32, 6, 77)
    net2 = xf.UNet(g2, net.params())
    fresh = xf.UNet(g2, seed=1)   # the untrained network
    bv = g2.vec(b2)
    hr, he = xf.harvest_pairs(A2, bv, iters=(3, 15, 60, 150))
    held_trained = np.mean([net2.train_step(r, e, update=False, op=A2) for r, e in zip(hr, he)])
    held_fresh = np.mean([fresh.train_step(r, e, update=False, op=A2) for r, e in zip(hr, he)])
    print("A-norm loss on a fresh geometry, untrained / trained:", held_fresh, held_trained)
    assert held_trained < 0.8 * held_fresh
    its = {}
    for name, kw in (("plain", {}), ("jacobi", {"precond": capi.XF_PRECOND_JACOBI}), ("unet", {"unet": net2})):
        x = g2.vec(np.zeros(g2.shape))
        st = xf.solve_fcg(A2, x, bv, rtol=1e-8, **kw)
        assert st.status == capi.XF_OK and st.rel_resid <= 1e-8, (name, st.status, st.rel_resid)
        its[name] = (st.iterations, st.fallbacks)
    print("FCG iterations, fallbacks (plain, jacobi, unet):", its)
    assert its["unet"][0] < its["plain"][0], its
