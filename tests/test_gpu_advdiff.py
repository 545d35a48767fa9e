"""GPU parity of the implicit advection-diffusion operator (momentum /
transport: the reference's ADI line coefficients, XProblem.cpp:1236-1238,
summed over the three directions; with XF_ADV_UPWIND the upwind scheme of
the concentration equation, :1828-1843) against the oracle's restatement,
and its solves by the reference Krylov methods.

Bars: FP64 rows with XF_EXACT bit-exact, the fast FP64 rows (the seven-
coefficient table) within 1e-13 x max|y|; FP32 rows within 2e-6 x max|y|; the packed form
within 1e-13 x max|y| (row dot in pack order vs the stencil's expression
order); solves of a manufactured system reach their stop rule and recover the
solution within 1e-6 relative max-norm.
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import capi
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def case(ctx, shape=(12, 11, 13), seed=3, tau=1e-2, D=0.05, flags=3):
    """Dirichlet-bounded box (PreDefined faces, PreNormal rims, non-uniform
    spacings) with a seeded advecting velocity."""
    rng = np.random.Generator(np.random.PCG64(seed))
    codes, nrm = wl.poisson_cube(*shape)
    nodes = [wl.random_nodes(n, rng) for n in shape]
    seps = [np.diff(x) for x in nodes]
    vel = [rng.uniform(-2, 2, shape) for _ in range(3)]
    g = xf.Grid(ctx, codes, *seps, nrm)
    A = xf.Operator(g, xf.XF_OP_ADVDIFF)
    A.set_advection(*(g.vec(v) for v in vel), tau, D, flags)
    og = O.Grid(codes, nrm, *seps)
    return g, A, og, vel, rng


@pytest.mark.parametrize("flags", [1, 2, 3, 5, 7])   # 4: the upwind form
def test_advdiff_rows_match_oracle(ctx, flags):
    g, A, og, vel, rng = case(ctx, flags=flags)
    x = rng.standard_normal(g.shape)
    want = O.apply_advdiff(og, x, *vel, 1e-2, 0.05, flags)
    sm = og.smask.astype(bool)
    y = g.vec(None)
    A.apply(g.vec(x), y, flags=xf.XF_ZERO_INACTIVE | xf.XF_EXACT)
    got = y.download()
    np.testing.assert_array_equal(got[sm], want[sm])
    A.apply(g.vec(x), y, flags=xf.XF_ZERO_INACTIVE)
    fast = y.download()
    assert np.abs(fast[sm] - want[sm]).max() <= 1e-13 * np.abs(want[sm]).max()
    assert not np.array_equal(fast[sm], want[sm])   # the fast form is the one a plain apply takes
    y32 = g.vec(None, xf.XF_F32)
    A.apply(g.vec(x, xf.XF_F32), y32, flags=xf.XF_ZERO_INACTIVE)
    assert np.abs(y32.download()[sm] - want[sm]).max() <= 2e-6 * np.abs(want[sm]).max()


def test_advdiff_solves(ctx):
    g, A, og, vel, rng = case(ctx, shape=(18, 16, 17), seed=9)
    sm = og.smask.astype(bool)
    xt = np.where(sm, rng.standard_normal(g.shape), 0.0)
    b = O.apply_advdiff(og, xt, *vel, 1e-2, 0.05, 3)
    bv = g.vec(b)
    for method in (xf.XF_BICGSTAB, xf.XF_MINRES):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=method, atol=1e-10)
        assert st.status == capi.XF_OK, (method, st.status)
        got = x.download()
        r = O.apply_advdiff(og, got, *vel, 1e-2, 0.05, 3) - b
        assert np.linalg.norm(r[sm]) <= 1e-8 * np.linalg.norm(b[sm])
        assert np.abs(got[sm] - xt[sm]).max() <= 1e-6 * np.abs(xt[sm]).max()
    # BiCG needs A^T: through the packed form of the same operator
    P = xf.PackedOperator(A)
    yp, ys = g.vec(None), g.vec(None)
    P.apply(g.vec(xt), yp, flags=xf.XF_ZERO_INACTIVE)
    A.apply(g.vec(xt), ys, flags=xf.XF_ZERO_INACTIVE)
    d = yp.download()[sm] - ys.download()[sm]
    assert np.abs(d).max() <= 1e-13 * np.abs(ys.download()[sm]).max()
    x = g.vec(np.zeros(g.shape))
    st = xf.solve(P, x, bv, method=xf.XF_BICG, atol=1e-9)
    assert st.status == capi.XF_OK, st.status
    assert np.abs(x.download()[sm] - xt[sm]).max() <= 1e-6 * np.abs(xt[sm]).max()


def test_upwind_transport_solves(ctx):
    """The concentration equation's operator (upwind convection plus diffusion) under minimal residuals and
    BiCGStab recovers a manufactured solution."""
    g, A, og, vel, rng = case(ctx, shape=(18, 16, 17), seed=11, flags=7)
    sm = og.smask.astype(bool)
    xt = np.where(sm, rng.standard_normal(g.shape), 0.0)
    b = O.apply_advdiff(og, xt, *vel, 1e-2, 0.05, 7)
    bv = g.vec(b)
    for method in (xf.XF_MINRES, xf.XF_BICGSTAB):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=method, atol=1e-10)
        assert st.status == capi.XF_OK, (method, st.status)
        assert np.abs(x.download()[sm] - xt[sm]).max() <= 1e-6 * np.abs(xt[sm]).max()


def test_jacobi_bicgstab_on_the_transport_operator(ctx):
    """Right Jacobi preconditioning of BiCGStab: the same stop rule on the true residual, the manufactured
    solution recovered, and fewer iterations than plain BiCGStab on a system whose border rows (semi-sums,
    normal differences) are far from the Actual rows' scale."""
    g, A, og, vel, rng = case(ctx, shape=(26, 22, 24), seed=13, tau=1e-3, D=0.02, flags=7)
    sm = og.smask.astype(bool)
    xt = np.where(sm, rng.standard_normal(g.shape), 0.0)
    b = O.apply_advdiff(og, xt, *vel, 1e-3, 0.02, 7)
    bv = g.vec(b)
    its = {}
    for pre in (capi.XF_PRECOND_NONE, capi.XF_PRECOND_JACOBI):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=xf.XF_BICGSTAB, precond=pre, atol=1e-9 * np.abs(b).max())
        assert st.status == capi.XF_OK, (pre, st.status)
        got = x.download()
        r = O.apply_advdiff(og, got, *vel, 1e-3, 0.02, 7) - b
        assert np.abs(r[sm]).max() <= 1e-9 * np.abs(b).max() * 1.0001
        assert np.abs(got[sm] - xt[sm]).max() <= 1e-5 * np.abs(xt[sm]).max()
        its[pre] = st.iterations
    assert its[capi.XF_PRECOND_JACOBI] < its[capi.XF_PRECOND_NONE], its
    # the Laplace operator of the same grid (Dirichlet faces: semi-sum rows beside rows of 1/h^2)
    L = xf.Operator(g, xf.XF_OP_LAPLACE)
    bl = O.apply(O.LAPLACE, og, xt)
    blv = g.vec(bl)
    its = {}
    for pre in (capi.XF_PRECOND_NONE, capi.XF_PRECOND_JACOBI):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(L, x, blv, method=xf.XF_BICGSTAB, precond=pre, atol=1e-9 * np.abs(bl).max())
        assert st.status == capi.XF_OK, (pre, st.status)
        assert np.abs(x.download()[sm] - xt[sm]).max() <= 1e-4 * np.abs(xt[sm]).max()
        its[pre] = st.iterations
    assert its[capi.XF_PRECOND_JACOBI] < its[capi.XF_PRECOND_NONE], its
    # a packed operator has no diagonal table: refused
    P = xf.PackedOperator(L)
    with pytest.raises(xf.XFError) as e:
        xf.solve(P, g.vec(np.zeros(g.shape)), blv, method=xf.XF_BICGSTAB, precond=capi.XF_PRECOND_JACOBI)
    assert e.value.status == capi.XF_ERR_UNSUPPORTED


def test_advdiff_needs_coefficients(ctx):
    codes, nrm = wl.poisson_cube(8, 8, 8)
    sep = np.full(7, 1 / 7)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g, xf.XF_OP_ADVDIFF)
    with pytest.raises(xf.XFError) as e:
        A.apply(g.vec(None), g.vec(None))
    assert e.value.status == capi.XF_ERR_STATE
    with pytest.raises(xf.XFError):
        A.set_advection(None, None, None, 0.0, 1.0)   # tau = 0
