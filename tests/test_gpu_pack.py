"""GPU parity of the packed operator (T1dPackOperator, XOperator.cpp:1135-1571)
and of TSLAE::SolveByBiConjugateGradients (XSLAE.cpp:159-348) against the
reference's own outputs (tests/golden/pack_*.npz, made by the compiled
reference).

Bars: both storages (order, columns, values) and A x, A^T x bit-exact; BiCG
meets the reference's stop rule (||r||_2 <= 1e-8) and its solution agrees with
the reference's within 1e-7 relative max-norm (tree-ordered GPU inner products
against the reference's sequential ones).
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from tests.helpers import golden, golden_names, seps
from xflow_gb300 import capi

pytestmark = pytest.mark.gpu

PACKS = golden_names("pack_")


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def setup(ctx, f):
    hx, hy, hz = seps(f)
    g = xf.Grid(ctx, f["codes"], hx, hy, hz, f["normals"])
    A = xf.Operator(g)
    return g, A, xf.PackedOperator(A)


def to_box(g, fwd, v_rn):
    box = np.zeros(g.shape)
    box[fwd[:, 0], fwd[:, 1], fwd[:, 2]] = v_rn
    return box


@pytest.mark.parametrize("name", PACKS)
def test_pack_storages_and_apply_bit_exact(ctx, name):
    f = golden(name)
    g, A, P = setup(ctx, f)
    _, fwd = g.rn_map()
    rows, nnz, nnz_t = P.size()
    assert rows == len(fwd) and nnz == len(f["ref_a_vals"]) and nnz_t == len(f["ref_t_vals"])
    for t, key in ((False, "a"), (True, "t")):
        ptr, cols, vals = P.csr(transpose=t)
        np.testing.assert_array_equal(ptr, f[f"ref_{key}_ptr"])
        np.testing.assert_array_equal(cols, f[f"ref_{key}_cols"])
        np.testing.assert_array_equal(vals, f[f"ref_{key}_vals"])
    x = g.vec(to_box(g, fwd, f["x_rn"]))
    y = g.vec(None)
    P.apply(x, y, flags=xf.XF_ZERO_INACTIVE)
    np.testing.assert_array_equal(y.download()[fwd[:, 0], fwd[:, 1], fwd[:, 2]], f["ref_ax"])
    P.transpose()
    P.apply(x, y, flags=xf.XF_ZERO_INACTIVE)
    np.testing.assert_array_equal(y.download()[fwd[:, 0], fwd[:, 1], fwd[:, 2]], f["ref_atx"])
    P.transpose()
    P.apply(x, y, flags=xf.XF_ZERO_INACTIVE)
    np.testing.assert_array_equal(y.download()[fwd[:, 0], fwd[:, 1], fwd[:, 2]], f["ref_ax"])


def test_bicg_matches_reference(ctx):
    f = golden("pack_cube")
    g, A, P = setup(ctx, f)
    _, fwd = g.rn_map()
    b = g.vec(to_box(g, fwd, f["b_rn"]))
    x = g.vec(np.full(g.shape, 3.0))   # ignored: the reference starts from 0 (XSLAE.cpp:171)
    st = xf.solve(P, x, b, method=xf.XF_BICG)
    assert st.status == capi.XF_OK, st.status
    assert st.abs_resid <= 1e-8
    got = x.download()[fwd[:, 0], fwd[:, 1], fwd[:, 2]]
    ref = f["ref_bicg_x"]
    assert np.abs(got - ref).max() <= 1e-7 * np.abs(ref).max()
    # the same iteration count as the oracle's restatement of the reference, within 10%
    hx, hy, hz = seps(f)
    pk = O.pack_build(O.LAPLACE, O.Grid(f["codes"], f["normals"], hx, hy, hz))
    _, ost, rc = O.bicg_reference(pk, f["b_rn"])
    assert rc == 0 and abs(st.iterations - ost.iterations) <= max(2, ost.iterations // 10)
    # an iteration cap ends it with XF_MAXIT
    st = xf.solve(P, x, b, method=xf.XF_BICG, maxit=3)
    assert st.status == capi.XF_MAXIT and st.iterations == 3


def test_packed_operator_in_other_solvers(ctx):
    """BiCGStab through the packed operator agrees with BiCGStab through the
    stencil it was built from (same system, FP64, both reach the reference's
    stop rule)."""
    f = golden("pack_cube")
    g, A, P = setup(ctx, f)
    rng = np.random.Generator(np.random.PCG64(5))
    sm = g.space_mask().astype(bool)
    b = g.vec(np.where(sm, rng.standard_normal(g.shape), 0.0))
    xs, xp = g.vec(np.zeros(g.shape)), g.vec(np.zeros(g.shape))
    s1 = xf.solve(A, xs, b, method=xf.XF_BICGSTAB)
    s2 = xf.solve(P, xp, b, method=xf.XF_BICGSTAB)
    assert s1.status == capi.XF_OK and s2.status == capi.XF_OK
    d1, d2 = xs.download()[sm], xp.download()[sm]
    assert np.abs(d1 - d2).max() <= 1e-3 * np.abs(d1).max()


def test_transpose_and_bicg_need_a_pack(ctx):
    f = golden("pack_cube")
    g, A, P = setup(ctx, f)
    assert capi.lib().xf_op_transpose(A.h) == capi.XF_ERR_UNSUPPORTED   # T3dLaplaceOperator::operator~ throws
    with pytest.raises(xf.XFError) as e:
        xf.solve(A, g.vec(np.zeros(g.shape)), g.vec(np.ones(g.shape)), method=xf.XF_BICG)
    assert e.value.status == capi.XF_ERR_UNSUPPORTED
    with pytest.raises(xf.XFError):   # packed operators are FP64
        P.apply(g.vec(None, xf.XF_F32), g.vec(None, xf.XF_F32))
