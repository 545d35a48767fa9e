"""GPU parity of the C-ABI path against the reference's golden vectors and the
CPU oracle.

Bars: integer/index work and XF_EXACT FP64 rows bit-exact; FP64 fast rows
within 1e-13 x max|y|; FP32 rows within 2e-6 x max|y|; FP64 reductions within
1e-13 relative (different summation order); solves reach their own stopping
rule and agree with the oracle's solve.
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from tests.helpers import golden, golden_names, seps
from xflow_gb300 import capi
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

MATVEC = golden_names("matvec_")


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def make_grid(ctx, f):
    hx, hy, hz = seps(f)
    return xf.Grid(ctx, f["codes"], hx, hy, hz, f["normals"])


@pytest.mark.parametrize("name", MATVEC)
def test_rn_numbering_bit_exact(ctx, name):
    f = golden(name)
    g = make_grid(ctx, f)
    assert g.end_index == int(f["ref_end_index"][0])
    np.testing.assert_array_equal(g.space_mask(), wl.space_mask(f["codes"]))
    inv, fwd = g.rn_map()
    R, inv_o, fwd_o = O.rn_map(wl.space_mask(f["codes"]))
    np.testing.assert_array_equal(inv, inv_o)
    np.testing.assert_array_equal(fwd, fwd_o)
    x = f["x"]
    np.testing.assert_array_equal(x[tuple(fwd.T)], f["ref_x_by_rn"])


@pytest.mark.parametrize("name", MATVEC)
def test_laplace_exact_rows_bit_exact(ctx, name):
    f = golden(name)
    g = make_grid(ctx, f)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    x, s = g.vec(f["x"]), g.vec(f["s"])
    for key, sign in (("ref_lap_y", 0), ("ref_lap_y_plus", 1), ("ref_lap_y_minus", -1)):
        y = g.vec(f["y_init"])
        A.apply(x, y, s if sign else None, sign, xf.XF_EXACT)
        np.testing.assert_array_equal(y.download().ravel(), f[key])


@pytest.mark.parametrize("name", [n for n in MATVEC if "vardiv" in n])
def test_vardiv_exact_rows_bit_exact(ctx, name):
    f = golden(name)
    g = make_grid(ctx, f)
    A = xf.Operator(g, xf.XF_OP_VARDIV, density=f["density"])
    y = g.vec(f["y_init"])
    A.apply(g.vec(f["x"]), y, flags=xf.XF_EXACT)
    np.testing.assert_array_equal(y.download().ravel(), f["ref_vd_y"])


@pytest.mark.parametrize("name", MATVEC)
@pytest.mark.parametrize("op", [xf.XF_OP_LAPLACE, xf.XF_OP_VARDIV])
def test_fast_rows_fp64_and_fp32(ctx, name, op):
    f = golden(name)
    if op == xf.XF_OP_VARDIV and "vardiv" not in name:
        pytest.skip("variable-density rows are defined only off the box faces")
    g = make_grid(ctx, f)
    A = xf.Operator(g, op, density=f["density"] if op == xf.XF_OP_VARDIV else None)
    ref = f["ref_lap_y"] if op == xf.XF_OP_LAPLACE else f["ref_vd_y"]
    sm = wl.space_mask(f["codes"]).ravel().astype(bool)
    scale = np.abs(ref[sm]).max()
    y = g.vec(f["y_init"])
    A.apply(g.vec(f["x"]), y)
    got = y.download().ravel()
    np.testing.assert_array_equal(got[~sm], f["y_init"].ravel()[~sm])
    assert np.abs(got[sm] - ref[sm]).max() <= 1e-13 * scale
    y32 = g.vec(f["y_init"], xf.XF_F32)
    A.apply(g.vec(f["x"], xf.XF_F32), y32)
    got = y32.download().ravel()
    assert np.abs(got[sm] - ref[sm]).max() <= 2e-6 * scale


@pytest.mark.parametrize("name", MATVEC)
def test_vector_algebra(ctx, name):
    f = golden(name)
    g = make_grid(ctx, f)
    x, s = g.vec(f["x"]), g.vec(f["s"])
    p1, p2 = float(f["p1"]), float(f["p2"])
    for key, args in (("ref_lc_p1x_p2s", (p1, x, p2, s)), ("ref_lc_x_minus_s", (1.0, x, -1.0, s)),
                      ("ref_lc_x_p2s", (1.0, x, p2, s)), ("ref_lc_p1x", (p1, x)), ("ref_lc_zero", (0.0, x))):
        z = g.vec(f["y_init"])
        z.lincomb(*args)
        np.testing.assert_array_equal(z.download().ravel(), f[key], err_msg=key)
    z = g.vec(f["y_init"])
    z.assign(x)
    np.testing.assert_array_equal(z.download().ravel(), f["ref_assign_x"])
    z = g.vec(f["y_init"]).fill(0.0)
    np.testing.assert_array_equal(z.download().ravel(), f["ref_lc_zero"])
    assert x.dot(s) == pytest.approx(f["ref_dot_xs"][0], rel=1e-13, abs=1e-13)
    assert x.norm() == pytest.approx(f["ref_norm_x"][0], rel=1e-14)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    assert A.dot_op(x, s) == pytest.approx(f["ref_dot_x_As"][0], rel=1e-11, abs=1e-9)
    assert x.absmax() == (f["ref_absmax_x"][0], f["ref_absmax_x_index"][0])
    assert s.absmax() == (f["ref_absmax_s"][0], f["ref_absmax_s_index"][0])
    z = g.vec(np.zeros(g.shape))
    assert z.absmax() == (0.0, 1)   # nothing beats 0: Rn index 1 (XSpace.cpp:3442)


def test_fused_dot_matches_separate(ctx):
    f = golden("matvec_mixed_b")
    g = make_grid(ctx, f)
    A = xf.Operator(g)
    x, y = g.vec(f["x"]), g.vec(f["y_init"])
    d = A.apply(x, y, want_dot=True)
    assert d == pytest.approx(x.dot(y), rel=1e-13)


def test_rejected_grids_match_reference_throws(ctx):
    f = golden("errors")
    names = sorted({k[: -len("_threw")] for k in f if k.endswith("_threw")})
    hx, hy, hz = (np.diff(f[k]) for k in ("x_nodes", "y_nodes", "z_nodes"))
    for n in names:
        assert bool(f[n + "_threw"])
        g = xf.Grid(ctx, f[n + "_codes"], hx, hy, hz, f[n + "_normals"])
        st, bad = g.check(xf.XF_OP_LAPLACE)
        assert st == capi.XF_ERR_MASK and bad >= 0, n
        with pytest.raises(xf.XFError) as e:
            xf.Operator(g, xf.XF_OP_LAPLACE)
        assert e.value.status == capi.XF_ERR_MASK


def test_vardiv_requires_density(ctx):
    f = golden("matvec_vardiv_a")
    g = make_grid(ctx, f)
    A = xf.Operator(g, xf.XF_OP_VARDIV)
    with pytest.raises(xf.XFError) as e:
        A.apply(g.vec(f["x"]), g.vec())
    assert e.value.status == capi.XF_ERR_STATE


def test_vardiv_rejects_face_prenormal_rows(ctx):
    f = golden("matvec_mixed_a")   # PreNormal rows on the faces
    g = make_grid(ctx, f)
    assert g.check(xf.XF_OP_LAPLACE)[0] == capi.XF_OK
    assert g.check(xf.XF_OP_VARDIV)[0] == capi.XF_ERR_MASK


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name,method,norm", [
    ("solve_cg_spd", xf.XF_CG_REFERENCE, 2),
    ("solve_minres_spd", xf.XF_MINRES, 2),
    ("solve_bicgstab_cube", xf.XF_BICGSTAB, np.inf),
    ("solve_bicgstab_vardiv", xf.XF_BICGSTAB, np.inf),
])
@pytest.mark.parametrize("exact", [True, False])
def test_reference_solvers_against_reference(ctx, name, method, norm, exact):
    f = golden(name)
    g = make_grid(ctx, f)
    op = int(f["op"])
    A = xf.Operator(g, op, density=f.get("density"))
    x, b = g.vec(f["x0"]), g.vec(f["b"])
    st = xf.solve(A, x, b, method=method, exact=exact, maxit=100000)
    assert st.status == capi.XF_OK
    got = x.download()
    hx, hy, hz = seps(f)
    og = O.Grid(f["codes"], f["normals"], hx, hy, hz, f.get("density"))
    r = O.apply(op, og, got, f["b"], -1)
    sm = og.smask.astype(bool)
    eps = {xf.XF_CG_REFERENCE: 1e-5, xf.XF_MINRES: 1e-7, xf.XF_BICGSTAB: 1e-5}[method]
    # the solve met the reference's own stopping rule ...
    assert np.linalg.norm(r[sm], ord=norm) <= eps * (1 + 1e-6)
    # ... and lands where the reference's solve landed
    ref = f["ref_result"].reshape(g.shape)
    err = np.abs(got - ref)[sm].max() / max(1.0, np.abs(ref[sm]).max())
    assert err <= 1e-4
    np.testing.assert_array_equal(got[~sm], f["x0"][~sm])
    # same iteration count as the same algorithm on the CPU, up to rounding
    fn = {xf.XF_CG_REFERENCE: O.cg_reference, xf.XF_MINRES: O.minres_reference,
          xf.XF_BICGSTAB: O.bicgstab_reference}[method]
    O.set_threads(1)
    _, ost = fn(op, og, f["x0"], f["b"])
    # BiCGStab's residual history is not smooth: a different summation order
    # can move its stopping iteration by a fair fraction.
    slack = ost.iterations // 3 + 5 if method == xf.XF_BICGSTAB else max(2, ost.iterations // 20)
    assert abs(st.iterations - ost.iterations) <= slack


def spheres_case(n, nsph, seed):
    codes, nrm, nodes, sep, _ = wl.spheres_grid(n, nsph, 0.02 * 64 / n if n < 64 else 0.02, 0.06, seed)
    b = wl.divergence_rhs(codes, (sep, sep, sep), seed + 1)
    return codes, nrm, sep, b


@pytest.mark.parametrize("precision", [xf.XF_PREC_FP64, xf.XF_PREC_MIXED])
@pytest.mark.parametrize("n", [40, 25])   # box 42 (even rows): fused direction update; box 27: three-kernel path
def test_plain_cg_matches_oracle_cg(ctx, precision, n):
    codes, nrm, sep, b = spheres_case(n, 6, 5)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    x, bv = g.vec(np.zeros(g.shape)), g.vec(b)
    st = xf.solve(A, x, bv, method=xf.XF_CG, precision=precision, rtol=1e-8)
    assert st.status == capi.XF_OK, st.status
    assert st.rel_resid <= 1e-8
    og = O.Grid(codes, nrm, sep, sep, sep)
    O.set_threads(8)
    xo, ost = O.cg_plain(O.LAPLACE, og, np.zeros(g.shape), b, 1e-10)
    O.set_threads(1)
    got = x.download()
    sm = og.smask.astype(bool)
    # singular (all-Neumann) system: compare after removing the mean
    d = (got - got[sm].mean()) - (xo - xo[sm].mean())
    rel = np.abs(d[sm]).max() / np.abs(xo[sm] - xo[sm].mean()).max()
    assert rel <= 1e-5, rel
    if precision == xf.XF_PREC_FP64:
        assert abs(st.iterations - ost.iterations) <= ost.iterations  # same method, looser tol on oracle
    else:
        assert st.replacements >= 1


def test_mixed_cg_refines_to_1e10(ctx):
    codes, nrm, sep, b = spheres_case(48, 8, 7)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    x, bv = g.vec(np.zeros(g.shape)), g.vec(b)
    st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-10)
    assert st.status == capi.XF_OK
    assert st.rel_resid <= 1e-10
    # independent FP64 check of the residual on the host
    og = O.Grid(codes, nrm, sep, sep, sep)
    r = O.apply(O.LAPLACE, og, x.download(), b, -1)
    sm = og.smask.astype(bool)
    assert np.linalg.norm(r[sm]) / np.linalg.norm(b[sm]) <= 1.01e-10


def test_solve_host_roundtrip(ctx):
    codes, nrm, sep, b = spheres_case(32, 4, 9)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    xh = np.zeros(g.shape)
    st = xf.solve_host(A, xh, np.ascontiguousarray(b), method=xf.XF_CG, rtol=1e-8)
    assert st.status == capi.XF_OK and st.rel_resid <= 1e-8
    og = O.Grid(codes, nrm, sep, sep, sep)
    r = O.apply(O.LAPLACE, og, xh, b, -1)
    sm = og.smask.astype(bool)
    assert np.linalg.norm(r[sm]) / np.linalg.norm(b[sm]) <= 1.01e-8


@pytest.mark.parametrize("precision", [xf.XF_PREC_FP64, xf.XF_PREC_MIXED])
def test_maxit_status(ctx, precision):
    codes, nrm, sep, b = spheres_case(32, 4, 11)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    st = xf.solve(A, g.vec(np.zeros(g.shape)), g.vec(b), method=xf.XF_CG, precision=precision, rtol=1e-12,
                  maxit=5)
    assert st.status == capi.XF_MAXIT and st.iterations == 5


# box 50, box 66 (P % 8 == 4: a half 8-cell group ends the plane) and box 72
# (3 tiles of the staged kernels, the last one partial)
@pytest.mark.parametrize("n", [48, 64, 70])
def test_fused_direction_update_matches_three_kernel_path(ctx, monkeypatch, n):
    """The mixed CG's fused iteration (p' = r + beta p inside the stencil, p
    ping-ponging between two buffers), by the bulk-staged kernel, the tiled
    kernel and the register march, against the three-kernel iteration on the
    same system: same iteration count within 2, same solution within the
    solve's own accuracy."""
    codes, nrm, sep, b = spheres_case(n, 8, 21)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    bv = g.vec(b)
    out = {}
    # "12b": the bulk-staged kernel on 3 blocks, several work items each (the cross-item load stream)
    for fuse, pqt, cap in (("1", "2", None), ("1", "2", "3"), ("1", "1", None), ("1", "0", None), ("0", "1", None)):
        monkeypatch.setenv("XF_PQ_FUSE", fuse)
        monkeypatch.setenv("XF_PQT", pqt)
        if cap:
            monkeypatch.setenv("XF_PQB_BLOCKS", cap)
        else:
            monkeypatch.delenv("XF_PQB_BLOCKS", raising=False)
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-9)
        assert st.status == capi.XF_OK and st.rel_resid <= 1e-9
        out[fuse + pqt + ("b" if cap else "")] = (st, x.download())
    monkeypatch.delenv("XF_PQB_BLOCKS", raising=False)
    s0, x0 = out["01"]
    sm = codes != 0
    for key in ("12", "12b", "11", "10"):
        s1, x1 = out[key]
        assert abs(s1.iterations - s0.iterations) <= 2, (key, s1.iterations, s0.iterations)
        d = (x1 - x1[sm].mean()) - (x0 - x0[sm].mean())
        assert np.abs(d[sm]).max() <= 1e-6 * np.abs(x0[sm] - x0[sm].mean()).max()


def test_nan_rhs_reports_nan(ctx):
    codes, nrm, sep, b = spheres_case(24, 2, 13)
    b = b.copy()
    act = np.argwhere(codes == 1)
    b[tuple(act[len(act) // 2])] = np.nan
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    for prec in (xf.XF_PREC_FP64, xf.XF_PREC_MIXED):
        st = xf.solve(A, g.vec(np.zeros(g.shape)), g.vec(b), method=xf.XF_CG, precision=prec)
        assert st.status == capi.XF_NAN


@pytest.mark.parametrize("n", [48, 64, 70])
def test_chebyshev_preconditioned_mixed_cg(ctx, monkeypatch, n):
    """Mixed CG with the Chebyshev polynomial preconditioner against plain
    mixed CG on the same system: degree 2 (both stencil levels of z = p(A) r
    in one pass) meets the same true FP64 tolerance in well under 0.6 x the
    iterations, degrees 4, 6, 8 (one pass per quadratic factor) in under 0.4,
    0.32, 0.26 x, and the solutions agree within the solve's own accuracy; also with a
    capped grid (several work items per block, the cross-item load stream)."""
    codes, nrm, sep, b = spheres_case(n, 8, 21)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    bv = g.vec(b)
    x0 = g.vec(np.zeros(g.shape))
    s0 = xf.solve(A, x0, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-9)
    assert s0.status == capi.XF_OK
    sm = codes != 0
    ref = x0.download()
    for cap, deg in ((None, 2), (None, 4), (None, 6), ("3", 2), ("3", 4), ("3", 8)):
        if cap:
            monkeypatch.setenv("XF_POLY_BLOCKS", cap)
        else:
            monkeypatch.delenv("XF_POLY_BLOCKS", raising=False)
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-9, precond=capi.XF_PRECOND_CHEB,
                      cheb_degree=deg)
        assert st.status == capi.XF_OK and st.rel_resid <= 1e-9, (deg, st.status, st.rel_resid)
        assert st.iterations < {2: 0.6, 4: 0.4, 6: 0.32, 8: 0.26}[deg] * s0.iterations, (deg, st.iterations,
                                                                                  s0.iterations)
        d = (x.download() - x.download()[sm].mean()) - (ref - ref[sm].mean())
        assert np.abs(d[sm]).max() <= 1e-6 * np.abs(ref[sm] - ref[sm].mean()).max()
    monkeypatch.delenv("XF_POLY_BLOCKS", raising=False)


@pytest.mark.parametrize("n,replace_every,deg", [(48, 50, 2), (70, 7, 2), (64, 1, 2), (48, 50, 4), (70, 7, 4),
                                                  (64, 1, 4), (48, 50, 6), (70, 7, 8)])
def test_fused_residual_update_matches_separate_launches(ctx, monkeypatch, n, replace_every, deg):
    """The preconditioned solve (degrees 2 to 8) with the residual update
    fused into the (first) polynomial pass (two residual buffers) against the
    same solve with the
    update and the polynomial as separate launches: the iterates are the same
    arithmetic, so the iteration counts and solutions agree exactly; also
    with a capped grid (several work items per block: the q copies and the
    raw ring carry their barrier phases across items) and with chunks of odd
    and unit length (the residual ends a chunk in either buffer)."""
    codes, nrm, sep, b = spheres_case(n, 8, 23)
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    bv = g.vec(b)
    for cap in (None, "5"):
        if cap:
            monkeypatch.setenv("XF_POLY_BLOCKS", cap)
        else:
            monkeypatch.delenv("XF_POLY_BLOCKS", raising=False)
        out = {}
        for fused in ("1", "0"):
            monkeypatch.setenv("XF_POLYR", fused)
            x = g.vec(np.zeros(g.shape))
            st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=1e-9,
                          precond=capi.XF_PRECOND_CHEB, replace_every=replace_every, cheb_degree=deg)
            assert st.status == capi.XF_OK and st.rel_resid <= 1e-9, (fused, st.status, st.rel_resid)
            out[fused] = (st.iterations, x.download())
        assert out["1"][0] == out["0"][0]
        assert np.array_equal(out["1"][1], out["0"][1])
    monkeypatch.delenv("XF_POLY_BLOCKS", raising=False)
    monkeypatch.delenv("XF_POLYR", raising=False)


def test_chebyshev_preconditioner_needs_uniform_grid(ctx):
    codes, nrm = wl.poisson_cube(12, 12, 12)
    rng = np.random.Generator(np.random.PCG64(2))
    seps = [np.diff(wl.random_nodes(12, rng)) for _ in range(3)]
    g = xf.Grid(ctx, codes, *seps, nrm)
    A = xf.Operator(g)
    with pytest.raises(xf.XFError) as e:
        xf.solve(A, g.vec(np.zeros(g.shape)), g.vec(np.ones(g.shape)), method=xf.XF_CG,
                 precision=xf.XF_PREC_MIXED, precond=capi.XF_PRECOND_CHEB)
    assert e.value.status == capi.XF_ERR_UNSUPPORTED
