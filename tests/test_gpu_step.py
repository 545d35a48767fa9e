"""GPU parity of the time-step passes around the pressure solve
(XProblem.cpp:5474-5829) against the CPU oracle: pressure right-hand side,
velocity correction of each component, control-balance divergence maximum.
Bar: bit-exact (FP64, the reference's expressions and order), the same first
offending cell and status where the reference throws.
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import workloads as wl_step
from xflow_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def grids(ctx, cs):
    gp = xf.Grid(ctx, cs["pc"], *cs["hP"])
    gu = xf.Grid(ctx, cs["uc"], *cs["hU"])
    gv = xf.Grid(ctx, cs["vc"], *cs["hV"])
    gw = xf.Grid(ctx, cs["wc"], *cs["hW"])
    return gp, gu, gv, gw


@pytest.mark.parametrize("with_density", [False, True])
def test_pressure_rhs_matches_oracle(ctx, with_density):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    dens = cs["density"] if with_density else None
    rhs = gp.vec(np.full(gp.shape, 9.0))
    xf.pressure_rhs(gp, gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]), cs["tau"], rhs,
                    density=gp.vec(dens) if dens is not None else None, border=gp.vec(cs["p_border"]))
    want, st, _ = O.pressure_rhs(cs["pc"], cs["u"], cs["v"], cs["w"], cs["hU"][0], cs["hV"][1], cs["hW"][2],
                                 cs["tau"], density=dens, border=cs["p_border"])
    assert st == 0
    np.testing.assert_array_equal(rhs.download(), want)


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_velocity_correct_matches_oracle(ctx, axis):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    g, codes, prev = [(gu, cs["uc"], cs["u"]), (gv, cs["vc"], cs["v"]), (gw, cs["wc"], cs["w"])][axis - 1]
    border = cs["u_border"] if axis == 1 else np.zeros(codes.shape)
    out = g.vec(np.full(g.shape, -5.0))
    xf.velocity_correct(axis, g.vec(prev), gp.vec(cs["p"]), cs["tau"], out, density=gp.vec(cs["density"]),
                        border=g.vec(border))
    want, st, _ = O.velocity_correct(axis, codes, prev, cs["p"], cs["hP"][axis - 1], cs["tau"],
                                     density=cs["density"], border=border, cur=np.full(codes.shape, -5.0))
    assert st == 0
    np.testing.assert_array_equal(out.download(), want)


def test_divergence_max_matches_oracle(ctx):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    got, ijk = xf.divergence_max(gp, gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]))
    want, wijk = O.divergence_max(cs["pc"], cs["u"], cs["v"], cs["w"], cs["hU"][0], cs["hV"][1], cs["hW"][2])
    assert got == want and ijk == wijk
    # a divergence-free field (all zero) reports no cell, as the reference's -1s
    z = xf.divergence_max(gp, gu.vec(np.zeros(gu.shape)), gv.vec(np.zeros(gv.shape)), gw.vec(np.zeros(gw.shape)))
    assert z == (0.0, (-1, -1, -1))


def test_step_errors_match_reference_throws(ctx):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    # a Defined inflow value that differs from the border value
    u = cs["u"].copy()
    cell = tuple(int(t) for t in np.argwhere(cs["uc"] == 3)[5])
    u[cell] += 1e-3
    with pytest.raises(xf.XFError) as e:
        xf.velocity_correct(1, gu.vec(u), gp.vec(cs["p"]), cs["tau"], gu.vec(None), border=gu.vec(cs["u_border"]))
    assert e.value.status == capi.XF_ERR_CHECK and str(cell) in str(e.value)
    _, st, bad = O.velocity_correct(1, cs["uc"], u, cs["p"], cs["hP"][0], cs["tau"], border=cs["u_border"])
    assert st == capi.XF_ERR_CHECK and bad == np.ravel_multi_index(cell, u.shape)
    # a Normal pressure cell: the reference's "not implemented" throw
    pc = cs["pc"].copy()
    pc[3, 4, 5] = 5
    gp2 = xf.Grid(ctx, pc, *cs["hP"])
    with pytest.raises(xf.XFError) as e:
        xf.pressure_rhs(gp2, gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]), cs["tau"], gp2.vec(None))
    assert e.value.status == capi.XF_ERR_MASK and "(3, 4, 5)" in str(e.value)
    _, st, bad = O.pressure_rhs(pc, cs["u"], cs["v"], cs["w"], cs["hU"][0], cs["hV"][1], cs["hW"][2], cs["tau"])
    assert st == capi.XF_ERR_MASK and bad == np.ravel_multi_index((3, 4, 5), pc.shape)
    # mismatched staggered shapes are refused before any launch
    with pytest.raises(xf.XFError):
        xf.pressure_rhs(gp, gv.vec(cs["v"]), gv.vec(cs["v"]), gw.vec(cs["w"]), cs["tau"], gp.vec(None))


def momentum_case(cs, seed=8):
    rng = np.random.Generator(np.random.PCG64(seed))
    vis = rng.uniform(0.01, 0.02, cs["pc"].shape)
    comps = ((1, cs["uc"], cs["hU"]), (2, cs["vc"], cs["hV"]), (3, cs["wc"], cs["hW"]))
    extra = {a: (rng.standard_normal(c.shape), rng.standard_normal(c.shape)) for a, c, _ in comps}
    return vis, comps, extra


@pytest.mark.parametrize("axis", [1, 2, 3])
@pytest.mark.parametrize("with_force", [False, True])
def test_momentum_rhs_matches_oracle(ctx, axis, with_force):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    vis, comps, extra = momentum_case(cs)
    _, codes, hs = comps[axis - 1]
    g = (gu, gv, gw)[axis - 1]
    border, force = extra[axis]
    force = force if with_force else None
    out = xf.momentum_rhs(axis, g, gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]), vis=gp.vec(vis),
                          border=g.vec(border), force=g.vec(force) if force is not None else None)
    want, st, _ = O.momentum_rhs(axis, codes, cs["u"], cs["v"], cs["w"], *hs, vis=vis, border=border, force=force)
    assert st == 0
    for name, o, w_ in zip(("uTr", "vTr", "wTr", "visTr", "rp"), out, want):
        np.testing.assert_array_equal(o.download(), w_, err_msg=name)


def test_momentum_rhs_normal_cells_and_throws(ctx):
    cs = wl_step.staggered_channel()
    gp, gu, gv, gw = grids(ctx, cs)
    uc = cs["uc"].copy()
    nrm = np.zeros(uc.shape + (3,))
    cells = np.argwhere(uc == 4)[:3]
    for c in cells:
        uc[tuple(c)] = 5
        nrm[tuple(c)] = (-1.0, 0.0, 0.0)
    border = np.arange(uc.size, dtype=np.float64).reshape(uc.shape)
    args = (gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]))
    gn = xf.Grid(ctx, uc, *cs["hU"], nrm)
    out = xf.momentum_rhs(1, gn, *args, border=gn.vec(border))
    want, st, _ = O.momentum_rhs(1, uc, cs["u"], cs["v"], cs["w"], *cs["hU"], border=border, normals=nrm)
    assert st == 0
    np.testing.assert_array_equal(out[4].download(), want[4])
    # a normal with a y component: the reference's throw at the first such cell
    nrm[tuple(cells[2])] = (-1.0, 0.25, 0.0)
    nrm[tuple(cells[1])] = (-1.0, 0.0, 0.25)
    gb = xf.Grid(ctx, uc, *cs["hU"], nrm)
    with pytest.raises(xf.XFError) as e:
        xf.momentum_rhs(1, gb, *args, border=gb.vec(border))
    assert e.value.status == capi.XF_ERR_MASK and "(%d, %d, %d)" % tuple(int(t) for t in cells[1]) in str(e.value)
    # Equation and PreNormal cells in the v equation
    for code in (7, 6):
        vc = cs["vc"].copy()
        c = tuple(int(t) for t in np.argwhere(vc == 1)[7])
        vc[c] = code
        gx = xf.Grid(ctx, vc, *cs["hV"])
        with pytest.raises(xf.XFError) as e:
            xf.momentum_rhs(2, gx, *args)
        assert e.value.status == capi.XF_ERR_MASK and "(%d, %d, %d)" % c in str(e.value)
    # wrong staggered shapes are argument errors
    with pytest.raises(xf.XFError) as e:
        xf.momentum_rhs(2, gu, *args)
    assert e.value.status == capi.XF_ERR_ARG


def test_momentum_equation_variable_viscosity(ctx):
    """The u equation end to end: rp from xf_momentum_rhs, the variable-viscosity advection-diffusion rows
    (diffCoefVar = visTr) bit-exact against the oracle (XF_EXACT; the fast rows within 1e-13), and the implicit system (1/tau) u + ... = u_prev/tau + rp
    solved by BiCGStab to its stop rule (max-norm of the true residual <= 1e-5, XSLAE.cpp:712)."""
    cs = wl_step.staggered_channel()
    gp, gu0, gv, gw = grids(ctx, cs)
    vis, comps, extra = momentum_case(cs)
    # the outflow face's PreDefined rows take the semi-sum with their inner neighbour: normal +x
    nrm = np.zeros(cs["uc"].shape + (3,))
    nrm[cs["uc"] == 4] = (1.0, 0.0, 0.0)
    gu = xf.Grid(ctx, cs["uc"], *cs["hU"], nrm)
    uTr, vTr, wTr, visTr, rp = xf.momentum_rhs(1, gu, gu0.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]),
                                               vis=gp.vec(vis), border=gu.vec(cs["u_border"]))
    tau = cs["tau"]
    A = xf.Operator(gu, xf.XF_OP_ADVDIFF)
    A.set_advection(uTr, vTr, wTr, tau, 0.0, xf.XF_ADV_CONVECTIVE | xf.XF_ADV_DIFFUSIVE)
    A.set_diffusion_field(visTr)
    og = O.Grid(cs["uc"], nrm, *cs["hU"])
    rng = np.random.Generator(np.random.PCG64(4))
    x = rng.standard_normal(gu.shape)
    y = gu.vec(None)
    A.apply(gu.vec(x), y, flags=xf.XF_ZERO_INACTIVE | xf.XF_EXACT)
    want = O.apply_advdiff(og, x, uTr.download(), vTr.download(), wTr.download(), tau, 0.0, 3,
                           Dfield=visTr.download())
    sm = og.smask.astype(bool)
    np.testing.assert_array_equal(y.download()[sm], want[sm])
    A.apply(gu.vec(x), y, flags=xf.XF_ZERO_INACTIVE)   # the fast rows (the solver's)
    assert np.abs(y.download()[sm] - want[sm]).max() <= 1e-13 * np.abs(want[sm]).max()
    # the constant form differs once the field is set, and returns when it is cleared
    A.set_diffusion_field(None)
    A.apply(gu.vec(x), y, flags=xf.XF_ZERO_INACTIVE | xf.XF_EXACT)
    np.testing.assert_array_equal(y.download()[sm], O.apply_advdiff(og, x, uTr.download(), vTr.download(),
                                                                     wTr.download(), tau, 0.0, 3)[sm])
    A.set_diffusion_field(visTr)
    # right-hand side u_prev / tau + rp on Actual rows, the border rows' values elsewhere
    b = np.where(cs["uc"] == 1, cs["u"] / tau + rp.download(), rp.download()) * sm
    xv = gu.vec(cs["u"] * sm)
    st = xf.solve(A, xv, gu.vec(b), method=xf.XF_BICGSTAB)
    assert st.status == capi.XF_OK and st.iterations > 0
    r = gu.vec(None)
    A.apply(xv, r, flags=xf.XF_ZERO_INACTIVE)
    assert np.abs(r.download()[sm] - b[sm]).max() <= 1e-5


@pytest.mark.parametrize("seed", [1, 20261203, 0xdeadbeef])
def test_reciprocal_division_is_ieee_bit_for_bit(ctx, seed):
    """The passes divide by spacings and the time step through correctly
    rounded reciprocals and one FMA correction; over 2^26 hashed operand
    pairs (the passes' operand ranges, plus fully random bit patterns) the
    quotient equals the IEEE division's in every bit."""
    assert xf.selftest_division(ctx, 1 << 26, seed) == 0
