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
