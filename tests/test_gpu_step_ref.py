"""The GPU time-step passes against the reference's own time step
(TVPProblem::SolveBySplitting run by oracle/ref_driver,
tests/golden/step_channel.npz), with no restatement in between: pressure
right-hand side (XProblem.cpp:5474-5512), velocity correction
(:5598-5777), control balance (:5782-5829), the momentum right-hand side
(:5088-5419) checked through the reference's own ADI line systems
(:3149-3276), the concentration equation's transfer terms (:5886-5935) and
the upwind advection operator's coefficients checked through its captured
line systems (SolveTransferEquation_, schemeType 1, :1822-1912), and the
device-formatted VTK file (:6132-6345).  Bar:
bit-exact, byte-identical file."""
import os

import numpy as np
import pytest

import step_ref
import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import timeloop as tl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def G():
    return step_ref.load()


def grids(ctx, G):
    return {c: xf.Grid(ctx, G[c + "_codes"], *G["h" + c]) for c in "puvw"}


def test_pressure_rhs_matches_reference_step(ctx, G):
    g = grids(ctx, G)
    rhs = g["p"].vec(np.full(g["p"].shape, 7.0))
    xf.pressure_rhs(g["p"], g["u"].vec(G["int_u"]), g["v"].vec(G["int_v"]), g["w"].vec(G["int_w"]), G["tau"], rhs,
                    density=g["p"].vec(G["dens1"]), border=g["p"].vec(G["p_bc"]))
    got = rhs.download()
    m = G["p_codes"] != 0
    np.testing.assert_array_equal(got[m], G["rhs"][m])


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_velocity_correction_matches_reference_step(ctx, G, axis):
    g = grids(ctx, G)
    c = "uvw"[axis - 1]
    out = g[c].vec(np.zeros(g[c].shape))
    xf.velocity_correct(axis, g[c].vec(G["int_" + c]), g["p"].vec(G["p"]), G["tau"], out,
                        density=g["p"].vec(G["dens1"]), border=g[c].vec(G[c + "_bc"]))
    m = G[c + "_codes"] != 0
    np.testing.assert_array_equal(out.download()[m], G[c][m])


def test_control_balance_matches_reference_step(ctx, G):
    g = grids(ctx, G)
    val, ijk = xf.divergence_max(g["p"], g["u"].vec(G["u"]), g["v"].vec(G["v"]), g["w"].vec(G["w"]))
    assert val == G["div_max"] and ijk == tuple(int(t) for t in G["div_ijk"])


def test_momentum_rhs_matches_reference_line_systems(ctx, G):
    g = grids(ctx, G)
    prev = {c: g[c].vec(G["s1_" + c]) for c in "uvw"}
    vis = g["p"].vec(G["s1_vis"])

    def fields(axis):
        c = "uvw"[axis - 1]
        out = xf.momentum_rhs(axis, g[c], prev["u"], prev["v"], prev["w"], vis=vis, border=g[c].vec(G[c + "_bc"]),
                              force=g[c].vec(G["force_" + c]))
        return tuple(o.download() for o in out)

    for axis, c in ((1, "u"), (2, "v"), (3, "w")):
        m = G[c + "_codes"] == 1
        np.testing.assert_array_equal(fields(axis)[axis - 1][m], G[f"tr_{axis}"][m])
    bad, used = step_ref.line_mismatches(G, fields, O.adi_line_coeffs, O.adi_first_rhs)
    assert all(v == 0 for v in bad.values()), bad
    assert used > 0


def conc_fields(ctx, G):
    """The reference's concentration grid with normals for its PreNormal rows (the outward normal on the box
    faces; along x for the interior corner point that no momentum box interior covers) and the box edges, which
    no line reaches, Fictive; and the device's transfer terms on it."""
    box, nrm = tl.scalar_box(G["p_codes"].shape)
    codes = step_ref.conc_codes(G)
    codes[box == 0] = 0
    for c in zip(*np.nonzero((codes == 6) & (box == 1))):
        assert codes[c[0] - 1, c[1], c[2]] == 1
        nrm[c] = (1.0, 0.0, 0.0)
    gc = xf.Grid(ctx, codes, *G["hp"], nrm)
    g = grids(ctx, G)
    out = xf.conc_transfer(gc, g["u"].vec(G["u"]), g["v"].vec(G["v"]), g["w"].vec(G["w"]))
    return gc, out


def test_conc_transfer_matches_reference_line_systems(ctx, G):
    gc, out = conc_fields(ctx, G)
    got = tuple(o.download() for o in out)
    want, st, _ = O.conc_transfer(step_ref.conc_codes(G), G["u"], G["v"], G["w"])
    assert st == 0
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    bad, rows, used = step_ref.conc_line_mismatches(G, got, O.adi_upwind_coeffs, O.adi_first_rhs_upwind)
    assert all(v == 0 for v in bad.values()), bad
    assert used == len(G["line_m"])


def test_upwind_operator_coefficients_match_reference_lines(ctx, G):
    """The packed form of the upwind operator built on the device from the device's transfer velocities: the
    neighbour coefficient of every Actual row toward m-1 / m+1 along each direction is the captured line's a / c,
    bit for bit (the operator's rows evaluated on unit probes)."""
    gc, (uT, vT, wT, rp) = conc_fields(ctx, G)
    A = xf.Operator(gc, xf.XF_OP_ADVDIFF)
    A.set_advection(uT, vT, wT, G["tau"], 0.0, xf.XF_ADV_CONVECTIVE | xf.XF_ADV_DIFFUSIVE | xf.XF_ADV_UPWIND)
    ptr, cols, vals = xf.PackedOperator(A).csr()
    inv, _ = gc.rn_map()
    cc = step_ref.conc_codes(G)
    n1, n2, n3 = cc.shape
    coef = {}
    for r in range(len(ptr) - 1):
        for t in range(ptr[r], ptr[r + 1]):
            coef[(r, int(cols[t]))] = vals[t]
    lm = G["line_m"]
    off = np.concatenate([[0], np.cumsum(lm + 1)])
    call = sum(len(step_ref.sectors(G[c + "_codes"], d)) for c in "uvw" for d in (1, 2, 3))
    checked = 0
    for direction, step in ((1, (1, 0, 0)), (2, (0, 1, 0)), (3, (0, 0, 1))):
        for cells in step_ref.sectors(cc, direction):
            o = int(off[call])
            for r, cell in enumerate(cells[1:-1], start=2):   # PreNormal ends: row 0 is the extra border row
                row = inv[cell] - 1   # Rn indices are 1-based, the CSR 0-based
                lo = tuple(x - s for x, s in zip(cell, step))
                hi = tuple(x + s for x, s in zip(cell, step))
                assert coef.get((row, inv[lo] - 1), 0.0) == G["line_a"][o + r]
                assert coef.get((row, inv[hi] - 1), 0.0) == G["line_c"][o + r]
                checked += 1
            call += 1
    assert checked == 3 * int((cc == 1).sum())


def test_conc_transfer_reports_the_first_throwing_point(ctx, G):
    cc = step_ref.conc_codes(G)
    cc[0, 3, 4] = 3   # Defined: not implemented for the concentration
    cc[4, 0, 4] = 5
    gc = xf.Grid(ctx, cc, *G["hp"])
    g = grids(ctx, G)
    with pytest.raises(xf.XFError) as e:
        xf.conc_transfer(gc, g["u"].vec(G["u"]), g["v"].vec(G["v"]), g["w"].vec(G["w"]))
    assert e.value.status == xf.capi.XF_ERR_MASK and "(0, 3, 4)" in str(e.value)


def test_vtk_matches_reference_file(ctx, G, tmp_path):
    pc = G["p_codes"]
    hp = G["hp"]
    gp = xf.Grid(ctx, pc, *hp)
    gd = xf.Grid(ctx, step_ref.density_mask(pc), *hp)
    gc = xf.Grid(ctx, step_ref.conc_mask(pc, [G[c + "_codes"] for c in "uvw"]), *hp)
    gn = xf.Grid(ctx, G["n_codes"], *G["hn"])
    g = grids(ctx, G)
    path = os.path.join(tmp_path, "step2_gpu.vtk")
    size = xf.write_vtk(path, gn, G["n_x"], G["n_y"], G["n_z"], g["u"].vec(G["u"]), g["v"].vec(G["v"]),
                        g["w"].vec(G["w"]), gp.vec(G["p"]), gd.vec(G["dens2"]), gc.vec(G["cnc"]), gc.vec(G["vis"]))
    data = open(path, "rb").read()
    assert size == len(data)
    assert data == G["vtk"].tobytes()
