"""The GPU time-step passes against the reference's own time step
(TVPProblem::SolveBySplitting run by oracle/ref_driver,
tests/golden/step_channel.npz), with no restatement in between: pressure
right-hand side (XProblem.cpp:5474-5512), velocity correction
(:5598-5777), control balance (:5782-5829), the momentum right-hand side
(:5088-5419) checked through the reference's own ADI line systems
(:3149-3276), and the device-formatted VTK file (:6132-6345).  Bar:
bit-exact, byte-identical file."""
import os

import numpy as np
import pytest

import step_ref
import xflow_gb300 as xf
from oracle import oracle as O

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
