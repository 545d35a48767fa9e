"""Pins the CPU oracle (oracle/xf_oracle.c) to golden vectors produced by the
reference's own compiled classes (tests/golden/make_golden.py).

Operator, vector algebra and numbering must be bit-exact: with one thread the
oracle follows the reference's loop and operation order.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import golden, golden_names, seps
from xflow_gb300 import workloads as wl

MATVEC = golden_names("matvec_")


@pytest.fixture(autouse=True)
def _one_thread():
    O.set_threads(1)
    yield
    O.set_threads(1)


def grid_of(f, with_density=True):
    hx, hy, hz = seps(f)
    return O.Grid(f["codes"], f["normals"], hx, hy, hz, f["density"] if with_density and "density" in f else None)


@pytest.mark.parametrize("name", MATVEC)
def test_space_mask_and_rn_numbering(name):
    f = golden(name)
    g = grid_of(f)
    np.testing.assert_array_equal(g.smask, wl.space_mask(f["codes"]))
    R, inv, fwd = O.rn_map(g.smask)
    assert R == int(f["ref_end_index"][0])
    # x read back through the reference's Rn indexing (TRnSpace::operator[]).
    x = f["x"].ravel()
    np.testing.assert_array_equal(x[inv.ravel() > 0][np.argsort(inv.ravel()[inv.ravel() > 0])], f["ref_x_by_rn"])
    np.testing.assert_array_equal(x[np.ravel_multi_index(fwd.T, f["codes"].shape)], f["ref_x_by_rn"])


@pytest.mark.parametrize("name", MATVEC)
def test_laplace_apply_bit_exact(name):
    f = golden(name)
    g = grid_of(f)
    y = O.apply(O.LAPLACE, g, f["x"], y_init=f["y_init"])
    np.testing.assert_array_equal(y.ravel(), f["ref_lap_y"])
    y = O.apply(O.LAPLACE, g, f["x"], f["s"], +1, y_init=f["y_init"])
    np.testing.assert_array_equal(y.ravel(), f["ref_lap_y_plus"])
    y = O.apply(O.LAPLACE, g, f["x"], f["s"], -1, y_init=f["y_init"])
    np.testing.assert_array_equal(y.ravel(), f["ref_lap_y_minus"])


@pytest.mark.parametrize("name", [n for n in MATVEC if "vardiv" in n])
def test_vardiv_apply_bit_exact(name):
    f = golden(name)
    g = grid_of(f)
    y = O.apply(O.VARDIV, g, f["x"], y_init=f["y_init"])
    np.testing.assert_array_equal(y.ravel(), f["ref_vd_y"])


@pytest.mark.parametrize("name", MATVEC)
def test_vector_algebra_bit_exact(name):
    f = golden(name)
    g = grid_of(f)
    m, y0, x, s, p1, p2 = g.smask, f["y_init"], f["x"], f["s"], float(f["p1"]), float(f["p2"])
    np.testing.assert_array_equal(O.lincomb(p1, x, p2, s, m, y0).ravel(), f["ref_lc_p1x_p2s"])
    np.testing.assert_array_equal(O.lincomb(1.0, x, -1.0, s, m, y0).ravel(), f["ref_lc_x_minus_s"])
    np.testing.assert_array_equal(O.lincomb(1.0, x, p2, s, m, y0).ravel(), f["ref_lc_x_p2s"])
    np.testing.assert_array_equal(O.lincomb(p1, x, 0.0, None, m, y0).ravel(), f["ref_lc_p1x"])
    np.testing.assert_array_equal(O.lincomb(0.0, x, 0.0, None, m, y0).ravel(), f["ref_lc_zero"])
    # TSpace::Assign copies the whole box, inactive cells included (XSpace.cpp:2343-2361).
    np.testing.assert_array_equal(x.ravel(), f["ref_assign_x"])
    assert O.dot(x, s, m) == f["ref_dot_xs"][0]
    assert O.norm(x, m) == f["ref_norm_x"][0]
    As = O.apply(O.LAPLACE, g, s)
    # (x, A s): the reference multiplies each entry as it evaluates the row.
    assert O.dot(x, As, m) == f["ref_dot_x_As"][0]
    _, inv, _ = O.rn_map(m)
    v, idx = O.absmax(x, m, inv)
    assert (v, idx) == (f["ref_absmax_x"][0], f["ref_absmax_x_index"][0])
    v, idx = O.absmax(s, m, inv)
    assert (v, idx) == (f["ref_absmax_s"][0], f["ref_absmax_s_index"][0])
    # The reference's abs-min starts from 0 and never moves (XSpace.cpp:3464-3471).
    assert (f["ref_absmin_x"][0], f["ref_absmin_x_index"][0]) == (0.0, 1)


def test_rejected_inputs_match_reference_throws():
    f = golden("errors")
    names = sorted({k[: -len("_threw")] for k in f if k.endswith("_threw")})
    assert names
    for n in names:
        st, bad = O.validate(O.LAPLACE, f[n + "_codes"], f[n + "_normals"])
        assert bool(f[n + "_threw"]) and st != 0, n


def _solve_fixture(name):
    f = golden(name)
    hx, hy, hz = seps(f)
    g = O.Grid(f["codes"], f["normals"], hx, hy, hz, f.get("density"))
    return f, g


@pytest.mark.parametrize("name,fn,norm", [
    ("solve_cg_spd", O.cg_reference, 2),
    ("solve_minres_spd", O.minres_reference, 2),
    ("solve_bicgstab_cube", O.bicgstab_reference, np.inf),
    ("solve_bicgstab_vardiv", O.bicgstab_reference, np.inf),
])
def test_reference_solvers(name, fn, norm):
    f, g = _solve_fixture(name)
    op = int(f["op"])
    x, st = fn(op, g, f["x0"], f["b"], maxit=200000)
    assert st.status == 0
    # Same arithmetic sequence with one thread: identical iterate.
    np.testing.assert_array_equal(x.ravel(), f["ref_result"])
    r = O.apply(op, g, x, f["b"], -1)
    m = g.smask.astype(bool)
    nr = np.linalg.norm(r[m], ord=norm)
    ref = f["ref_resid_l2"][0] if norm == 2 else f["ref_resid_inf"][0]
    assert nr == pytest.approx(ref, rel=1e-12, abs=0)


def test_thomas_lines():
    f = golden("thomas")
    M = int(f["M"])
    for l in range(f["u0"].shape[0]):
        u = O.thomas(M, f["u0"][l], f["a"][l], f["b"][l], f["c"][l], f["f"][l])
        np.testing.assert_array_equal(u, f["ref_u"][l])


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_immersed_boundary_steps(axis):
    f = golden(f"ib_axis{axis}")
    nodes = f["nodes"]
    h0 = np.array([nodes[1] - nodes[0]] * 3)
    pos = f["pos"]
    vel = O.ib_interpolate(f["velocity"], h0, axis, pos)
    np.testing.assert_array_equal(vel, f["ref_node_vel"])
    pos2 = O.ib_update(axis, float(f["ref_tau_eff"][0]), vel, pos)
    np.testing.assert_array_equal(pos2.ravel(), f["ref_pos_after"])
    F = O.ib_forces(axis, pos2, f["ref"], f["kind"], f["next"], f["prev"], f["dist0"], f["curv0"],
                    f["node_stiff"], f["params"])
    np.testing.assert_array_equal(F, f["ref_node_force"])
    box = O.ib_spread(f["codes"].shape, h0, axis, pos2, F)
    np.testing.assert_array_equal(box.ravel(), f["ref_force_box"])


@pytest.mark.parametrize("name", golden_names("pack_"))
def test_pack_operator_and_bicg(name):
    """T1dPackOperator storages, A x / A^T x and the reference BiCG (the
    reference's own outputs) against the oracle's restatement: bit-exact."""
    f = golden(name)
    hx, hy, hz = seps(f)
    g = O.Grid(f["codes"], f["normals"], hx, hy, hz)
    pk = O.pack_build(O.LAPLACE, g)
    for side, key in ((pk.a, "a"), (pk.t, "t")):
        np.testing.assert_array_equal(side[0], f[f"ref_{key}_ptr"])
        np.testing.assert_array_equal(side[1], f[f"ref_{key}_cols"])
        np.testing.assert_array_equal(side[2], f[f"ref_{key}_vals"])
    np.testing.assert_array_equal(O.pack_apply(pk, f["x_rn"]), f["ref_ax"])
    np.testing.assert_array_equal(O.pack_apply(pk, f["x_rn"], transpose=True), f["ref_atx"])
    if "b_rn" in f:
        x, st, rc = O.bicg_reference(pk, f["b_rn"])
        assert rc == 0 and st.status == 0
        np.testing.assert_array_equal(x, f["ref_bicg_x"])
