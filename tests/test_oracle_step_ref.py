"""The oracle's restatement of the time-step passes against the reference's
own time step (TVPProblem::SolveBySplitting run by oracle/ref_driver,
tests/golden/step_channel.npz): pressure right-hand side
(XProblem.cpp:5474-5512), velocity correction (:5598-5777), control balance
(:5782-5829), momentum right-hand side (:5088-5419) through the reference's
own ADI line systems (:3149-3276), the concentration equation's transfer
terms (:5886-5935) and upwind line systems (SolveTransferEquation_ with
schemeType 1, :1822-1912), and the VTK file (:6132-6345).  Bar:
bit-exact, byte-identical file."""
import os

import numpy as np

import step_ref
from oracle import oracle as O


def test_pressure_rhs_matches_reference_step():
    G = step_ref.load()
    rhs, st, _ = O.pressure_rhs(G["p_codes"], G["int_u"], G["int_v"], G["int_w"], G["hu"][0], G["hv"][1],
                                G["hw"][2], G["tau"], density=G["dens1"], border=G["p_bc"])
    assert st == 0
    np.testing.assert_array_equal(rhs, G["rhs"])


def test_velocity_correction_matches_reference_step():
    G = step_ref.load()
    for axis, c in ((1, "u"), (2, "v"), (3, "w")):
        cc = G[c + "_codes"]
        got, st, _ = O.velocity_correct(axis, cc, G["int_" + c], G["p"], G["hp"][axis - 1], G["tau"],
                                        density=G["dens1"], border=G[c + "_bc"])
        assert st == 0
        m = cc != 0
        np.testing.assert_array_equal(got[m], G[c][m])
        # the intermediate and the corrected velocity differ: p moved the field
        assert not np.array_equal(G["int_" + c][cc == 1], G[c][cc == 1])


def test_control_balance_matches_reference_step():
    G = step_ref.load()
    val, ijk = O.divergence_max(G["p_codes"], G["u"], G["v"], G["w"], G["hu"][0], G["hv"][1], G["hw"][2])
    assert val == G["div_max"] and ijk == tuple(int(t) for t in G["div_ijk"])


def _momentum(G, axis):
    c = "uvw"[axis - 1]
    out, st, _ = O.momentum_rhs(axis, G[c + "_codes"], G["s1_u"], G["s1_v"], G["s1_w"], *G["h" + c],
                                vis=G["s1_vis"], border=G[c + "_bc"], force=G["force_" + c])
    assert st == 0
    return out


def test_momentum_rhs_matches_reference_transfer_velocities():
    G = step_ref.load()
    for axis, c in ((1, "u"), (2, "v"), (3, "w")):
        tr = _momentum(G, axis)[axis - 1]
        m = G[c + "_codes"] == 1
        np.testing.assert_array_equal(tr[m], G[f"tr_{axis}"][m])


def test_momentum_rhs_and_line_coefficients_match_reference_line_systems():
    G = step_ref.load()
    bad, used = step_ref.line_mismatches(G, lambda a: _momentum(G, a), O.adi_line_coeffs, O.adi_first_rhs)
    assert all(v == 0 for v in bad.values()), bad
    assert 0 < used < len(G["line_m"])   # the rest are the concentration equation's lines


def test_conc_transfer_and_upwind_lines_match_reference_line_systems():
    G = step_ref.load()
    cc = step_ref.conc_codes(G)
    tr, st, _ = O.conc_transfer(cc, G["u"], G["v"], G["w"])
    assert st == 0
    bad, rows, used = step_ref.conc_line_mismatches(G, tr, O.adi_upwind_coeffs, O.adi_first_rhs_upwind)
    assert all(v == 0 for v in bad.values()), bad
    assert all(v == int((cc == 1).sum()) for v in rows.values()), rows
    assert used == len(G["line_m"])   # every captured line system is accounted for
    # the central scheme of the momentum equations does not give these lines
    a, b, c = O.adi_line_coeffs(1, cc, *G["hp"], tr[0], np.zeros(cc.shape), G["tau"])
    a2, b2, c2 = O.adi_upwind_coeffs(1, cc, *G["hp"], tr[0], 0.0, G["tau"])
    m = cc == 1
    assert not np.array_equal(b[m], b2[m])


def test_conc_transfer_throws_where_the_reference_does():
    G = step_ref.load()
    cc = step_ref.conc_codes(G)
    for code, cell, want in ((3, (0, 3, 4), 1), (5, (4, 0, 4), 1), (1, (0, 3, 4), 2), (9, (2, 2, 0), 1)):
        bad_codes = cc.copy()
        bad_codes[cell] = code
        _, st, at = O.conc_transfer(bad_codes, G["u"], G["v"], G["w"])
        assert (st, at) == (want, int(np.ravel_multi_index(cell, cc.shape))), (code, cell)
    # the inlet value lands on PreDefined points of the face i = 0 only
    inl = cc.copy()
    inl[0, 2:5, 3:6] = 4
    inl[-1, 2:5, 3:6] = 4
    val = np.arange(cc.size, dtype=float).reshape(cc.shape)
    (_, _, _, rp), st, _ = O.conc_transfer(inl, G["u"], G["v"], G["w"], inlet=val)
    assert st == 0
    want = np.zeros(cc.shape)
    want[0, 2:5, 3:6] = val[0, 2:5, 3:6]
    np.testing.assert_array_equal(rp, want)


def test_vtk_matches_reference_file(tmp_path):
    G = step_ref.load()
    pc = G["p_codes"]
    path = os.path.join(tmp_path, "step2.vtk")
    O.vtk_write(path, G["n_codes"], G["n_x"], G["n_y"], G["n_z"], G["u"], G["v"], G["w"], pc, G["p"],
                step_ref.density_mask(pc), G["dens2"], step_ref.conc_mask(pc, [G[c + "_codes"] for c in "uvw"]),
                G["cnc"], G["vis"])
    assert open(path, "rb").read() == G["vtk"].tobytes()
