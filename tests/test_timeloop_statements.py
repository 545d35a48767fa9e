"""The time loop's statements (xflow_gb300.timeloop) and the CPU
restatement of its outflow pass (tests/timeloop_cpu.py), on the CPU: the
concentration grid validates as an operator grid, the Gaussian inlet, the
channel's outflow and wall options, and the convective outflow's flux
balance."""
import numpy as np

import timeloop_cpu
from oracle import oracle as O
from xflow_gb300 import timeloop as tl


def test_scalar_box_is_a_valid_operator_grid():
    shape = (14, 9, 11)
    inlet = np.zeros(shape[1:], bool)
    inlet[3:6, 4:8] = True
    codes, nrm = tl.scalar_box(shape, inlet)
    st, bad = O.validate(O.LAPLACE, codes, nrm)
    assert st == 0, bad
    assert (codes[1:-1, 1:-1, 1:-1] == tl.ACTUAL).all()
    # inlet points on the face i = 0 only, PreNormal elsewhere on the faces, Fictive box edges
    assert (codes[0][inlet[:, :] & (codes[0] != tl.FICTIVE)] == tl.PREDEFINED).all()
    assert (codes[-1, 1:-1, 1:-1] == tl.PRENORMAL).all()
    for e in (codes[0, 0, :], codes[-1, :, -1], codes[:, 0, 0]):
        assert (e == tl.FICTIVE).all()
    # outward normals on the faces
    assert (nrm[-1, 1:-1, 1:-1, 0] == 1).all() and (nrm[1:-1, 0, 1:-1, 1] == -1).all()


def test_gaussian_inlet_and_with_scalar():
    st = tl.channel(16, 8, 8, outflow="convective")
    g = tl.gaussian_inlet(st["p"][0].shape, st["h"], sigma=0.05)
    j, k = np.unravel_index(g.argmax(), g.shape)
    y, z = (j - 0.5) / 8, (k - 0.5) / 8
    assert abs(y - 0.5) <= 1 / 16 + 1e-12 and abs(z - 0.5) <= 1 / 16 + 1e-12
    assert 0 < g.min() and g.max() <= 1
    sc = tl.with_scalar(st, g, schmidt=2.0)["scalar"]
    assert sc["D"] == st["vis"] / 2.0
    pre = sc["codes"] == tl.PREDEFINED
    assert pre[0].sum() == 8 * 8 and not pre[1:].any()   # the whole inlet face inside the edges
    np.testing.assert_array_equal(sc["inlet"][0][pre[0]], g[pre[0]])
    assert (sc["inlet"][1:] == 0).all() and (sc["c0"] == 0).all()


def test_channel_outflow_and_wall_options():
    zg = tl.channel(16, 8, 8)
    cv = tl.channel(16, 8, 8, outflow="convective", walls="free_slip")
    assert zg["pressure"] == "outlet" and (zg["p"][0][-1, 1:-1, 1:-1] == tl.PREDEFINED).all()
    assert cv["pressure"] == "neumann" and (cv["p"][0][-1] == tl.FICTIVE).all()
    uc = cv["comps"][0][0]
    assert (uc[-1, 1:-1, 1:-1] == tl.DEFINED).all() and cv["convective"] == (1, 1.0)
    assert set(cv["follow"]) == {(1, 1), (2, 0), (2, 1), (3, 0), (3, 1)}
    try:
        tl.channel(16, 8, 8, walls="slip")
        raise AssertionError("an unknown wall option must be refused")
    except ValueError:
        pass


def test_convective_outflow_balances_the_flux():
    st = tl.channel(16, 8, 8, outflow="convective")
    codes, _, bc = st["comps"][0]
    hp = st["p"][3]
    h = [0.5 * (hp[0][:-1] + hp[0][1:]), hp[1], hp[2]]
    rng = np.random.Generator(np.random.PCG64(3))
    vel = np.where(codes == tl.ACTUAL, 1 + 0.2 * rng.standard_normal(codes.shape), 0.0)
    bc = bc.copy()
    bc[0, 1:-1, 1:-1] = 1 + 0.1 * rng.standard_normal((8, 8))   # a non-uniform inflow
    timeloop_cpu.outflow_convective(codes, vel, bc, h, 1, 1.0, st["tau"])
    inflow, outflow = bc[0, 1:-1, 1:-1].sum(), bc[-1, 1:-1, 1:-1].sum()   # uniform face cells
    assert abs(outflow - inflow) <= 1e-12 * abs(inflow)
    # a uniform state is left as it is
    bc2 = np.where(codes == tl.DEFINED, st["comps"][0][2], 0.0)
    u = np.where(codes == tl.ACTUAL, 1.0, bc2)
    before = bc2.copy()
    timeloop_cpu.outflow_convective(codes, u, bc2, h, 1, 1.0, st["tau"])
    np.testing.assert_allclose(bc2, before, rtol=0, atol=1e-14)
