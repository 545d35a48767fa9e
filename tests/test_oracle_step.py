"""The oracle's restatement of the time-step passes (XProblem.cpp:5474-5829)
against an independent vectorised numpy restatement of the same expressions
(parity of these rows is unpinned by the reference: they live inside
TVPProblem::SolveBySplitting, which cannot run alone).  Bit-exact: numpy
evaluates the same FP64 operations in the same order per element."""
import numpy as np

from oracle import oracle as O
from xflow_gb300 import workloads as wl_step


def np_rhs(cs, dens, border):
    pc, u, v, w = cs["pc"], cs["u"], cs["v"], cs["w"]
    hxU, hyV, hzW = cs["hU"][0], cs["hV"][1], cs["hW"][2]
    out = np.zeros(pc.shape)
    i, j, k = np.nonzero(pc == 1)
    d = dens[i, j, k] if dens is not None else np.ones(len(i))
    div = d * d * ((u[i, j, k] - u[i - 1, j, k]) / hxU[i - 1]) + ((v[i, j, k] - v[i, j - 1, k]) / hyV[j - 1]) + \
        ((w[i, j, k] - w[i, j, k - 1]) / hzW[k - 1])
    out[i, j, k] = -(div / cs["tau"])
    out[pc == 4] = border[pc == 4]
    return out


def test_pressure_rhs_restatements_agree():
    cs = wl_step.staggered_channel()
    for dens in (None, cs["density"]):
        got, st, _ = O.pressure_rhs(cs["pc"], cs["u"], cs["v"], cs["w"], cs["hU"][0], cs["hV"][1], cs["hW"][2],
                                    cs["tau"], density=dens, border=cs["p_border"])
        assert st == 0
        np.testing.assert_array_equal(got, np_rhs(cs, dens, cs["p_border"]))


def test_velocity_correct_restatements_agree():
    cs = wl_step.staggered_channel()
    uc, u, p, tau, rho, b = cs["uc"], cs["u"], cs["p"], cs["tau"], cs["density"], cs["u_border"]
    got, st, _ = O.velocity_correct(1, uc, u, p, cs["hP"][0], tau, density=rho, border=b)
    assert st == 0
    want = np.zeros(uc.shape)
    i, j, k = np.nonzero(uc == 1)
    want[i, j, k] = u[i, j, k] - tau * ((p[i + 1, j, k] - p[i, j, k]) / cs["hP"][0][i]) / rho[i, j, k]
    want[uc == 3] = b[uc == 3]
    i, j, k = np.nonzero(uc == 4)   # the outflow face mirrors its i-1 neighbour
    want[i, j, k] = 2 * b[i, j, k] - want[i - 1, j, k]
    np.testing.assert_array_equal(got, want)


def test_divergence_max_restatements_agree():
    cs = wl_step.staggered_channel()
    u, v, w = cs["u"], cs["v"], cs["w"]
    val, ijk = O.divergence_max(cs["pc"], u, v, w, cs["hU"][0], cs["hV"][1], cs["hW"][2])
    i, j, k = np.nonzero(cs["pc"] == 1)   # C order: np.nonzero walks i -> j -> k
    div = ((u[i, j, k] - u[i - 1, j, k]) / cs["hU"][0][i - 1]) + ((v[i, j, k] - v[i, j - 1, k]) / cs["hV"][1][j - 1]) + \
        ((w[i, j, k] - w[i, j, k - 1]) / cs["hW"][2][k - 1])
    q = int(np.argmax(np.abs(div)))   # first occurrence of the maximum
    assert val == np.abs(div)[q] and ijk == (int(i[q]), int(j[q]), int(k[q]))


def np_momentum(axis, codes, u, v, w, vis, hx, hy, hz, border, force):
    """Vectorised restatement of XProblem.cpp:5088-5419 (same FP64 operations per element, same order)."""
    tr = [np.zeros(codes.shape) for _ in range(5)]
    uT, vT, wT, visT, rp = tr
    i, j, k = np.nonzero(codes == 1)
    if axis == 1:
        uT[i, j, k] = u[i, j, k]
        vT[i, j, k] = (v[i, j, k] + v[i + 1, j, k] + v[i, j - 1, k] + v[i + 1, j - 1, k]) / 4
        wT[i, j, k] = (w[i, j, k] + w[i + 1, j, k] + w[i, j, k - 1] + w[i + 1, j, k - 1]) / 4
        visT[i, j, k] = (vis[i, j, k] + vis[i + 1, j, k]) / 2
    elif axis == 2:
        uT[i, j, k] = (u[i, j, k] + u[i, j + 1, k] + u[i - 1, j, k] + u[i - 1, j + 1, k]) / 4
        vT[i, j, k] = v[i, j, k]
        wT[i, j, k] = (w[i, j, k] + w[i, j + 1, k] + w[i, j, k - 1] + w[i, j + 1, k - 1]) / 4
        visT[i, j, k] = (vis[i, j, k] + vis[i, j + 1, k]) / 2
    else:
        uT[i, j, k] = (u[i, j, k] + u[i, j, k + 1] + u[i - 1, j, k] + u[i - 1, j, k + 1]) / 4
        vT[i, j, k] = (v[i, j, k] + v[i, j, k + 1] + v[i, j - 1, k] + v[i, j - 1, k + 1]) / 4
        wT[i, j, k] = w[i, j, k]
        visT[i, j, k] = (vis[i, j, k] + vis[i, j, k + 1]) / 2
    bd = (codes == 3) | (codes == 4) | (codes == 5)
    rp[bd] = border[bd]
    rp[i, j, k] = force[i, j, k]
    ddx, ddy, ddz = hx[i] + hx[i - 1], hy[j] + hy[j - 1], hz[k] + hz[k - 1]
    d = lambda f, di, dj, dk, h: (f[i + di, j + dj, k + dk] - f[i - di, j - dj, k - dk]) / h  # noqa: E731
    step = [(1, 0, 0, ddx), (0, 1, 0, ddy), (0, 0, 1, ddz)][axis - 1]
    dVisX, dVisY, dVisZ = d(visT, 1, 0, 0, ddx), d(visT, 0, 1, 0, ddy), d(visT, 0, 0, 1, ddz)
    dU, dV, dW = d(uT, *step), d(vT, *step), d(wT, *step)
    vel = tr[axis - 1]
    dVelX, dVelY, dVelZ = d(vel, 1, 0, 0, ddx), d(vel, 0, 1, 0, ddy), d(vel, 0, 0, 1, ddz)
    rp[i, j, k] = rp[i, j, k] + (dVisX * (dVelX + dU) + dVisY * (dVelY + dV) + dVisZ * (dVelZ + dW))
    return tr


def test_momentum_rhs_restatements_agree():
    cs = wl_step.staggered_channel()
    rng = np.random.Generator(np.random.PCG64(8))
    vis = rng.uniform(0.01, 0.02, cs["pc"].shape)
    for axis, codes, hs in ((1, cs["uc"], cs["hU"]), (2, cs["vc"], cs["hV"]), (3, cs["wc"], cs["hW"])):
        border = rng.standard_normal(codes.shape)
        force = rng.standard_normal(codes.shape)
        got, st, _ = O.momentum_rhs(axis, codes, cs["u"], cs["v"], cs["w"], *hs, vis=vis, border=border, force=force)
        assert st == 0
        want = np_momentum(axis, codes, cs["u"], cs["v"], cs["w"], vis, *hs, border, force)
        for g, w_ in zip(got, want):
            np.testing.assert_array_equal(g, w_)
        # no force (the base class's GetForce) and no viscosity: rp is the border values only
        got0, st, _ = O.momentum_rhs(axis, codes, cs["u"], cs["v"], cs["w"], *hs, border=border)
        assert st == 0
        assert not got0[4][codes == 1].any() and not got0[3].any()


def test_momentum_rhs_throws_like_reference():
    cs = wl_step.staggered_channel()
    uc = cs["uc"].copy()
    nrm = np.zeros(uc.shape + (3,))
    # Normal u cells along x: accepted for the u equation
    cells = np.argwhere(uc == 4)[:3]
    for c in cells:
        uc[tuple(c)] = 5
        nrm[tuple(c)] = (1.0, 0.0, 0.0)
    border = np.arange(uc.size, dtype=np.float64).reshape(uc.shape)
    out, st, _ = O.momentum_rhs(1, uc, cs["u"], cs["v"], cs["w"], *cs["hU"], border=border, normals=nrm)
    assert st == 0
    assert all(out[4][tuple(c)] == border[tuple(c)] for c in cells)
    # a Normal cell with a y component throws, at the first such cell in i -> j -> k order
    nrm[tuple(cells[1])] = (1.0, 0.5, 0.0)
    nrm[tuple(cells[2])] = (1.0, 0.0, 0.5)
    _, st, bad = O.momentum_rhs(1, uc, cs["u"], cs["v"], cs["w"], *cs["hU"], border=border, normals=nrm)
    assert st == O.XFO_ERR_MASK and bad == np.ravel_multi_index(tuple(cells[1]), uc.shape)
    # Normal cells are not implemented for the v equation; nor Equation / PreNormal cells
    vc = cs["vc"].copy()
    c = tuple(np.argwhere(vc == 1)[7])
    for code in (5, 6, 7, 8, 9):
        vc2 = vc.copy()
        vc2[c] = code
        _, st, bad = O.momentum_rhs(2, vc2, cs["u"], cs["v"], cs["w"], *cs["hV"])
        assert st == O.XFO_ERR_MASK and bad == np.ravel_multi_index(c, vc.shape), code


def test_oracle_fixed6_is_correctly_rounded():
    """The C library's "%f" (the reference's VTK number format) against Python's correctly rounded formatting:
    ties at the sixth decimal go to even, signs of negative zeros and tiny negatives are kept."""
    v = np.array([k / 128 for k in range(-257, 258, 2)] + [-0.0, -1e-9, 1e-300, 2.0 ** 70, 0.1, 5e-7, -5e-7])
    assert O.format_fixed6(v) == "".join("%f\n" % t for t in v).encode()


def test_npy_golden_headers_follow_cnpy():
    """The fixtures written by the reference's cnpy: v1.0 magic, '<f8', C order, shape, and the dict padded with
    spaces so that 10 + its length is a multiple of 16, ending in a newline."""
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for name, shape in (("npy_box_a", (5, 6, 7)), ("npy_box_b", (10, 2, 3)), ("npy_box_c", (130, 129, 3))):
        with open(os.path.join(here, name + ".npy"), "rb") as fh:
            blob = fh.read()
        hl = blob[8] | (blob[9] << 8)
        d = "{'descr': '<f8', 'fortran_order': False, 'shape': (%s), }" % ", ".join(map(str, shape))
        pad = 16 - (10 + len(d)) % 16
        assert blob[:10] == b"\x93NUMPY\x01\x00" + bytes([hl & 255, hl >> 8])
        assert blob[10:10 + hl] == (d + " " * (pad - 1) + "\n").encode()
        assert len(blob) == 10 + hl + 8 * int(np.prod(shape))
