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
