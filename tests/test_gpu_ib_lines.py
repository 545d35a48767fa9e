"""GPU parity of the immersed-boundary marker kernels and the batched
tridiagonal lines against the reference's golden vectors and the CPU oracle.

Bars: Thomas lines bit-exact (FP64, the reference's operation order); marker
position updates and node forces bit-exact given the same inputs; interpolated
velocities within 1e-14 x max|v| (CUDA's cos against the host libm's, a few
ulp); spread force boxes within 1e-13 x max|f| (cos, plus atomics adding the
markers' contributions to one cell in any order).
"""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from tests.helpers import golden
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def box_grid(ctx, shape):
    codes, nrm = wl.neumann_box(*shape)
    return xf.Grid(ctx, codes, *(np.full(n - 1, 1.0 / (n - 1)) for n in shape), nrm)


# ---------------------------------------------------------------------------
# TSLAE::SolveByScalarRunning (XSLAE.cpp:416-445)
def test_thomas_golden_lines(ctx):
    f = golden("thomas")
    M = int(f["M"])
    nl, L = f["u0"].shape
    assert L == M + 1
    g = box_grid(ctx, (nl, 3, L))
    vecs = {}
    for k in ("u0", "a", "b", "c", "f"):
        box = np.zeros(g.shape)
        box[:, 1, :] = f[k]
        if k == "b":   # the padding lines (j = 0, 2) solve 1 * u = 0
            box[:, 0, :] = box[:, 2, :] = 1.0
        vecs[k] = g.vec(box)
    # the nl lines along k at j = 1: l1 = i (stride s1), one l2, m along k
    s1 = g.shape[1] * g.shape[2]
    u = vecs["u0"]
    base = xf.capi.lib().xf_vec_data(u.h) + 8 * L   # j = 1
    xf.thomas_lines(ctx, M, base, *(xf.capi.lib().xf_vec_data(vecs[k].h) + 8 * L for k in ("a", "b", "c", "f")),
                    nl1=nl, nl2=1, ls1=s1, ls2=0, ms=1)
    ctx.synchronize()
    got = u.download()[:, 1, :]
    np.testing.assert_array_equal(got, f["ref_u"])


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_thomas_box_lines_match_oracle(ctx, axis):
    shape = (9, 12, 14)
    g = box_grid(ctx, shape)
    rng = np.random.Generator(np.random.PCG64(100 + axis))
    a = rng.uniform(-1, 0, shape)
    c = rng.uniform(-1, 0, shape)
    b = 2.5 + rng.uniform(0, 1, shape)   # diagonally dominant
    f = rng.standard_normal(shape)
    u0 = rng.standard_normal(shape)
    vu, va, vb, vc, vf = (g.vec(v) for v in (u0, a, b, c, f))
    M, nl1, nl2, ls1, ls2, ms = xf.box_lines(shape, axis)
    xf.thomas_lines(ctx, M, vu, va, vb, vc, vf, nl1, nl2, ls1, ls2, ms)
    ctx.synchronize()
    got = vu.download()
    want = u0.copy()
    ax = axis - 1
    mv = lambda t: np.moveaxis(t, ax, -1)  # noqa: E731
    W, A, B, Cc, F = mv(want), mv(a), mv(b), mv(c), mv(f)
    for idx in np.ndindex(W.shape[:-1]):
        W[idx] = O.thomas(M, W[idx], A[idx], B[idx], Cc[idx], F[idx])
    np.testing.assert_array_equal(got, want)


# ---------------------------------------------------------------------------
# Immersed boundary (XProblem.cpp:8436-8894)
def markers_from(ctx, f, pos=None):
    return xf.Markers(ctx, f["pos"] if pos is None else pos, f["ref"], f["kind"], f["next"], f["prev"], f["dist0"],
                      f["curv0"], f["node_stiff"], f["params"])


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_ib_golden_step(ctx, axis):
    f = golden(f"ib_axis{axis}")
    nodes = f["nodes"]
    h0 = np.array([nodes[1] - nodes[0]] * 3)
    sep = np.diff(nodes)
    g = xf.Grid(ctx, f["codes"], sep, sep, sep, None)
    vel = g.vec(f["velocity"])
    mk = markers_from(ctx, f)
    a = axis - 1
    # Interpolate
    mk.interpolate(vel, h0, axis)
    v = mk.get(xf.XF_IB_VEL)[a]
    ref_v = f["ref_node_vel"]
    assert np.abs(v - ref_v).max() <= 1e-14 * np.abs(ref_v).max()
    # UpdateBoundaryPosition, from the reference's own node velocities: bit-exact
    vv = mk.get(xf.XF_IB_VEL)
    vv[a] = ref_v
    mk.set(xf.XF_IB_VEL, vv)
    mk.update_position(axis, float(f["ref_tau_eff"][0]))
    np.testing.assert_array_equal(mk.get(xf.XF_IB_POS).ravel(), f["ref_pos_after"])
    # ComputeBoundaryForces: bit-exact
    mk.compute_forces(axis)
    np.testing.assert_array_equal(mk.get(xf.XF_IB_FORCE)[a], f["ref_node_force"])
    # SpreadForce
    fb = g.vec(np.full(g.shape, 7.0))   # stale contents: the call zeroes the box first
    mk.spread(fb, h0, axis)
    got = fb.download().ravel()
    ref = f["ref_force_box"]
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def ring_markers(n, centre, radius, seed):
    """n markers on a tilted circle, linked next/prev as a ring, with every node kind."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = np.stack([centre[0] + radius * np.cos(t), centre[1] + radius * np.sin(t),
                    centre[2] + 0.3 * radius * np.sin(2 * t)], 1)
    ref = pos + rng.normal(0, 0.01 * radius, pos.shape)
    pos = pos + rng.normal(0, 0.005 * radius, pos.shape)
    kind = (np.arange(n) % 5).astype(np.int32)
    nxt = ((np.arange(n) + 1) % n).astype(np.int32)
    prv = ((np.arange(n) - 1) % n).astype(np.int32)
    nxt[n // 3] = -1   # an open chain end
    prv[n // 3 + 1] = -1
    dist0 = np.linalg.norm(pos - pos[nxt], axis=1) * rng.uniform(0.9, 1.1, n)
    curv0 = rng.normal(0, 1e-3, (n, 3))
    stiff = rng.uniform(0.5, 2.0, n)
    params = np.array([3.0, 2.0, 0.5, 1e-3])
    return pos, ref, kind, nxt, prv, dist0, curv0, stiff, params


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_ib_ring_matches_oracle(ctx, axis):
    n = 40
    shape = (n + 1,) * 3
    h = 1.0 / n
    h0 = np.array([h, h, h])
    g = box_grid(ctx, shape)
    rng = np.random.Generator(np.random.PCG64(7 + axis))
    vel = rng.standard_normal(shape)
    m = ring_markers(500, (0.5, 0.5, 0.5), 0.3, 11 + axis)
    mk = xf.Markers(ctx, *m)
    a = axis - 1
    mk.interpolate(g.vec(vel), h0, axis)
    v = mk.get(xf.XF_IB_VEL)[a]
    ov = O.ib_interpolate(vel, h0, axis, m[0])
    assert np.abs(v - ov).max() <= 1e-14 * np.abs(ov).max()
    vv = mk.get(xf.XF_IB_VEL)
    vv[a] = ov
    mk.set(xf.XF_IB_VEL, vv)
    mk.update_position(axis, 2e-3)
    pos2 = O.ib_update(axis, 2e-3, ov, m[0])
    np.testing.assert_array_equal(mk.get(xf.XF_IB_POS), pos2)
    mk.compute_forces(axis)
    oF = O.ib_forces(axis, pos2, *m[1:])
    np.testing.assert_array_equal(mk.get(xf.XF_IB_FORCE)[a], oF)
    fb = g.vec(None)
    mk.spread(fb, h0, axis)
    ob = O.ib_spread(shape, h0, axis, pos2, oF)
    assert np.abs(fb.download() - ob).max() <= 1e-13 * np.abs(ob).max()


def test_ib_rejects_bad_input(ctx):
    m = list(ring_markers(10, (0.5, 0.5, 0.5), 0.3, 1))
    m[2] = m[2].copy()
    m[2][3] = 9   # unknown node kind
    with pytest.raises(xf.XFError):
        xf.Markers(ctx, *m)
    m = list(ring_markers(10, (0.5, 0.5, 0.5), 0.3, 1))
    m[3] = m[3].copy()
    m[3][0] = 10   # neighbour outside the list
    with pytest.raises(xf.XFError):
        xf.Markers(ctx, *m)
    mk = xf.Markers(ctx, *ring_markers(10, (0.5, 0.5, 0.5), 0.3, 1))
    g = box_grid(ctx, (6, 6, 6))   # smaller than the 7-point delta stencil
    with pytest.raises(xf.XFError):
        mk.interpolate(g.vec(None), np.array([0.2] * 3), 1)
    with pytest.raises(xf.XFError):
        mk.compute_forces(4)
