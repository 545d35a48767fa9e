"""Voxelisation of a closed triangle surface into the point-code box: the
device kernel against the oracle's numpy restatement of the same rule (bit
for bit, including meshes whose vertices and edges sit exactly on grid
points), and the restatement against geometry (volume of a sphere, a cube's
half-open faces)."""
import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import workloads as wl


def cube_mesh(lo, hi):
    """Axis-aligned box [lo, hi]^3 as 12 outward triangles."""
    v = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])], float)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    return v, np.array(f, np.int32)


def test_oracle_sphere_volume():
    v, f = wl.icosphere_mesh(3)
    n = 40
    x = (np.arange(n) + 0.5) / n
    out = O.voxelize_mesh(np.ones((n, n, n), np.int32), x, x, x, 0.5 + 0.3 * v, f, 0)
    inside = (out == 0).sum()
    # the subdivided icosahedron is inscribed in the sphere: a little less than its volume
    want = 4 / 3 * np.pi * 0.3 ** 3 * n ** 3
    assert 0.93 * want < inside < 1.0 * want


def test_oracle_cube_half_open():
    """Points on the faces: inside on (lo, hi] along x; along y and z the
    top-left rule keeps exactly one of the two opposite faces."""
    n = 12
    x = np.arange(n, dtype=float)
    v, f = cube_mesh((2, 3, 4), (7, 8, 9))
    out = O.voxelize_mesh(np.zeros((n, n, n), np.int32), x, x, x, v, f, 5)
    ins = np.argwhere(out == 5)
    assert ins[:, 0].min() == 3 and ins[:, 0].max() == 7
    for ax, (lo, hi) in ((1, (3, 8)), (2, (4, 9))):
        span = ins[:, ax].max() - ins[:, ax].min() + 1
        assert span == hi - lo   # one face of each pair counts
    assert len(ins) == 5 * 5 * 5


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere", "aligned_sphere", "cube", "two_spheres"])
def test_gpu_voxelize_matches_oracle(case):
    ctx = xf.Context(0)
    try:
        rng = np.random.Generator(np.random.PCG64(7))
        n1, n2, n3 = 37, 30, 28
        x, y, z = (np.sort(rng.uniform(0, 1, n)) for n in (n1, n2, n3))
        codes = rng.integers(1, 4, (n1, n2, n3)).astype(np.int32)
        if case == "sphere":
            v, f = wl.icosphere_mesh(3)
            v = np.array([0.48, 0.51, 0.47]) + 0.31 * v
        elif case == "aligned_sphere":   # vertices snapped to grid coordinates: exact edge and vertex hits
            v, f = wl.icosphere_mesh(2)
            v = 0.5 + 0.35 * v
            v = np.stack([x[np.abs(x[:, None] - v[None, :, 0]).argmin(0)], y[np.abs(y[:, None] - v[None, :, 1]).argmin(0)],
                          z[np.abs(z[:, None] - v[None, :, 2]).argmin(0)]], 1)
        elif case == "cube":
            v, f = cube_mesh((x[5], y[4], z[3]), (x[30], y[25], z[20]))
        else:
            v1, f1 = wl.icosphere_mesh(3)
            v = np.concatenate([0.3 + 0.2 * v1, 0.7 + 0.2 * v1])
            f = np.concatenate([f1, f1 + len(v1)]).astype(np.int32)
        got = xf.voxelize_mesh(ctx, codes, x, y, z, v, f, 0)
        want = O.voxelize_mesh(codes, x, y, z, v, f, 0)
        np.testing.assert_array_equal(got, want)
        assert (got == 0).any()
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_voxelize_rejects_bad_faces():
    ctx = xf.Context(0)
    try:
        v, f = wl.icosphere_mesh(1)
        f = f.copy()
        f[3, 1] = len(v)
        x = np.linspace(0, 1, 8)
        with pytest.raises(xf.XFError) as e:
            xf.voxelize_mesh(ctx, np.ones((8, 8, 8), np.int32), x, x, x, v, f, 0)
        assert e.value.status == xf.capi.XF_ERR_ARG
    finally:
        ctx.close()
