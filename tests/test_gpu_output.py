"""Field output against the oracle and the reference: the device-formatted
VTK volume (XProblem.cpp:6132-6345) byte for byte against the reference's
loops and format strings run through the C library's fprintf; "%f" of hard
values (ties at the sixth decimal, subnormals, huge magnitudes, signed zeros,
non-finite values) against the C library; NPY files byte for byte against
files the reference's own cnpy::npy_save wrote (tests/golden/npy_box_*.npy).
"""
import os

import numpy as np
import pytest

import xflow_gb300 as xf
from oracle import oracle as O
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def hard_values(seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    v = [0.0, -0.0, 1.0, -1.0, 0.5, 1e-7, -1e-7, 4.9e-7, 5e-7, 5.000001e-7, -5e-7, 1.5e-6, 2.5e-6,
         np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
         -1.7976931348623157e308, 2.0 ** 53, 2.0 ** 63, 2.0 ** 64, 18446744073709.0, 18446744073710.0,
         9.2e12, 1e13, 1e15 + 0.3, 123456789.0078125, 0.1, 0.2, 0.3, 1 / 3, 2 / 3]
    v += [k / 128 for k in range(-257, 258, 2)]              # exact ties at the sixth decimal
    v += [k / 2.0 ** 20 for k in range(1, 2000, 37)]
    v += list(rng.standard_normal(500))
    v += list(rng.standard_normal(500) * 10.0 ** rng.integers(-12, 40, 500))
    v += list(np.ldexp(rng.random(200), rng.integers(-1074, 1024, 200)))
    return np.array(v)


def test_format_fixed6_matches_c_library(ctx):
    v = hard_values()
    assert xf.format_fixed6(ctx, v) == O.format_fixed6(v)
    assert xf.format_fixed6(ctx, np.zeros(0)) == b""


def vtk_case(seed=3):
    cs = wl.staggered_channel(seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed + 10))
    pc = cs["pc"]
    n1, n2, n3 = pc.shape
    node_codes = pc[:-1, :-1, :-1].copy()
    node_codes[0] = 3                                          # non-Fictive node faces
    x = np.concatenate([[0.0], np.cumsum(cs["hP"][0][:n1 - 2])])
    y = np.concatenate([[0.0], np.cumsum(cs["hP"][1][:n2 - 2])])
    z = np.concatenate([[0.0], np.cumsum(cs["hP"][2][:n3 - 2])])
    dc = np.where(pc == 4, 0, pc)                              # density grid: PreDefined -> Fictive
    cc = pc.copy()
    cc[1:-1, 0, 1:-1] = 6                                      # concentration grid: PreNormal side walls
    p = rng.standard_normal(pc.shape)
    p[2, 2, 2:6] = (1 / 128, -0.0, -1e-9, 3 / 128)
    fields = dict(p=p, density=rng.uniform(0.5, 2.0, pc.shape), conc=rng.random(pc.shape),
                  vis=rng.uniform(0.01, 0.02, pc.shape))
    return cs, node_codes, (x, y, z), dc, cc, fields


def test_vtk_matches_reference_writer(ctx, tmp_path):
    cs, node_codes, (x, y, z), dc, cc, f = vtk_case()
    gp = xf.Grid(ctx, cs["pc"], *cs["hP"])
    gd = xf.Grid(ctx, dc, *cs["hP"])
    gc = xf.Grid(ctx, cc, *cs["hP"])
    gn = xf.Grid(ctx, node_codes, *(np.diff(a) for a in (x, y, z)))
    gu = xf.Grid(ctx, cs["uc"], *cs["hU"])
    gv = xf.Grid(ctx, cs["vc"], *cs["hV"])
    gw = xf.Grid(ctx, cs["wc"], *cs["hW"])
    path_gpu, path_ref = tmp_path / "gpu.vtk", tmp_path / "ref.vtk"
    size = xf.write_vtk(path_gpu, gn, x, y, z, gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"]), gp.vec(f["p"]),
                        gd.vec(f["density"]), gc.vec(f["conc"]), gc.vec(f["vis"]))
    O.vtk_write(path_ref, node_codes, x, y, z, cs["u"], cs["v"], cs["w"], cs["pc"], f["p"], dc, f["density"], cc,
                f["conc"], f["vis"])
    got, want = path_gpu.read_bytes(), path_ref.read_bytes()
    assert size == len(got)
    assert got == want


def test_vtk_rejects_bad_shapes(ctx, tmp_path):
    cs, node_codes, (x, y, z), dc, cc, f = vtk_case()
    gp = xf.Grid(ctx, cs["pc"], *cs["hP"])
    gn = xf.Grid(ctx, node_codes, *(np.diff(a) for a in (x, y, z)))
    gu = xf.Grid(ctx, cs["uc"], *cs["hU"])
    vp = gp.vec(f["p"])
    with pytest.raises(xf.XFError):   # u passed where v belongs
        xf.write_vtk(tmp_path / "bad.vtk", gn, x, y, z, gu.vec(cs["u"]), gu.vec(cs["u"]), gu.vec(cs["u"]), vp, vp,
                     vp, vp)


@pytest.mark.parametrize("name", ["npy_box_a", "npy_box_b", "npy_box_c"])
def test_npy_matches_reference_cnpy(ctx, tmp_path, name):
    golden = os.path.join(GOLDEN, name + ".npy")
    data = np.load(golden)
    g = xf.Grid(ctx, np.ones(data.shape, np.int32), *(np.ones(n - 1) for n in data.shape))
    out = tmp_path / "x.npy"
    xf.write_npy(out, g.vec(data))
    with open(golden, "rb") as fh:
        assert out.read_bytes() == fh.read()
    # single precision: numpy reads back the FP32 box
    v32 = g.vec(data, xf.XF_F32)
    xf.write_npy(out, v32)
    np.testing.assert_array_equal(np.load(out), data.astype(np.float32))
