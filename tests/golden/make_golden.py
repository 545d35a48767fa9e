"""Regenerate the golden fixtures in this folder from the reference itself.

Test infrastructure only.  Builds oracle/_ref/ref_driver (the reference's own
XSLAE/XOperator/XSpace/... sources compiled in place by oracle/Makefile), feeds
it seeded inputs and stores inputs + outputs as .npz files here.  Needs the
reference tree, named by the environment variable XFLOW_REF (build the driver
first: `make -C oracle ref REF=$XFLOW_REF`); the fixtures it writes are what
the tests read, so the tests themselves never need the reference.

    XFLOW_REF=<reference tree> python tests/golden/make_golden.py [pack | npy]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.bagio import read_bag, write_bag  # noqa: E402
from xflow_gb300 import workloads as wl  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def run(task, rec):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_bag(fin, rec)
        if os.environ.get("XF_KEEP_INPUT"):
            write_bag(os.environ["XF_KEEP_INPUT"], rec)
        # One OpenMP thread: ComputeBoundaryForces (XProblem.cpp:8541-8544) races
        # on neighbours' forces when run with more.
        env = dict(os.environ, OMP_NUM_THREADS="1")
        p = subprocess.run([DRIVER, task, fin, fout], capture_output=True, text=True, timeout=300, env=env)
        if p.returncode != 0:
            return None, p.stderr.strip()
        return read_bag(fout), None


def grid_rec(codes, nrm, nodes):
    n1, n2, n3 = codes.shape
    return {
        "dims": np.array([n1, n2, n3], np.int32),
        "x_nodes": nodes[0], "y_nodes": nodes[1], "z_nodes": nodes[2],
        "codes": codes.astype(np.int32).ravel(),
        "normals": nrm.reshape(-1),
    }


def matvec_case(name, codes, nrm, nodes, seed, vardiv=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = codes.shape
    x = rng.standard_normal(shape)
    s = rng.standard_normal(shape)
    # A tie for the abs-max: the first cell in i->j->k order must win.
    act = np.argwhere(wl.space_mask(codes) == 1)
    a, b = act[len(act) // 3], act[2 * len(act) // 3]
    x[tuple(a)], x[tuple(b)] = -7.5, 7.5
    rho = rng.uniform(0.5, 2.0, shape)
    y0 = rng.standard_normal(shape)
    rec = grid_rec(codes, nrm, nodes)
    rec.update({"x": x.ravel(), "s": s.ravel(), "density": rho.ravel(), "y_init": y0.ravel(),
                "p1": np.array([0.75]), "p2": np.array([-1.25])})
    if vardiv:
        rec["vardiv"] = np.array([1], np.int32)
    out, err = run("matvec", rec)
    if out is None:
        raise RuntimeError(f"{name}: {err}")
    inv = np.zeros(codes.size, np.int32)
    sm = wl.space_mask(codes).ravel().astype(bool)
    inv[sm] = np.arange(1, sm.sum() + 1)
    save = dict(codes=codes, normals=nrm, x_nodes=nodes[0], y_nodes=nodes[1], z_nodes=nodes[2],
                x=x, s=s, density=rho, y_init=y0, p1=0.75, p2=-1.25)
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, f"matvec_{name}.npz"), **save)
    print(f"matvec_{name}: end_index={out['end_index'][0]} absmax={out['absmax_x'][0]} idx={out['absmax_x_index'][0]}")


def error_case(name, codes, nrm, nodes):
    """Inputs the reference rejects with a throw (bad codes / normals)."""
    shape = codes.shape
    rec = grid_rec(codes, nrm, nodes)
    z = np.zeros(shape).ravel()
    rec.update({"x": z, "s": z, "density": z + 1, "y_init": z, "p1": np.array([1.0]), "p2": np.array([1.0])})
    out, err = run("matvec", rec)
    return err


def solve_case(name, codes, nrm, nodes, op, method, b, x0, rho=None):
    rec = grid_rec(codes, nrm, nodes)
    rec.update({"op": np.array([op], np.int32), "method": np.array([method], np.int32),
                "x0": x0.ravel(), "b": b.ravel()})
    if rho is not None:
        rec["density"] = rho.ravel()
    out, err = run("solve", rec)
    if out is None:
        raise RuntimeError(f"{name}: {err}")
    save = dict(codes=codes, normals=nrm, x_nodes=nodes[0], y_nodes=nodes[1], z_nodes=nodes[2],
                op=op, method=method, b=b, x0=x0)
    if rho is not None:
        save["density"] = rho
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, f"solve_{name}.npz"), **save)
    print(f"solve_{name}: resid_l2={out['resid_l2'][0]:.3e} resid_inf={out['resid_inf'][0]:.3e}")


def pack_case(name, codes, nrm, nodes, seed, bicg):
    """T1dPackOperator from the Laplace operator: both storages, A x, A^T x and,
    when `bicg`, TSLAE::SolveByBiConjugateGradients on the packed system."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sm = wl.space_mask(codes).astype(bool)
    R = int(sm.sum())
    rec = grid_rec(codes, nrm, nodes)
    rec["x"] = np.zeros(codes.size)
    x_rn = rng.standard_normal(R)
    rec["x_rn"] = x_rn
    b_rn = rng.standard_normal(R)
    if bicg:
        rec["b_rn"] = b_rn
    out, err = run("pack", rec)
    if out is None:
        raise RuntimeError(f"{name}: {err}")
    save = dict(codes=codes, normals=nrm, x_nodes=nodes[0], y_nodes=nodes[1], z_nodes=nodes[2], x_rn=x_rn)
    if bicg:
        save["b_rn"] = b_rn
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, f"pack_{name}.npz"), **save)
    print(f"pack_{name}: rows={R} nnz={len(out['a_vals'])}" + (" bicg ok" if bicg else ""))


def pack_fixtures():
    rng = np.random.Generator(np.random.PCG64(4040))
    codes, nrm = wl.mixed_grid(12, 11, 10, seed=41)
    nodes = [wl.random_nodes(n, rng) for n in codes.shape]
    pack_case("mixed", codes, nrm, nodes, 42, bicg=False)
    codes, nrm = wl.poisson_cube(9, 8, 10)
    nodes = [wl.random_nodes(n, rng) for n in codes.shape]
    pack_case("cube", codes, nrm, nodes, 43, bicg=True)


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True,
                   stdout=subprocess.DEVNULL)
    rng = np.random.Generator(np.random.PCG64(2024))

    # --- operator / vector-algebra / numbering fixtures ---------------------
    for name, shape, seed in (("mixed_a", (12, 11, 10), 11), ("mixed_b", (17, 9, 14), 12)):
        codes, nrm = wl.mixed_grid(*shape, seed=seed)
        nodes = [wl.random_nodes(n, rng) for n in shape]
        matvec_case(name, codes, nrm, nodes, seed + 100)
    for name, shape, seed in (("vardiv_a", (11, 12, 13), 21), ("vardiv_b", (9, 16, 10), 22)):
        codes, nrm = wl.mixed_grid(*shape, seed=seed, face_prenormal=False, interior_rows=12)
        nodes = [wl.random_nodes(n, rng) for n in shape]
        matvec_case(name, codes, nrm, nodes, seed + 100, vardiv=True)
    codes, nrm = wl.poisson_cube(10, 10, 10)
    nodes = [wl.uniform_nodes(-1 / 16, 1 + 1 / 16, 1 / 8)[0]] * 3
    matvec_case("poisson_cube", codes, nrm, nodes, 7)

    # --- inputs the reference rejects ----------------------------------------
    errs = {}
    codes, nrm = wl.mixed_grid(8, 8, 8, seed=5)
    nodes = [wl.random_nodes(8, rng) for _ in range(3)]
    c2 = codes.copy(); c2[3, 3, 3] = wl.NORMAL
    errs["normal_code_active"] = (c2, nrm)
    c2 = codes.copy(); c2[4, 4, 4] = 2
    errs["unknown_code"] = (c2, nrm)
    c2 = codes.copy(); n2 = nrm.copy()
    face = np.argwhere(codes[0] == wl.PREDEFINED)
    if len(face):
        j, k = face[0]
        n2[0, j, k] = (-1.0, 0.5, 0.0)
        errs["predefined_oblique_normal"] = (c2, n2)
    face = np.argwhere(codes[0] == wl.PRENORMAL)
    if len(face):
        j, k = face[0]
        n2 = nrm.copy(); n2[0, j, k] = 0.0
        errs["prenormal_no_normal"] = (c2, n2)
    rec = {}
    for name, (c, n) in errs.items():
        err = error_case(name, c, n, nodes)
        rec[name + "_codes"] = c
        rec[name + "_normals"] = n
        rec[name + "_threw"] = err is not None
        print(f"error case {name}: {err}")
    rec["x_nodes"], rec["y_nodes"], rec["z_nodes"] = nodes
    np.savez_compressed(os.path.join(HERE, "errors.npz"), **rec)

    # --- solver fixtures -------------------------------------------------------
    # SPD system: uniform Neumann box with one Defined (pinned) cell holding 0.
    # (Non-uniform spacings make the flux-form operator nonsymmetric.)
    shape = (11, 10, 9)
    codes, nrm = wl.neumann_box(*shape)
    codes[5, 5, 4] = wl.DEFINED
    nodes = [wl.uniform_nodes(-0.05, 1.05, 0.1)[0][:n] for n in shape]
    b = np.where(codes == wl.ACTUAL, rng.standard_normal(shape), 0.0)
    x0 = np.zeros(shape)
    solve_case("cg_spd", codes, nrm, nodes, 0, 0, b, x0)
    solve_case("minres_spd", codes, nrm, nodes, 0, 2, b, x0)
    # Time-loop style nonsymmetric system (Dirichlet semi-sum rows) by BiCGStab,
    # warm-started from a nonzero x0.
    codes, nrm = wl.poisson_cube(10, 9, 11)
    nodes = [wl.random_nodes(n, rng) for n in codes.shape]
    sm = wl.space_mask(codes).astype(bool)
    b = np.where(sm, rng.standard_normal(codes.shape), 0.0)
    x0 = np.where(sm, 0.1 * rng.standard_normal(codes.shape), 0.0)
    solve_case("bicgstab_cube", codes, nrm, nodes, 0, 1, b, x0)
    # Variable density: PreNormal rows off the faces (see matvec fixtures).
    codes, nrm = wl.mixed_grid(10, 9, 11, seed=31, face_prenormal=False)
    nodes = [wl.random_nodes(n, rng) for n in codes.shape]
    sm = wl.space_mask(codes).astype(bool)
    b = np.where(sm, rng.standard_normal(codes.shape), 0.0)
    x0 = np.where(sm, 0.1 * rng.standard_normal(codes.shape), 0.0)
    rho = rng.uniform(0.8, 1.25, codes.shape)
    solve_case("bicgstab_vardiv", codes, nrm, nodes, 1, 1, b, x0, rho)

    # --- Thomas lines (TSLAE::SolveByScalarRunning) ---------------------------
    nl, M = 7, 12
    a = rng.uniform(-1, 0, (nl, M + 1))
    c = rng.uniform(-1, 0, (nl, M + 1))
    bb = 2.5 + rng.uniform(0, 1, (nl, M + 1))
    f = rng.standard_normal((nl, M + 1))
    u = rng.standard_normal((nl, M + 1))
    out, err = run("thomas", {"nlines": np.array([nl], np.int32), "M": np.array([M], np.int32),
                              "u": u, "a": a, "b": bb, "c": c, "f": f})
    if out is None:
        raise RuntimeError(err)
    np.savez_compressed(os.path.join(HERE, "thomas.npz"), u0=u, a=a, b=bb, c=c, f=f,
                        M=M, ref_u=out["u"].reshape(nl, M + 1))
    print("thomas ok")

    # --- immersed boundary (interpolate, move, forces, spread) ----------------
    n = 20
    shape = (n, n, n)
    hx = 1.0 / (n - 2)
    nodes1 = np.array([i * hx for i in range(n)])
    codes, nrm = wl.neumann_box(*shape)
    nn = 14
    th = np.linspace(0, 2 * np.pi, nn, endpoint=False)
    pos = np.stack([0.5 + 0.2 * np.cos(th), 0.5 + 0.2 * np.sin(th), 0.45 + 0.05 * np.sin(2 * th)], 1)
    pos += 0.01 * rng.standard_normal(pos.shape)
    ref = pos + 0.02 * rng.standard_normal(pos.shape)
    kind = np.array([(0, 1, 2, 3)[q % 4] for q in range(nn)], np.int32)
    nxt = np.array([(q + 1) if q < nn - 1 else -1 for q in range(nn)], np.int32)
    prv = np.array([(q - 1) if q > 0 else -1 for q in range(nn)], np.int32)
    d0 = np.array([np.linalg.norm(pos[q] - pos[nxt[q]]) * 0.9 if nxt[q] >= 0 else 0.0 for q in range(nn)])
    curv0 = 0.01 * rng.standard_normal((nn, 3))
    kst = rng.uniform(50, 150, nn)
    params = np.array([30.0, 1000.0, 5.0, 4 * np.pi * 0.04 / nn])
    vel = rng.standard_normal(shape)
    tau = 1e-3
    for axis in (1, 2, 3):
        rec = grid_rec(codes, nrm, [nodes1] * 3)
        rec.update({"tau": np.array([tau]), "pos": pos.ravel(), "ref": ref.ravel(), "kind": kind,
                    "next": nxt, "prev": prv, "dist0": d0, "curv0": curv0.ravel(), "node_stiff": kst,
                    "params": params, "velocity": vel.ravel(), "axis": np.array([axis], np.int32)})
        out, err = run("ib", rec)
        if out is None:
            raise RuntimeError(err)
        np.savez_compressed(os.path.join(HERE, f"ib_axis{axis}.npz"), codes=codes, nodes=nodes1, tau=tau,
                            pos=pos, ref=ref, kind=kind, next=nxt, prev=prv, dist0=d0, curv0=curv0,
                            node_stiff=kst, params=params, velocity=vel, axis=axis,
                            **{"ref_" + k: v for k, v in out.items()})
        print(f"ib axis {axis}: max|vel|={np.abs(out['node_vel']).max():.3e} "
              f"max|F|={np.abs(out['node_force']).max():.3e} sum f={out['force_box'].sum():.3e}")


def npy_fixtures():
    """NPY files written by the reference's cnpy::npy_save (XProblem.cpp:6545-6590) for three box shapes
    (header dicts of three lengths, so three different space paddings)."""
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, stdout=subprocess.DEVNULL)
    rng = np.random.Generator(np.random.PCG64(77))
    for name, shape in (("npy_box_a", (5, 6, 7)), ("npy_box_b", (10, 2, 3)), ("npy_box_c", (130, 129, 3))):
        data = rng.standard_normal(shape)
        data[0, 0, :2] = (np.inf, -0.0)
        with tempfile.TemporaryDirectory() as td:
            fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            write_bag(fin, {"shape": np.array(shape, np.int32), "data": data.ravel()})
            subprocess.run([DRIVER, "npy", fin, fout], check=True, timeout=60)
            with open(fout + ".npy", "rb") as f:
                blob = f.read()
        with open(os.path.join(HERE, name + ".npy"), "wb") as f:
            f.write(blob)


def step_fixture():
    """Two time steps of the reference's TVPProblem::SolveBySplitting on
    workloads.reference_step_case (ref_driver task `step`), run twice: as
    given, and with the second step's pressure solve replaced by p = 0, which
    makes its velocity correction return the intermediate velocity u_.
    Writes step_channel.npz: the statement, the state after step 1 (the
    inputs of step 2), step 2's pressure right-hand side, corrected
    velocities, control balance, ADI line systems, transfer velocities and
    its VTK file."""
    case = wl.reference_step_case()
    rec = {"params": case["params"], "conc0": case["conc0"].ravel().astype(np.float64)}
    for pre in ("p", "u", "v", "w", "n"):
        codes, xyz, nrm, bc = case[pre]
        rec[pre + "_dims"] = np.array(codes.shape, np.int32)
        rec[pre + "_codes"] = codes.ravel()
        rec[pre + "_x"], rec[pre + "_y"], rec[pre + "_z"] = xyz
        if nrm is not None:
            rec[pre + "_nrm"] = nrm.ravel()
        if bc is not None:
            rec[pre + "_bc"] = bc.ravel()
    for pre, f in zip("uvw", case["force"]):
        rec["force_" + pre] = f.ravel()
    outs = {}
    for zero_p in (0, 1):
        with tempfile.TemporaryDirectory() as td:
            wd = os.path.join(td, "run")
            os.makedirs(wd)
            os.makedirs(os.path.join(td, "Res"))
            fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            write_bag(fin, dict(rec, zero_p=np.array([zero_p], np.int32)))
            # one OpenMP thread (OMP_THREAD_LIMIT caps the step's num_threads(3)
            # regions): the three momentum equations then call the line
            # solver in order, eq 1, 2, 3
            env = dict(os.environ, OMP_NUM_THREADS="1", OMP_THREAD_LIMIT="1")
            p = subprocess.run([DRIVER, "step", fin, fout], capture_output=True, text=True, timeout=600, env=env,
                               cwd=wd)
            if p.returncode != 0:
                raise RuntimeError(f"step: {p.stderr[-2000:]}")
            outs[zero_p] = read_bag(fout)
            vtks = sorted(os.listdir(os.path.join(td, "Res")))
            if zero_p == 0:
                if len(vtks) != 2:
                    raise RuntimeError(f"step: expected two VTK files, got {vtks}")
                # flow0.0000.vtk is step 1; the other is step 2
                outs["vtk"] = open(os.path.join(td, "Res", [v for v in vtks if v != "flow0.0000.vtk"][0]), "rb").read()
    a, b = outs[0], outs[1]
    save = {}
    for pre in ("p", "u", "v", "w", "n"):
        codes, xyz, nrm, bc = case[pre]
        save[pre + "_codes"] = codes
        save[pre + "_x"], save[pre + "_y"], save[pre + "_z"] = xyz
        if nrm is not None:
            save[pre + "_nrm"] = nrm
        if bc is not None:
            save[pre + "_bc"] = bc
    shp = {pre: case[pre][0].shape for pre in ("p", "u", "v", "w")}
    save.update(params=case["params"], conc0=case["conc0"],
                force_u=case["force"][0], force_v=case["force"][1], force_w=case["force"][2])
    # state after step 1 (the inputs of step 2)
    for c in "uvw":
        save["s1_" + c] = a["s1_" + c].reshape(shp[c])
    for k in ("s1_p", "s1_cnc", "s1_vis"):
        save[k] = a[k].reshape(shp["p"])
    # step 2 as given
    save["rhs"] = a["rhs"].reshape(shp["p"])
    save["p0"] = a["p0"].reshape(shp["p"])
    save["p"] = a["p"].reshape(shp["p"])
    for c in "uvw":
        save[c] = a[c].reshape(shp[c])
        save["int_" + c] = b[c].reshape(shp[c])    # intermediate velocity (p = 0 run)
    for q, c in zip((1, 2, 3), "uvw"):
        save[f"tr_{q}"] = a[f"tr_{q}"].reshape(shp[c])
    save["cnc"] = a["cnc"].reshape(shp["p"])
    save["vis"] = a["vis"].reshape(shp["p"])
    save["div_max"] = a["div_max"][0]
    save["div_ijk"] = a["div_ijk"]
    for k in ("line_m", "line_thread", "line_a", "line_b", "line_c", "line_f", "line_u"):
        save[k] = a[k]
    save["vtk"] = np.frombuffer(outs["vtk"], np.uint8)
    # the p = 0 run must agree with the real one up to its pressure solve
    assert np.array_equal(a["rhs"], b["rhs"]) and np.array_equal(a["line_f"][:1000], b["line_f"][:1000])
    np.savez_compressed(os.path.join(HERE, "step_channel.npz"), **save)
    print("step_channel.npz:", {k: np.shape(v) for k, v in save.items() if k.startswith(("line", "vtk", "rhs"))})


if __name__ == "__main__":
    # `make_golden.py pack` / `npy` regenerate only those fixtures
    if sys.argv[1:] == ["pack"]:
        pack_fixtures()
    elif sys.argv[1:] == ["step"]:
        step_fixture()
    elif sys.argv[1:] == ["npy"]:
        npy_fixtures()
    else:
        main()
        pack_fixtures()
        npy_fixtures()
