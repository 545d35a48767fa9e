"""Synthetic grids and right-hand sides for the pressure-projection path.

Every array follows the reference's box convention: a grid of N intervals per
axis has N+1 nodes, arrays are indexed [i][j][k] with k fastest (C order), and
the integer mask holds the reference's point codes
  0 Fictive, 1 Actual (XMask.h:6-7), 3 Defined, 4 PreDefined, 5 Normal,
  6 PreNormal, 7 Equation, 8 PreEquation (XOperator.h:13-18).
Normals are float64 (n1, n2, n3, 3); all-zero means "no normal" (NULL in the
reference's T3dVector**** table, XGrid.h:279-299).

Inputs are made on the host with numpy's PCG64 so that the oracle and the GPU
see bit-identical data.
"""
from __future__ import annotations

import math

import numpy as np

FICTIVE, ACTUAL, DEFINED, PREDEFINED, NORMAL, PRENORMAL, EQUATION, PREEQUATION = 0, 1, 3, 4, 5, 6, 7, 8


def uniform_nodes(start: float, end: float, h: float):
    """Node coordinates and separations of TUniformSeparator (XSeparator.cpp:25-64):
    the step is shrunk so that the interval divides evenly."""
    res = (end - start) / h
    ipart = math.floor(res)
    n = int(ipart)
    if abs(res - ipart) > 1e-11:
        n += 1
    step = (end - start) / float(n)
    dims = np.empty(n + 1)
    dims[0] = start
    for i in range(1, n):
        dims[i] = dims[i - 1] + step
    dims[n] = end
    sep = np.full(n, step)
    return dims, sep


def space_mask(codes: np.ndarray) -> np.ndarray:
    """Grid codes -> space mask {0,1} as XProblem.cpp:4155-4182."""
    act = np.isin(codes, (ACTUAL, PREDEFINED, NORMAL, PRENORMAL, PREEQUATION))
    return act.astype(np.uint8)


def neumann_box(n1: int, n2: int, n3: int):
    """Interior Actual, ghost layer Fictive (homogeneous Neumann walls)."""
    codes = np.zeros((n1, n2, n3), np.int32)
    codes[1:-1, 1:-1, 1:-1] = ACTUAL
    return codes, np.zeros((n1, n2, n3, 3))


def poisson_cube(n1: int, n2: int, n3: int):
    """Mask codes and normals of the reference's verification grid
    (T3dPoissonProblem, XProblem.cpp:431-519): PreDefined rows on the z faces
    (PreNormal on their rim), PreNormal on the x and y faces."""
    N, L, M = n1 - 1, n2 - 1, n3 - 1
    codes = np.zeros((n1, n2, n3), np.int32)
    nrm = np.zeros((n1, n2, n3, 3))
    for i in range(n1):
        for j in range(n2):
            for k in range(n3):
                if i not in (0, N) and j not in (0, L) and k not in (0, M):
                    codes[i, j, k] = ACTUAL
                    continue
                inner_ij = i not in (0, N) and j not in (0, L)
                if inner_ij and k in (0, M):
                    rim = i in (1, N - 1) or j in (1, L - 1)
                    codes[i, j, k] = PRENORMAL if rim else PREDEFINED
                    nrm[i, j, k] = (0, 0, -1 if k == 0 else 1)
                elif i in (0, N) and j not in (0, L) and k not in (0, M):
                    codes[i, j, k] = PRENORMAL
                    nrm[i, j, k] = (-1 if i == 0 else 1, 0, 0)
                elif j in (0, L) and i not in (0, N) and k not in (0, M):
                    codes[i, j, k] = PRENORMAL
                    nrm[i, j, k] = (0, -1 if j == 0 else 1, 0)
    return codes, nrm


def mixed_grid(n1: int, n2: int, n3: int, seed: int, oblique: bool = True,
               face_prenormal: bool = True, interior_rows: int = 0):
    """A small grid that exercises every operator branch: Fictive holes,
    inactive Defined/Equation cells read by Actual neighbours, PreDefined
    (Dirichlet semi-sum) rows and PreNormal rows with axis and oblique outward
    normals on the faces.  `face_prenormal=False` keeps PreNormal rows off the
    box faces; `interior_rows` turns that many interior Actual cells into
    PreDefined/PreNormal rows (the variable-density operator is only defined
    for PreNormal rows away from the box faces)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    codes = np.zeros((n1, n2, n3), np.int32)
    nrm = np.zeros((n1, n2, n3, 3))
    codes[1:-1, 1:-1, 1:-1] = ACTUAL
    inner = np.argwhere(codes == ACTUAL)
    pick = rng.choice(len(inner), size=max(3, len(inner) // 12), replace=False)
    for q, p in enumerate(pick):
        codes[tuple(inner[p])] = (FICTIVE, DEFINED, EQUATION)[q % 3]
    dims = (n1, n2, n3)
    for i in range(n1):
        for j in range(n2):
            for k in range(n3):
                idx = (i, j, k)
                ext = [a for a in range(3) if idx[a] in (0, dims[a] - 1)]
                if len(ext) != 1:
                    continue
                a = ext[0]
                out = -1.0 if idx[a] == 0 else 1.0
                u = rng.random()
                if u < 0.25:
                    codes[idx] = FICTIVE
                elif u < 0.5:
                    codes[idx] = PREDEFINED
                    nrm[idx][a] = out
                elif u < 0.85 and face_prenormal:
                    codes[idx] = PRENORMAL
                    nrm[idx][a] = out
                    if oblique and rng.random() < 0.5:
                        for b in range(3):
                            if b != a:
                                nrm[idx][b] = rng.choice((-1.0, 1.0)) * rng.uniform(0.1, 0.6)
                elif u < 0.93:
                    codes[idx] = DEFINED
                else:
                    codes[idx] = EQUATION
    if interior_rows:
        inner = np.argwhere(codes[1:-1, 1:-1, 1:-1] == ACTUAL) + 1
        pick = rng.choice(len(inner), size=interior_rows, replace=False)
        for q, p in enumerate(pick):
            idx = tuple(inner[p])
            a = q % 3
            if q % 2 == 0:
                codes[idx] = PREDEFINED
                nrm[idx][a] = rng.choice((-1.0, 1.0))
            else:
                codes[idx] = PRENORMAL
                nrm[idx] = rng.uniform(-1, 1, 3)
                nrm[idx][a] = rng.choice((-1.0, 1.0))
    return codes, nrm


def random_nodes(n: int, rng, start: float = 0.0) -> np.ndarray:
    """n node coordinates with random positive spacings (TRandomSeparator input)."""
    h = rng.uniform(0.5, 1.5, size=n - 1) / (n - 1)
    return start + np.concatenate([[0.0], np.cumsum(h)])


def spheres_grid(n: int, nspheres: int, rmin: float, rmax: float, seed: int):
    """Unit cube, n cells per axis, cell-centred with one ghost layer
    (nodes -h/2 .. 1+h/2 as XProblem.cpp:392-394), Fictive ghost layer
    (homogeneous Neumann walls) and `nspheres` non-overlapping spheres with
    radii U[rmin, rmax] masked Fictive.  Active cells left with no open face
    are made Fictive so that every active row couples to the rest."""
    h = 1.0 / n
    nodes, sep = uniform_nodes(-h / 2, 1 + h / 2, h)
    nb = len(nodes)
    rng = np.random.Generator(np.random.PCG64(seed))
    centres, radii = [], []
    tries = 0
    while len(centres) < nspheres:
        tries += 1
        if tries > 100000:
            raise RuntimeError("sphere packing failed")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r, 1 - r, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 for c2, r2 in zip(centres, radii)):
            centres.append(c)
            radii.append(r)
    codes = np.zeros((nb, nb, nb), np.int32)
    codes[1:-1, 1:-1, 1:-1] = ACTUAL
    x = nodes
    for c, r in zip(centres, radii):
        lo = np.searchsorted(x, c - r - h)
        hi = np.searchsorted(x, c + r + h) + 1
        sl = tuple(slice(max(1, lo[a]), min(nb - 1, hi[a])) for a in range(3))
        X, Y, Z = np.meshgrid(x[sl[0]], x[sl[1]], x[sl[2]], indexing="ij")
        inside = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 < r * r
        sub = codes[sl]
        sub[inside] = FICTIVE
    _drop_isolated(codes)
    return codes, np.zeros((nb, nb, nb, 3)), nodes, sep, (np.array(centres), np.array(radii))


def coarse_grid(codes: np.ndarray, sep, F: int):
    """Point codes and separations of the coarse grid whose interior cells are
    the F x F x F blocks of a fine grid's interior (ghost layers match): a
    block with any active fine cell is Actual, else Fictive; the ghost layer is
    Fictive.  `sep` is the fine grid's uniform separations (one axis).  This is
    the grid of the learned two-level preconditioner's network."""
    n = np.array(codes.shape) - 2
    if np.any(n % F):
        raise ValueError(f"interior {tuple(n)} is not a whole number of {F}^3 blocks")
    act = space_mask(codes)[1:-1, 1:-1, 1:-1].astype(bool)
    m = act.reshape(n[0] // F, F, n[1] // F, F, n[2] // F, F).any(axis=(1, 3, 5))
    out = np.zeros(tuple(n // F + 2), np.int32)
    out[1:-1, 1:-1, 1:-1][m] = ACTUAL
    _drop_isolated(out)
    H = float(sep[0]) * F
    return out, np.full(out.shape[0] - 1, H), np.full(out.shape[1] - 1, H), np.full(out.shape[2] - 1, H)


def _drop_isolated(codes: np.ndarray) -> None:
    act = codes == ACTUAL
    nonfict = codes != FICTIVE
    opened = np.zeros_like(act)
    for a in range(3):
        for s in (-1, 1):
            opened[1:-1, 1:-1, 1:-1] |= np.roll(nonfict, -s, axis=a)[1:-1, 1:-1, 1:-1]
    codes[act & ~opened] = FICTIVE


def divergence_rhs(codes: np.ndarray, sep, seed: int) -> np.ndarray:
    """b = -(div u) of an i.i.d. N(0,1) staggered velocity field on Actual cells
    (the pressure right-hand side of XProblem.cpp:5474-5512 with rho = 1 and
    tau = 1), zero elsewhere, projected to zero mean over active cells."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n1, n2, n3 = codes.shape
    hx, hy, hz = sep
    b = np.zeros(codes.shape)
    u = rng.standard_normal((n1, n2, n3))
    v = rng.standard_normal((n1, n2, n3))
    w = rng.standard_normal((n1, n2, n3))
    div = np.zeros(codes.shape)
    div[1:, :, :] += (u[1:] - u[:-1]) / np.asarray(hx)[:, None, None]
    div[:, 1:, :] += (v[:, 1:] - v[:, :-1]) / np.asarray(hy)[None, :, None]
    div[:, :, 1:] += (w[:, :, 1:] - w[:, :, :-1]) / np.asarray(hz)[None, None, :]
    act = codes == ACTUAL
    b[act] = -div[act]
    sm = space_mask(codes).astype(bool)
    b[sm] -= b[sm].mean()
    return b


# ---------------------------------------------------------------------------
U_IN = 1.25   # inflow velocity of the staggered channel case


def _stag_seps(rng, n):
    return rng.uniform(0.8, 1.2, n - 1) / (n - 1)


def staggered_channel(n1=14, n2=11, n3=12, seed=3):
    """Staggered channel case for the time-step passes around the pressure
    solve (TVPProblem::SolveBySplitting, XProblem.cpp:5474-5829).

    Pressure box n1 x n2 x n3 with a Fictive ghost layer, Actual interior, a
    masked (Fictive) sphere, and PreDefined cells on the outlet face; u box
    (n1-1) x n2 x n3 with a Defined inflow face (border value U_IN) and a
    PreDefined outflow face whose values mirror the interior as the
    reference's check demands; v and w boxes with Fictive ghosts.  Separations
    are seeded and non-uniform so that every index of hxU/hyV/hzW and
    hxP/hyP/hzP is exercised."""
    rng = np.random.Generator(np.random.PCG64(seed))
    hP = [_stag_seps(rng, n) for n in (n1, n2, n3)]
    ii, jj, kk = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij")
    sphere = (ii - n1 / 2) ** 2 + (jj - n2 / 2) ** 2 + (kk - n3 / 2) ** 2 < (min(n1, n2, n3) / 5) ** 2

    pc = np.zeros((n1, n2, n3), np.int32)
    pc[1:-1, 1:-1, 1:-1] = 1
    pc[-1, 1:-1, 1:-1] = 4            # outlet: PreDefined pressure
    pc[sphere] = 0

    uc = np.zeros((n1 - 1, n2, n3), np.int32)
    uc[1:-1, 1:-1, 1:-1] = 1
    uc[0, 1:-1, 1:-1] = 3             # inflow: Defined
    uc[-1, 1:-1, 1:-1] = 4            # outflow: PreDefined (one Actual neighbour, i-1)
    uc[sphere[:-1]] = 0
    vc = np.zeros((n1, n2 - 1, n3), np.int32)
    vc[1:-1, 1:-1, 1:-1] = 1
    vc[sphere[:, :-1]] = 0
    wc = np.zeros((n1, n2, n3 - 1), np.int32)
    wc[1:-1, 1:-1, 1:-1] = 1
    wc[sphere[:, :, :-1]] = 0
    # a PreDefined u cell next to the sphere could see no Actual neighbour:
    # keep the outflow face clear of it
    uc[-1][uc[-2] != 1] = 0

    # separations of the staggered grids: u nodes sit between p nodes along x
    hU = [np.full(n1 - 2, 0.0), hP[1], hP[2]]
    hU[0] = 0.5 * (hP[0][:-1] + hP[0][1:])
    hV = [hP[0], 0.5 * (hP[1][:-1] + hP[1][1:]), hP[2]]
    hW = [hP[0], hP[1], 0.5 * (hP[2][:-1] + hP[2][1:])]

    u = rng.standard_normal(uc.shape)
    v = rng.standard_normal(vc.shape)
    w = rng.standard_normal(wc.shape)
    u_border = np.zeros(uc.shape)
    u_border[uc == 3] = U_IN
    u_border[uc == 4] = rng.uniform(0.5, 1.5, int((uc == 4).sum()))
    u[uc == 3] = U_IN
    # PreDefined previous values satisfy |prev - (2 b - prev[i-1])| <= 1e-10
    face = uc[-1] == 4
    u[-1][face] = 2 * u_border[-1][face] - u[-2][face]
    density = rng.uniform(0.5, 2.0, pc.shape)
    p_border = np.where(pc == 4, rng.standard_normal(pc.shape), 0.0)
    p = rng.standard_normal(pc.shape)
    return dict(pc=pc, uc=uc, vc=vc, wc=wc, hP=hP, hU=hU, hV=hV, hW=hW, u=u, v=v, w=w, u_border=u_border,
                density=density, p_border=p_border, p=p, tau=1e-3)


def icosphere(subdiv: int) -> np.ndarray:
    """Unit icosphere vertices: the icosahedron's 12 vertices, each triangle
    split in four `subdiv` times with midpoints pushed to the sphere
    (10 * 4**subdiv + 2 vertices: 2562 at subdivision 4, the immersed-body
    config's marker set)."""
    return icosphere_mesh(subdiv)[0]


def icosphere_mesh(subdiv: int):
    """The closed icosphere surface: (vertices (V, 3), faces (F, 3) int32,
    outward counter-clockwise), 20 * 4**subdiv faces."""
    t = (1.0 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int32)


def read_stl(path):
    """Triangles of an ASCII or binary STL file as (vertices (V, 3) float64,
    faces (F, 3) int32), vertices merged where their coordinates are equal
    (the reference reads its geometry through stl_reader.h the same way)."""
    data = open(path, "rb").read()
    tri = None
    if len(data) >= 84:
        nf = int(np.frombuffer(data[80:84], "<u4")[0])
        if 84 + 50 * nf == len(data):   # binary: 50-byte records after an 80-byte header
            rec = np.frombuffer(data[84:], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
            tri = rec["v"].astype(np.float64)
    if tri is None:
        pts = [list(map(float, line.split()[1:4])) for line in data.decode("ascii", "replace").splitlines()
               if line.strip().startswith("vertex")]
        tri = np.array(pts, dtype=np.float64).reshape(-1, 3, 3)
    verts, inv = np.unique(tri.reshape(-1, 3), axis=0, return_inverse=True)
    return verts, inv.reshape(-1, 3).astype(np.int32)


def reference_step_case(n1=11, n2=8, n3=9, seed=11):
    """A channel statement the reference's own time step (TVPProblem::
    SolveBySplitting, XProblem.cpp:4255-6650) runs as given: every velocity
    line through Actual points starts and ends on a border point (the ADI
    sector rule, XProblem.cpp:2940-2960), and every PreDefined velocity point
    has exactly one Actual neighbour (XProblem.cpp:5698-5735).

    Pressure box n1 x n2 x n3: Actual interior, Fictive ghost layer except a
    PreDefined outlet face (i = n1 - 1, outward normal +x, seeded border
    pressures).  u box (n1-1) x n2 x n3: Defined inflow face (u = 1), seeded
    PreDefined outflow face, PreDefined no-slip walls (0) on the j and k
    faces; v and w boxes likewise with Defined zero normal velocity on their
    own walls and PreDefined zero tangential values elsewhere.  Box edges are
    Fictive.  Coordinates are seeded and non-uniform; the staggered boxes sit
    at the midpoints of the pressure nodes and the node box (the VTK grid) at
    (x_u, y_v, z_w).  Also seeded: per-cell forces for the three momentum
    equations, and an initial concentration blob (0.45 where set,
    XProblem.cpp:4636-4650) that gives non-uniform density and viscosity."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xp = [np.concatenate([[0.0], np.cumsum(rng.uniform(0.8, 1.2, n - 1) / (n - 1))]) for n in (n1, n2, n3)]
    mid = [0.5 * (a[:-1] + a[1:]) for a in xp]

    def faces(shape, normal_axis, normal_code, normal_val, tangential_val_hi):
        """codes/border values of a staggered box: Actual interior, the two
        faces across `normal_axis` Defined (normal_code), the others
        PreDefined; edges and corners Fictive."""
        c = np.zeros(shape, np.int32)
        bc = np.zeros(shape)
        c[1:-1, 1:-1, 1:-1] = 1
        for ax in range(3):
            for side in (0, -1):
                sl = [slice(1, -1)] * 3
                sl[ax] = side
                sl = tuple(sl)
                c[sl] = normal_code if ax == normal_axis else 4
        return c, bc

    uc, ubc = faces((n1 - 1, n2, n3), 0, 3, 1.0, None)
    # x faces of the u box: inflow Defined u = 1, outflow PreDefined (seeded)
    uc[0, 1:-1, 1:-1] = 3
    ubc[0, 1:-1, 1:-1] = 1.0
    uc[-1, 1:-1, 1:-1] = 4
    ubc[-1, 1:-1, 1:-1] = rng.uniform(0.8, 1.2, (n2 - 2, n3 - 2))
    vc, vbc = faces((n1, n2 - 1, n3), 1, 3, 0.0, None)
    vbc[-1, 1:-1, 1:-1] = rng.uniform(-0.1, 0.1, (n2 - 3, n3 - 2))
    wc, wbc = faces((n1, n2, n3 - 1), 2, 3, 0.0, None)
    wbc[-1, 1:-1, 1:-1] = rng.uniform(-0.1, 0.1, (n2 - 2, n3 - 3))

    pc = np.zeros((n1, n2, n3), np.int32)
    pc[1:-1, 1:-1, 1:-1] = 1
    pc[-1, 1:-1, 1:-1] = 4
    pnrm = np.zeros((n1, n2, n3, 3))
    pnrm[-1, 1:-1, 1:-1, 0] = 1.0
    pbc = np.zeros((n1, n2, n3))
    pbc[-1, 1:-1, 1:-1] = rng.uniform(-0.5, 0.5, (n2 - 2, n3 - 2))

    nc = np.zeros((n1 - 1, n2 - 1, n3 - 1), np.int32)
    nc[1:-1, 1:-1, 1:-1] = 1

    ii, jj, kk = np.meshgrid(*(np.arange(n) for n in (n1, n2, n3)), indexing="ij")
    conc0 = (((ii - n1 / 3) ** 2 + (jj - n2 / 2) ** 2 + (kk - n3 / 2) ** 2) < (min(n1, n2, n3) / 3.5) ** 2)
    conc0 = (conc0 & (pc == 1)).astype(np.int32)
    force = [rng.standard_normal(c.shape) * 0.3 for c in (uc, vc, wc)]
    return dict(p=(pc, (xp[0], xp[1], xp[2]), pnrm, pbc), u=(uc, (mid[0], xp[1], xp[2]), None, ubc),
                v=(vc, (xp[0], mid[1], xp[2]), None, vbc), w=(wc, (xp[0], xp[1], mid[2]), None, wbc),
                n=(nc, (mid[0], mid[1], mid[2]), None, None), conc0=conc0, force=force,
                params=np.array([1.0 / 512, 0.02, 0.05, 1.0, 1.6]))

