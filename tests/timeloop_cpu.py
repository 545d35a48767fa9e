"""The time step of xflow_gb300.timeloop restated on the CPU from the
oracle's passes (each pinned bit for bit to the reference's own time step,
tests/test_oracle_step_ref.py) and numpy Krylov solves: the checker of the
GPU time loop.  Test infrastructure only."""
import numpy as np

from oracle import oracle as O

ACTIVE = (1, 4, 5, 6, 8)


def bicgstab(apply, x, b, act, tol):
    """BiCGStab on the active cells (inactive entries of x stay as given):
    stops when max |b - A x| <= tol."""
    r = np.where(act, b - apply(x), 0.0)
    rh, p, v = r.copy(), np.zeros_like(r), np.zeros_like(r)
    rho = alpha = omega = 1.0
    for it in range(20000):
        if np.abs(r).max() <= tol:
            return x, it
        rho_n = np.dot(rh[act], r[act])
        beta = (rho_n / rho) * (alpha / omega)
        p = r + beta * (p - omega * v)
        z = x.copy()
        z[act] = 0.0
        base = apply(z)   # the fixed (inactive) part's contribution
        Ap = lambda d: np.where(act, apply(np.where(act, d, 0.0) + z) - base, 0.0)  # noqa: E731
        v = Ap(p)
        alpha = rho_n / np.dot(rh[act], v[act])
        s = r - alpha * v
        t = Ap(s)
        omega = np.dot(t[act], s[act]) / np.dot(t[act], t[act])
        x = np.where(act, x + alpha * p + omega * s, x)
        r = np.where(act, b - apply(x), 0.0)
        rho = rho_n
    raise RuntimeError("CPU BiCGStab did not converge")


def face(shape, axis, side):
    """Index of the face plane (axis 1..3, side 0 low / 1 high) of a box."""
    sl = [slice(None)] * 3
    sl[axis - 1] = 0 if side == 0 else shape[axis - 1] - 1
    return tuple(sl)


def inward(shape, axis, side):
    """Index of the layer next to that face, inside."""
    sl = [slice(None)] * 3
    sl[axis - 1] = 1 if side == 0 else shape[axis - 1] - 2
    return tuple(sl)


def border_follow(codes, vel, bc, axis, side):
    """PreDefined points of the face take their Actual neighbour's value as border value (xf_border_follow)."""
    f, n = face(codes.shape, axis, side), inward(codes.shape, axis, side)
    m = (codes[f] == 4) & (codes[n] == 1)
    bc[f] = np.where(m, vel[n], bc[f])


def outflow_convective(codes, vel, bc, h, axis, speed, tau):
    """xf_outflow_convective: the Defined outlet values (high face of `axis`) take an upwind step of
    db/dt + speed db/dn = 0, then shift so that their area-weighted sum equals the inlet face's.  The sums
    are formed in float64 by numpy (another order than the device's tree): agreement to rounding."""
    f0, f1, n1 = face(codes.shape, axis, 0), face(codes.shape, axis, 1), inward(codes.shape, axis, 1)
    oth = [d for d in range(3) if d != axis - 1]
    wid = []
    for d in oth:
        hd, n = h[d], codes.shape[d]
        w = np.zeros(n)
        w[1:n - 1] = (hd[:-1] + hd[1:])[: n - 2] / 2
        wid.append(w)
    area = wid[0][:, None] * wid[1][None, :]
    c = speed * tau / h[axis - 1][codes.shape[axis - 1] - 2]
    m_in, m_out = codes[f0] == 3, codes[f1] == 3
    b = bc[f1].copy()
    b = np.where(m_out, b - c * (b - vel[n1]), b)
    s_in = (area * bc[f0])[m_in].sum()
    s_out, a_out = (area * b)[m_out].sum(), area[m_out].sum()
    b = np.where(m_out, b + (s_in - s_out) / a_out, b)
    bc[f1] = b


def scalar_step(sc, hp, vel, c, tau, tol=1e-13):
    """The concentration equation (XProblem.cpp:5850-5977) from the corrected velocities, with the upwind
    transfer operator unsplit and solved by BiCGStab, as on the GPU."""
    codes = sc["codes"]
    (uT, vT, wT, rp), s, _ = O.conc_transfer(codes, vel[0], vel[1], vel[2], inlet=sc["inlet"])
    assert s == 0
    act = np.isin(codes, ACTIVE)
    rhs = np.where(codes == 1, (1 / tau) * c + rp, np.where(act, rp, c))
    og = O.Grid(codes, sc["nrm"], *hp)
    apply = lambda x: O.apply_advdiff(og, x, uT, vT, wT, tau, sc["D"], 7)  # noqa: E731
    x, _ = bicgstab(apply, c.copy(), rhs, act, tol * np.abs(rhs[act]).max())
    return x


def step(st, vel, p, tol_mom=1e-12, rtol_p=1e-12, scalar=None):
    """One time step of the statement `st` (timeloop.cavity / channel /
    with_scalar, no markers) from the velocity boxes `vel`, pressure `p` (and
    the scalar box `scalar`); returns the new velocity boxes, the pressure and the control
    balance (and the scalar).  The border values of `st` are updated in
    place, as the GPU loop updates its border boxes."""
    tau = st["tau"]
    pc, pn, pbc, hp = st["p"]
    for axis, side in st.get("follow", ()):
        for a, (codes, _, bc) in enumerate(st["comps"]):
            border_follow(codes, vel[a], bc, axis, side)
    if "convective" in st:
        axis, speed = st["convective"]
        codes, _, bc = st["comps"][axis - 1]
        hh = [hp[d] for d in range(3)]
        hh[axis - 1] = 0.5 * (hp[axis - 1][:-1] + hp[axis - 1][1:])
        outflow_convective(codes, vel[axis - 1], bc, hh, axis, speed, tau)
    hs = []
    mid = []
    for a, (codes, nrm, bc) in enumerate(st["comps"]):
        hh = [hp[d] for d in range(3)]
        hh[a] = 0.5 * (hp[a][:-1] + hp[a][1:])
        hs.append(hh)
        vis = np.full(pc.shape, st["vis"])
        (uT, vT, wT, visT, rp), s, _ = O.momentum_rhs(a + 1, codes, vel[0], vel[1], vel[2], *hh, vis=vis, border=bc,
                                                     normals=nrm)
        assert s == 0
        act = np.isin(codes, ACTIVE)
        rhs = np.where(codes == 1, (1 / tau) * vel[a] + rp, np.where(act, rp, vel[a]))
        og = O.Grid(codes, nrm, *hh)
        apply = lambda x: O.apply_advdiff(og, x, uT, vT, wT, tau, 0.0, 3, Dfield=visT)  # noqa: E731
        x, _ = bicgstab(apply, vel[a].copy(), rhs, act, tol_mom * np.abs(rhs[act]).max())
        for c in zip(*np.nonzero(codes == 3)):   # Defined sector ends take their border value
            nb = [tuple(np.add(c, d)) for d in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
            if any(all(0 <= q[t] < codes.shape[t] for t in range(3)) and codes[q] == 1 for q in nb):
                x[c] = bc[c]
        for c in zip(*np.nonzero(codes == 4)):   # the PreDefined border values exact
            nb = [tuple(np.add(c, d)) for d in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
            nb = [q for q in nb if all(0 <= q[t] < codes.shape[t] for t in range(3)) and codes[q] == 1]
            x[c] = 2 * bc[c] - x[nb[0]]
        mid.append(x)
    rhs, s, _ = O.pressure_rhs(pc, mid[0], mid[1], mid[2], hs[0][0], hs[1][1], hs[2][2], tau, border=pbc)
    assert s == 0
    og = O.Grid(pc, pn if pn is not None else np.zeros(pc.shape + (3,)), *hp)
    p, _ = O.cg_plain(O.LAPLACE, og, p, rhs, rtol_p)
    out = []
    for a, (codes, nrm, bc) in enumerate(st["comps"]):
        v, s, _ = O.velocity_correct(a + 1, codes, mid[a], p, hp[a], tau, border=bc, cur=vel[a])
        assert s == 0
        out.append(v)
    div = O.divergence_max(pc, out[0], out[1], out[2], hs[0][0], hs[1][1], hs[2][2])
    if scalar is not None:
        return out, p, div, scalar_step(st["scalar"], hp, out, scalar, tau)
    return out, p, div
