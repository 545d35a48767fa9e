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


def step(st, vel, p, tol_mom=1e-12, rtol_p=1e-12):
    """One time step of the statement `st` (timeloop.cavity / channel, no
    markers) from the velocity boxes `vel` and pressure `p`; returns the new
    velocity boxes, the pressure and the control balance."""
    tau = st["tau"]
    pc, pn, pbc, hp = st["p"]
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
    return out, p, div
