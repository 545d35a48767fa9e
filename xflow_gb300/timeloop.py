"""The time step of TVPProblem::SolveBySplitting (XProblem.cpp:4255-6650) on
the GPU, every pass through the C ABI of include/xflow.h:

  momentum, per velocity component eq (XProblem.cpp:5017-5446):
    xf_momentum_rhs      transfer velocities, face viscosity, border values,
                         forces, viscous terms (the reference's loops)
    xf_transfer_rhs      (1/tau) f_1 + rp
    XF_OP_ADVDIFF solve  the implicit transfer equation, unsplit (the sum of
                         the reference's three ADI line operators), BiCGStab
    xf_border_recalc     the PreDefined border values exact, as the ADI
                         sweeps leave them
  pressure (XProblem.cpp:5452-5594):
    xf_pressure_rhs, then the pressure solve (mixed-precision CG on
    all-Neumann systems, BiCGStab where border rows make it nonsymmetric)
  xf_velocity_correct per component (XProblem.cpp:5598-5777)
  xf_divergence_max, the control balance (XProblem.cpp:5782-5829)
  concentration, with a scalar (XProblem.cpp:5850-5977):
    xf_conc_transfer     transfer velocities from the corrected velocities,
                         the inlet values on the PreDefined inlet points
    XF_OP_ADVDIFF solve  the upwind transfer operator (SolveTransferEquation_'s
                         scheme), unsplit, BiCGStab

With markers, each momentum equation's force is the immersed boundary's
(TImmersedBoundaryProblem::GetForce order, XProblem.cpp:8350-8353):
interpolate the component's velocity at the markers, move them, compute
their forces, spread them into the force box.

Statements are boxes: a pressure grid of n1 x n2 x n3 cell centres with a
ghost layer, staggered velocity grids one smaller along their own axis
(XStatement.h:127-135), Actual interiors; on every face of a velocity box
the component normal to the face is Defined (its value kept) and the
tangential ones PreDefined (the semi-sum across the face equals the border
value, XOperator.cpp:1034-1069), box edges Fictive.  A scalar is passive
(single fluid, rho = 1: the reference's density and viscosity updates from
the concentration keep their values when rho1 = rho2 and mu1 = mu2).

The pressure solve is plain FP64 CG, mixed-precision CG, or the learned
two-level preconditioner under mixed-precision FCG (a U-Net on the coarse
grid of 4^3 blocks), each warm-started from the previous step's pressure,
on all-Neumann statements; BiCGStab where outlet rows make the system
nonsymmetric.
"""
import time

import numpy as np

from . import capi

FICTIVE, ACTUAL, DEFINED, PREDEFINED, PRENORMAL = 0, 1, 3, 4, 6


def _face_slices(shape, ax, side):
    sl = [slice(1, n - 1) for n in shape]
    sl[ax] = 0 if side == 0 else shape[ax] - 1
    return tuple(sl)


def velocity_box(pshape, axis, faces):
    """Codes, outward normals and border values of velocity component `axis`
    (0 u, 1 v, 2 w) for a pressure box of shape pshape.  faces[(ax, side)]
    gives this component's value on that face (side 0 low, 1 high); the
    faces listed in faces['outflow'] make the normal component PreDefined
    there too (its value then plays the outflow's border value)."""
    shape = list(pshape)
    shape[axis] -= 1
    shape = tuple(shape)
    codes = np.zeros(shape, np.int32)
    nrm = np.zeros(shape + (3,))
    bc = np.zeros(shape)
    codes[1:-1, 1:-1, 1:-1] = ACTUAL
    outflow = faces.get("outflow", ())
    for ax in range(3):
        for side in (0, 1):
            sl = _face_slices(shape, ax, side)
            pre = ax != axis or (ax, side) in outflow
            codes[sl] = PREDEFINED if pre else DEFINED
            if pre:
                nrm[sl + (ax,)] = -1.0 if side == 0 else 1.0
            bc[sl] = faces.get((ax, side), 0.0)
    return codes, nrm, bc


def scalar_box(pshape, inlet=None):
    """Codes and outward normals of the concentration grid of a pressure box
    (the reference's gridC, XProblem.cpp:4555-4600): Actual interior,
    PreNormal faces (zero normal gradient), PreDefined points on the face
    i = 0 where `inlet` (an n2 x n3 boolean array) is set, box edges Fictive
    (no line or stencil of an Actual point reaches them)."""
    codes = np.zeros(pshape, np.int32)
    nrm = np.zeros(tuple(pshape) + (3,))
    codes[1:-1, 1:-1, 1:-1] = ACTUAL
    for ax in range(3):
        for side in (0, 1):
            sl = _face_slices(pshape, ax, side)
            codes[sl] = PRENORMAL
            nrm[sl + (ax,)] = -1.0 if side == 0 else 1.0
    if inlet is not None:
        face = codes[0]
        face[np.asarray(inlet, bool) & (face == PRENORMAL)] = PREDEFINED
    return codes, nrm


def gaussian_inlet(pshape, h, sigma=0.05, centre=(0.5, 0.5)):
    """A Gaussian blob exp(-r^2 / (2 sigma^2)) of the distance r from `centre`
    in the inlet plane, at the cell centres ((j - 1/2) h_y, (k - 1/2) h_z) of
    the face i = 0: the inlet values (an n2 x n3 array) of a scalar."""
    n2, n3 = pshape[1], pshape[2]
    y = (np.arange(n2) - 0.5) * h[1][0]
    z = (np.arange(n3) - 0.5) * h[2][0]
    r2 = (y[:, None] - centre[0]) ** 2 + (z[None, :] - centre[1]) ** 2
    return np.exp(-r2 / (2 * sigma * sigma))


def with_scalar(st, inlet_values, schmidt=1.0, c0=0.0):
    """A passive scalar added to a statement: PreDefined inlet points on the
    whole face i = 0 with `inlet_values` (n2 x n3) as their border values,
    diffusion coefficient viscosity / Schmidt, initial value c0 inside."""
    pc = st["p"][0]
    codes, nrm = scalar_box(pc.shape, np.ones(pc.shape[1:], bool))
    inlet = np.zeros(pc.shape)
    inlet[0] = np.where(codes[0] == PREDEFINED, inlet_values, 0.0)
    c = np.where(codes == ACTUAL, c0, 0.0)
    st = dict(st)
    st["scalar"] = dict(codes=codes, nrm=nrm, inlet=inlet, c0=c, D=st["vis"] / schmidt, schmidt=schmidt)
    st["name"] += f", scalar Sc={schmidt:g}"
    return st


def cavity(n, lid=1.0, re=100.0, tau=1e-3, noise=1e-3, seed=1):
    """The lid-driven cavity: unit cube of n^3 cells (h = 1/n), lid velocity u
    = `lid` on the top face z = 1, no-slip elsewhere, all-Neumann pressure,
    viscosity 1/Re, initial velocity zero plus seeded i.i.d. N(0, noise) on
    the Actual points."""
    B = n + 2
    pshape = (B, B, B)
    h = [np.full(B - 1, 1.0 / n)] * 3
    pc = np.zeros(pshape, np.int32)
    pc[1:-1, 1:-1, 1:-1] = ACTUAL
    comps = [velocity_box(pshape, 0, {(2, 1): lid}), velocity_box(pshape, 1, {}), velocity_box(pshape, 2, {})]
    rng = np.random.Generator(np.random.PCG64(seed))
    vel0 = []
    for codes, _, bc in comps:
        v = np.where(codes == DEFINED, bc, 0.0)
        v[codes == ACTUAL] = rng.normal(0.0, noise, int((codes == ACTUAL).sum()))
        vel0.append(v)
    return dict(name=f"lid-driven cavity {n}^3, Re={re:g}, dt={tau:g}", p=(pc, None, None, h), comps=comps,
                h=h, vel0=vel0, vis=1.0 / re, tau=tau, pressure="neumann")


def channel(nx, ny, nz, length=4.0, u_in=1.0, re=200.0, tau=2e-3, outflow="zero_gradient", walls="no_slip"):
    """The channel [0, length] x [0, 1] x [0, 1] of nx x ny x nz cells:
    Defined inflow u = u_in at x = 0, an outflow at x = length, side walls
    with zero normal velocity, viscosity 1/Re; the velocity starts at the
    inflow value.
      outflow="zero_gradient": PreDefined pressure 0 on the outlet and
        PreDefined velocities whose border values follow the last interior
        layer, lagged by a step (the pressure system has outlet rows);
      outflow="convective": the outlet's normal velocity Defined and advanced
        each step by a convective outflow at speed u_in, its flux balanced
        against the inflow (xf_outflow_convective); the tangential ones follow
        the interior; the pressure is all-Neumann.
      walls="no_slip": zero tangential border values; "free_slip": the
        tangential components' border values follow the interior (a lagged
        zero normal gradient).  With free-slip walls the flow accelerates
        without bound: the momentum right-hand side's viscous term
        dVis . (dVel + dU) (XProblem.cpp:5352-5419) sees the face viscosity
        drop to 0 on the border points, a forcing of the wall layer that no
        wall friction balances (a property of the reference's
        discretisation, reproduced by the CPU restatement)."""
    if outflow not in ("zero_gradient", "convective") or walls not in ("no_slip", "free_slip"):
        raise ValueError("outflow: zero_gradient | convective; walls: no_slip | free_slip")
    pshape = (nx + 2, ny + 2, nz + 2)
    h = [np.full(nx + 1, length / nx), np.full(ny + 1, 1.0 / ny), np.full(nz + 1, 1.0 / nz)]
    pc = np.zeros(pshape, np.int32)
    pc[1:-1, 1:-1, 1:-1] = ACTUAL
    pn = np.zeros(pshape + (3,))
    pbc = np.zeros(pshape)
    follow = [(1, 1)]
    if outflow == "zero_gradient":
        pc[-1, 1:-1, 1:-1] = PREDEFINED
        pn[-1, 1:-1, 1:-1, 0] = 1.0
        out = {"outflow": ((0, 1),)}
    else:
        out = {}
    if walls == "free_slip":
        follow += [(2, 0), (2, 1), (3, 0), (3, 1)]
    ufaces = dict(out)
    ufaces.update({(0, 0): u_in, (0, 1): u_in})
    comps = [velocity_box(pshape, 0, ufaces), velocity_box(pshape, 1, dict(out)), velocity_box(pshape, 2, dict(out))]
    vel0 = []
    for a, (codes, _, bc) in enumerate(comps):
        v = np.where(codes == DEFINED, bc, 0.0)
        if a == 0:
            v[codes == ACTUAL] = u_in
        vel0.append(v)
    name = f"channel {nx}x{ny}x{nz} on [0,{length:g}]x[0,1]x[0,1], Re={re:g}, dt={tau:g}"
    if outflow == "convective" or walls == "free_slip":
        name += f", {outflow.replace('_', '-')} outflow, {walls.replace('_', '-')} walls"
    st = dict(name=name, p=(pc, pn, pbc, h), comps=comps, h=h, vel0=vel0, vis=1.0 / re, tau=tau,
              pressure="outlet" if outflow == "zero_gradient" else "neumann", follow=tuple(follow))
    if outflow == "convective":
        st["convective"] = (1, u_in)
    return st


def sphere_markers(center, radius, subdiv=4, stiffness=1e3):
    """Target markers on an icosphere (subdivision 4: 2562 vertices), each
    pulled back to its own starting point (TTargetNode, XImmersedBoundary.cpp:
    720-759); the marker area is the sphere's over the markers."""
    from . import workloads as wl

    verts = wl.icosphere(subdiv) * radius + np.asarray(center, float)
    nn = len(verts)
    idx = np.arange(nn)
    return dict(pos=verts, ref=verts.copy(), kind=np.full(nn, capi.XF_IB_TARGET, np.int32),
                nxt=np.roll(idx, -1).astype(np.int32), prv=np.roll(idx, 1).astype(np.int32), dist0=np.zeros(nn),
                curv0=np.zeros((nn, 3)), stiff=np.ones(nn),
                params=np.array([stiffness, 0.0, 0.0, 4 * np.pi * radius * radius / nn]))


class SplittingLoop:
    """The time loop of a statement (cavity(), channel(), with_scalar()) on
    one device: `step()` advances one time step and returns its per-step
    figures.  pressure_solver (all-Neumann statements): "mixed" (mixed-
    precision CG), "fp64" (plain FP64 CG) or "learned" (the two-level
    preconditioner under mixed-precision FCG; net_params the U-Net's, on the
    coarse grid of 4^3 blocks of a uniform grid)."""

    def __init__(self, ctx, st, markers=None, momentum_rtol=1e-10, pressure_rtol=1e-8, pressure_solver="mixed",
                 net_params=None, scalar_rtol=1e-10, two_level=(1, 4, 6), jacobi=True):
        import xflow_gb300 as xf
        from . import workloads as wl

        self.xf, self.ctx, self.st = xf, ctx, st
        self.tau = st["tau"]
        pc, pn, pbc, hp = st["p"]
        self.gp = xf.Grid(ctx, pc, *hp, pn)
        self.pbc = self.gp.vec(pbc) if pbc is not None else None
        self.g, self.bc, self.vel, self.mid, self.ops, self.rhs = [], [], [], [], [], []
        for a, (codes, nrm, bc) in enumerate(st["comps"]):
            hh = [hp[d][:-1] if d == a else hp[d] for d in range(3)]
            hh[a] = 0.5 * (hp[a][:-1] + hp[a][1:])   # staggered nodes sit between the pressure nodes
            g = xf.Grid(ctx, codes, *hh, nrm)
            self.g.append(g)
            self.bc.append(g.vec(bc))
            self.vel.append(g.vec(st["vel0"][a]))
            self.mid.append(g.vec(st["vel0"][a]))
            self.ops.append(xf.Operator(g, xf.XF_OP_ADVDIFF))
            self.rhs.append(g.vec(None))
        self.mom = [tuple(g.vec(None) for _ in range(5)) for g in self.g]
        self.force = [g.vec(np.zeros(g.shape)) for g in self.g]
        self.vis = self.gp.vec(np.full(self.gp.shape, st["vis"]))
        self.pop = xf.Operator(self.gp, xf.XF_OP_LAPLACE)
        self.p = self.gp.vec(np.zeros(self.gp.shape))
        self.prhs = self.gp.vec(None)
        if pressure_solver not in ("mixed", "fp64", "learned"):
            raise ValueError("pressure_solver: mixed | fp64 | learned")
        self.pressure_solver, self.net, self.two_level = pressure_solver, None, two_level
        if pressure_solver == "learned" and st["pressure"] == "neumann":
            if net_params is None:
                raise ValueError("the learned pressure solve needs the network's parameters")
            cc, c1, c2, c3 = wl.coarse_grid(pc, hp[0], 4)
            self.net = xf.UNet(xf.Grid(ctx, cc, c1, c2, c3, None), params=net_params)
        self.scalar = None
        if "scalar" in st:
            sc = st["scalar"]
            self.gc = xf.Grid(ctx, sc["codes"], *hp, sc["nrm"])
            self.cin = self.gc.vec(sc["inlet"])
            self.c = self.gc.vec(sc["c0"])
            self.cnext = self.gc.vec(sc["c0"])
            self.ctr = tuple(self.gc.vec(None) for _ in range(4))
            self.cop = xf.Operator(self.gc, xf.XF_OP_ADVDIFF)
            self.crhs = self.gc.vec(None)
            self.scalar = sc
        self.scalar_rtol = scalar_rtol
        # the transport solves (momentum, scalar): BiCGStab, Jacobi-preconditioned by default
        self.transport_precond = capi.XF_PRECOND_JACOBI if jacobi else capi.XF_PRECOND_NONE
        self.markers = None
        if markers is not None:
            m = markers
            self.markers = xf.Markers(ctx, m["pos"], m["ref"], m["kind"], m["nxt"], m["prv"], m["dist0"], m["curv0"],
                                      m["stiff"], m["params"])
            self.h0 = np.array([hp[0][0], hp[1][0], hp[2][0]])
        self.momentum_rtol, self.pressure_rtol = momentum_rtol, pressure_rtol
        self.steps = 0

    def step(self):
        xf, tau = self.xf, self.tau
        self.ctx.synchronize()
        t0 = time.perf_counter()
        phase = {"borders": 0.0, "ib": 0.0, "momentum": 0.0, "pressure": 0.0, "correction": 0.0, "scalar": 0.0}
        mark = [t0]

        def lap(name):   # wall ms of each phase (synchronised; the step's own total is the record's ms)
            self.ctx.synchronize()
            t = time.perf_counter()
            phase[name] += (t - mark[0]) * 1e3
            mark[0] = t

        its = []
        u1, v1, w1 = self.vel
        for axis, side in self.st.get("follow", ()):   # zero-gradient faces take the interior's values
            for a in range(3):
                xf.border_follow(self.vel[a], self.bc[a], axis, side)
        if "convective" in self.st:   # the outlet's normal velocity: convective outflow, flux balanced
            axis, speed = self.st["convective"]
            xf.outflow_convective(self.vel[axis - 1], self.bc[axis - 1], axis, speed, tau)
        lap("borders")
        for a in range(3):
            force = None
            if self.markers is not None:   # GetForce: interpolate, move, forces, spread
                self.force[a].fill(0.0)
                self.markers.interpolate(self.vel[a], self.h0, a + 1)
                self.markers.update_position(a + 1, tau)
                self.markers.compute_forces(a + 1)
                self.markers.spread(self.force[a], self.h0, a + 1)
                force = self.force[a]
                lap("ib")
            uTr, vTr, wTr, visTr, rp = xf.momentum_rhs(a + 1, self.g[a], u1, v1, w1, vis=self.vis, border=self.bc[a],
                                                       force=force, out=self.mom[a])
            A = self.ops[a]
            A.set_advection(uTr, vTr, wTr, tau, 0.0, capi.XF_ADV_CONVECTIVE | capi.XF_ADV_DIFFUSIVE)
            A.set_diffusion_field(visTr)
            xf.transfer_rhs(self.vel[a], rp, tau, self.rhs[a])
            self.mid[a].assign(self.vel[a])   # warm start from f_1 (its Defined points hold their values)
            # BiCGStab's own stop rule, max |r| <= atol (XSLAE.cpp:712-716), relative to the right-hand side
            s = xf.solve(A, self.mid[a], self.rhs[a], method=xf.XF_BICGSTAB, precond=self.transport_precond,
                         atol=self.momentum_rtol * self.rhs[a].absmax()[0], maxit=20000)
            if s.status != capi.XF_OK:
                raise xf.XFError(s.status, f"momentum equation {a + 1}: status {s.status}")
            xf.border_recalc(self.mid[a], self.bc[a])   # the sector ends exact, as the ADI leaves them
            its.append(s.iterations)
            lap("momentum")
        xf.pressure_rhs(self.gp, *self.mid, tau, self.prhs, border=self.pbc)
        # every pressure solve starts from the previous step's pressure
        if self.st["pressure"] == "neumann" and self.pressure_solver == "learned":
            window, degree, ratio = self.two_level
            s = xf.solve_fcg(self.pop, self.p, self.prhs, unet=self.net, precond=capi.XF_PRECOND_UNET2,
                             rtol=self.pressure_rtol, window=window, degree=degree, ratio=ratio,
                             precision=xf.XF_PREC_MIXED, maxit=100000)
        elif self.st["pressure"] == "neumann":
            prec = xf.XF_PREC_MIXED if self.pressure_solver == "mixed" else xf.XF_PREC_FP64
            s = xf.solve(self.pop, self.p, self.prhs, method=xf.XF_CG, precision=prec, rtol=self.pressure_rtol,
                         maxit=100000)
        else:   # outlet rows: BiCGStab (Jacobi took 813 iterations a step where plain BiCGStab takes 655, channel
            # 256x64x64: one face of semi-sum rows beside uniform Actual rows gains nothing from the scaling)
            s = xf.solve(self.pop, self.p, self.prhs, method=xf.XF_BICGSTAB,
                         atol=self.pressure_rtol * self.prhs.absmax()[0], maxit=100000)
        if s.status != capi.XF_OK:
            raise xf.XFError(s.status, f"pressure: status {s.status}")
        its.append(s.iterations)
        lap("pressure")
        for a in range(3):
            xf.velocity_correct(a + 1, self.mid[a], self.p, tau, self.vel[a], border=self.bc[a])
        div, ijk = xf.divergence_max(self.gp, *self.vel)
        lap("correction")
        rec = {"pressure_iterations": its[3], "pressure_fallbacks": int(getattr(s, "fallbacks", 0))}
        if self.scalar is not None:   # the concentration equation, from the corrected velocities
            uT, vT, wT, rp = xf.conc_transfer(self.gc, *self.vel, inlet=self.cin, out=self.ctr)
            self.cop.set_advection(uT, vT, wT, tau, self.scalar["D"],
                                   capi.XF_ADV_CONVECTIVE | capi.XF_ADV_DIFFUSIVE | capi.XF_ADV_UPWIND)
            xf.transfer_rhs(self.c, rp, tau, self.crhs)
            self.cnext.assign(self.c)
            # BiCGStab, max |r| <= atol relative to the right-hand side, as the momentum equations.  Minimal
            # residuals (x += alpha r) stalls here: the border rows (semi-sums of scale 1/2, normal differences
            # of scale 1/h) sit beside Actual rows of scale 1/tau, and at 128x32x32 it had gained one decade
            # in 400 iterations where BiCGStab reaches 1e-10 in about 110, and Jacobi BiCGStab in 6.
            s = xf.solve(self.cop, self.cnext, self.crhs, method=xf.XF_BICGSTAB, precond=self.transport_precond,
                         atol=self.scalar_rtol * self.crhs.absmax()[0], maxit=20000)
            if s.status != capi.XF_OK:
                raise xf.XFError(s.status, f"concentration: status {s.status}")
            self.c, self.cnext = self.cnext, self.c
            rec["scalar_iterations"] = s.iterations
            lap("scalar")
        self.ctx.synchronize()
        self.steps += 1
        rec.update({"step": self.steps, "ms": (time.perf_counter() - t0) * 1e3, "momentum_iterations": its[:3],
                    "divergence_max": div, "divergence_cell": ijk, "phase_ms": phase,
                    "velocity_max": [v.absmax()[0] for v in self.vel]})
        return rec

    def fields(self):
        """Velocities and pressure (and the scalar, with one) as host arrays."""
        out = [v.download() for v in self.vel] + [self.p.download()]
        if self.scalar is not None:
            out.append(self.c.download())
        return out
