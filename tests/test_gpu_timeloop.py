"""The GPU time loop (xflow_gb300.timeloop: TVPProblem::SolveBySplitting's
momentum, pressure, correction and control-balance passes through the C ABI)
against its CPU restatement from the oracle's pinned passes and numpy
solves (tests/timeloop_cpu.py), three steps of the lid-driven cavity.  Bar:
velocities within 1e-7 of their range, pressure (zero-mean: the Neumann
system fixes it up to a constant) within 1e-6; both control balances at
rounding level (below 1e-9 of the velocity scale over the cell size)."""
import numpy as np
import pytest

import timeloop_cpu
import xflow_gb300 as xf
from xflow_gb300 import timeloop as tl

pytestmark = pytest.mark.gpu


def test_cavity_three_steps_match_the_cpu_restatement():
    ctx = xf.Context(0)
    try:
        st = tl.cavity(20, tau=2e-3)
        loop = tl.SplittingLoop(ctx, st, momentum_rtol=1e-13, pressure_rtol=1e-11)
        vel = [v.copy() for v in st["vel0"]]
        p = np.zeros(st["p"][0].shape)
        act_p = st["p"][0] == 1
        for k in range(3):
            rec = loop.step()
            vel, p, (div, ijk) = timeloop_cpu.step(st, vel, p)
            got = loop.fields()
            for a in range(3):
                codes = st["comps"][a][0]
                m = codes != 0
                scale = np.abs(vel[a][m]).max()
                assert np.abs(got[a][m] - vel[a][m]).max() <= 1e-7 * scale, (k, a)
            gp, cp = got[3][act_p], p[act_p]
            d = (gp - gp.mean()) - (cp - cp.mean())
            assert np.abs(d).max() <= 1e-6 * np.abs(cp - cp.mean()).max(), k
            bound = 1e-9 * max(np.abs(v).max() for v in vel) * 20   # velocity scale / h, h = 1/20
            assert rec["divergence_max"] <= bound and div <= bound, (rec, div)
            assert rec["pressure_iterations"] > 0 and min(rec["momentum_iterations"]) > 0
    finally:
        ctx.close()


def test_channel_with_an_immersed_sphere_runs_and_stays_bounded():
    """The immersed-body channel at a reduced size: markers on an icosphere
    force the momentum equations (interpolate, move, forces, spread), the
    outlet pressure system is solved by BiCGStab; every step ends with a
    finite, bounded velocity, and a control balance below 5% of the inflow
    flux through a cell face (its largest values sit at the outlet, where the
    outflow velocity is a PreDefined border value, as the reference's sectors
    require, rather than a projected one)."""
    ctx = xf.Context(0)
    try:
        st = tl.channel(64, 16, 16, tau=2e-3)
        loop = tl.SplittingLoop(ctx, st, markers=tl.sphere_markers((1.0, 0.5, 0.5), 0.15, subdiv=2))
        for k in range(4):
            rec = loop.step()
            u = loop.fields()[0]
            assert np.isfinite(u).all() and np.abs(u).max() < 10.0, (k, rec)
            assert rec["divergence_max"] * (4.0 / 64) < 0.05, rec
    finally:
        ctx.close()


def scalar_channel(nx, ny, nz):
    st = tl.channel(nx, ny, nz, tau=2e-3, outflow="convective", walls="free_slip")
    return tl.with_scalar(st, tl.gaussian_inlet(st["p"][0].shape, st["h"], sigma=0.15))


def test_scalar_channel_three_steps_match_the_cpu_restatement():
    """The channel with a convective, flux-balanced outflow, free-slip walls
    (lagged zero-gradient tangential border values) and a passive scalar
    entering as a Gaussian blob on the inlet: three steps against the CPU
    restatement (the oracle's pinned passes, its restatement of the outflow
    pass, numpy solves).  Bar: velocities within 1e-7 of their range,
    zero-mean pressure within 1e-6, scalar within 1e-7 of its inlet peak;
    the outlet's flux equals the inlet's to rounding."""
    import copy

    import timeloop_cpu

    ctx = xf.Context(0)
    try:
        st = scalar_channel(24, 8, 8)
        cpu = copy.deepcopy(st)
        loop = tl.SplittingLoop(ctx, st, momentum_rtol=1e-13, pressure_rtol=1e-11, pressure_solver="fp64",
                                scalar_rtol=1e-13)
        vel = [v.copy() for v in cpu["vel0"]]
        p = np.zeros(cpu["p"][0].shape)
        c = cpu["scalar"]["c0"].copy()
        act_p = cpu["p"][0] == 1
        for k in range(3):
            rec = loop.step()
            vel, p, (div, ijk), c = timeloop_cpu.step(cpu, vel, p, scalar=c)
            got = loop.fields()
            for a in range(3):
                m = cpu["comps"][a][0] != 0
                scale = np.abs(vel[a][m]).max()
                assert np.abs(got[a][m] - vel[a][m]).max() <= 1e-7 * scale, (k, a)
            gp, cp = got[3][act_p], p[act_p]
            d = (gp - gp.mean()) - (cp - cp.mean())
            assert np.abs(d).max() <= 1e-6 * np.abs(cp - cp.mean()).max(), k
            mc = cpu["scalar"]["codes"] != 0
            assert np.abs(got[4][mc] - c[mc]).max() <= 1e-7, k
            assert rec["scalar_iterations"] > 0 and rec["pressure_iterations"] > 0
            u = got[0]
            assert abs(u[-1, 1:-1, 1:-1].sum() - u[0, 1:-1, 1:-1].sum()) <= 1e-12 * u[0, 1:-1, 1:-1].sum()
        inner = got[4][cpu["scalar"]["codes"] == 1]
        assert 0.01 < inner.max() <= 1.0 and inner.min() >= -1e-12   # the blob entered, bounded
    finally:
        ctx.close()


def test_learned_and_mixed_pressure_solves_stay_on_the_fp64_trajectory():
    """Warm-started pressure solves by mixed-precision CG and by the learned
    two-level FCG (untrained network: its fallback keeps it convergent) give
    the plain FP64 run's fields after three steps, within a few times the
    pressure tolerance (1e-8)."""
    ctx = xf.Context(0)
    try:
        runs = {}
        for solver in ("fp64", "mixed", "learned"):
            st = scalar_channel(128, 32, 32)   # h = 1/32 on every axis (the two-level solver's coarse grid is
            # isotropic), coarse interior 32x8x8 (the network wants 8 or more cells per axis)
            loop = tl.SplittingLoop(ctx, st, pressure_solver=solver,
                                    net_params=xf.unet_init_params(1) if solver == "learned" else None)
            for _ in range(3):
                rec = loop.step()
            runs[solver] = loop.fields()
            assert rec["pressure_iterations"] > 0, solver
            del loop
        ref = runs["fp64"]
        for solver in ("mixed", "learned"):
            for a in range(3):
                scale = np.abs(ref[a]).max()
                assert np.abs(runs[solver][a] - ref[a]).max() <= 1e-6 * scale, (solver, a)
            assert np.abs(runs[solver][4] - ref[4]).max() <= 1e-6, solver
    finally:
        ctx.close()


def test_outflow_pass_matches_its_cpu_restatement():
    """xf_outflow_convective against tests/timeloop_cpu.py's restatement on a non-uniform state: the upwind
    step and the common shift agree to rounding (the device sums in a fixed tree, numpy in its own order), and
    the outlet's area-weighted flux equals the inlet's."""
    import timeloop_cpu

    ctx = xf.Context(0)
    try:
        st = tl.channel(24, 10, 12, outflow="convective")
        codes, nrm, bc = st["comps"][0]
        hp = st["p"][3]
        h = [0.5 * (hp[0][:-1] + hp[0][1:]), hp[1], hp[2]]
        g = xf.Grid(ctx, codes, *h, nrm)
        rng = np.random.Generator(np.random.PCG64(21))
        vel = np.where(codes == tl.ACTUAL, 1 + 0.3 * rng.standard_normal(codes.shape), 0.0)
        bc = bc.copy()
        bc[0, 1:-1, 1:-1] = 1 + 0.2 * rng.standard_normal(bc[0, 1:-1, 1:-1].shape)
        bc[-1, 1:-1, 1:-1] = 1 + 0.2 * rng.standard_normal(bc[-1, 1:-1, 1:-1].shape)
        bv = g.vec(bc)
        xf.outflow_convective(g.vec(vel), bv, 1, 1.0, st["tau"])
        got = bv.download()
        want = bc.copy()
        timeloop_cpu.outflow_convective(codes, vel, want, h, 1, 1.0, st["tau"])
        assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()
        np.testing.assert_array_equal(got[:-1], bc[:-1])   # only the outlet face changes
        assert abs(got[-1, 1:-1, 1:-1].sum() - got[0, 1:-1, 1:-1].sum()) <= 1e-12 * got[0].sum()
    finally:
        ctx.close()
