"""Staggered channel cases for the time-step passes around the pressure solve
(TVPProblem::SolveBySplitting, XProblem.cpp:5474-5829).

Pressure box n1 x n2 x n3 with a Fictive ghost layer, Actual interior, a
masked (Fictive) sphere, and PreDefined cells on the outlet face; u box
(n1-1) x n2 x n3 with a Defined inflow face (border value U_in) and a
PreDefined outflow face whose values mirror the interior as the reference's
check demands; v and w boxes with Fictive ghosts.  Separations are seeded and
non-uniform so that every index of hxU/hyV/hzW and hxP/hyP/hzP is exercised.
"""
import numpy as np

U_IN = 1.25


def _seps(rng, n):
    return rng.uniform(0.8, 1.2, n - 1) / (n - 1)


def channel(n1=14, n2=11, n3=12, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    hP = [_seps(rng, n) for n in (n1, n2, n3)]
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
