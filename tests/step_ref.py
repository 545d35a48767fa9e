"""Shared pieces of the time-step parity tests against the reference's own
two-step run (tests/golden/step_channel.npz, written by make_golden.py step
through oracle/ref_driver's `step` task).

Step 2 of TVPProblem::SolveBySplitting is the case: its inputs are the state
the reference left after step 1 (velocities s1_u/v/w, concentration s1_cnc,
viscosity s1_vis) plus the statement's border values and forces; its
outputs are the pressure right-hand side, the corrected velocities, the
control balance, the ADI line systems of the three momentum equations and
the VTK file.  The intermediate velocity u_ (int_u/v/w) comes from the same
run with step 2's pressure solve replaced by p = 0."""
import numpy as np

from helpers import golden


def load():
    G = golden("step_channel")
    G["tau"], G["mu1"], G["mu2"], G["rho1"], G["rho2"] = (float(t) for t in G["params"])
    for pre in "puvwn":
        G["h" + pre] = [np.diff(G[f"{pre}_{a}"]) for a in "xyz"]
    # density as the reference recomputes it from the concentration
    # (XProblem.cpp:5960-5966): after step 1 (step 2's input) and after step 2
    G["dens1"] = G["s1_cnc"] * (G["rho2"] - G["rho1"]) + G["rho1"]
    G["dens2"] = G["cnc"] * (G["rho2"] - G["rho1"]) + G["rho1"]
    return G


def density_mask(pc):
    """The density grid's codes built from the pressure grid's (XProblem.cpp:4700-4760)."""
    N, L, M = (s - 1 for s in pc.shape)
    d = pc.copy()
    for i, j, k in zip(*np.nonzero((pc == 4) | (pc == 0))):
        m = pc[i, j, k]
        if m == 4:
            d[i, j, k] = 4 if (i == 0 or j == 0 or k == 0) else 6
        elif (j in (0, L)) and i not in (0, N) and k not in (0, M):
            d[i, j, k] = 6
        elif (k in (0, M)) and i not in (0, N) and j not in (0, L):
            d[i, j, k] = 6
        elif (i in (0, N)) and k not in (0, M) and j not in (0, L):
            d[i, j, k] = 6
    return d


def conc_mask(pc, comps):
    """The concentration grid's codes: PreNormal everywhere when no inlet mask
    is given (XProblem.cpp:4566-4575), with each momentum equation's box
    interior made Actual on the way (XProblem.cpp:5308-5319)."""
    c = np.full(pc.shape, 6, np.int32)
    for cc in comps:
        N, L, M = (s - 1 for s in cc.shape)
        c[1:N, 1:L, 1:M] = 1
    return c


def sectors(codes, direction):
    """The ADI line sectors of a box along `direction` in the reference's
    order (XProblem.cpp:2903-2945): lists of cells from the opening border
    point through the Actual points to the closing one."""
    n1, n2, n3 = codes.shape
    d1e, d2e, de = {1: (n3, n2, n1), 2: (n3, n1, n2), 3: (n2, n1, n3)}[direction]
    out = []
    for d1 in range(d1e):
        for d2 in range(d2e):
            beg = -1
            for t in range(de):
                cell = {1: (t, d2, d1), 2: (d2, t, d1), 3: (d2, d1, t)}[direction]
                if beg < 0:
                    if codes[cell] == 1:
                        beg = t - 1
                elif codes[cell] != 1:
                    out.append([{1: (q, d2, d1), 2: (d2, q, d1), 3: (d2, d1, q)}[direction] for q in range(beg, t + 1)])
                    beg = -1
    return out


def line_mismatches(G, momentum_fields, adi_line_coeffs, adi_first_rhs):
    """Compares the captured step-2 line systems of the three momentum
    equations (x, y, z sweeps in call order) with the coefficients built from
    `momentum_fields(axis)` = (uTr, vTr, wTr, visTr, rp): a, b, c of every
    Actual row in all three sweeps, and f of the first (x) sweep.  Returns
    ({(axis, direction): mismatching rows}, number of line calls used)."""
    lm = G["line_m"]
    off = np.concatenate([[0], np.cumsum(lm + 1)])
    call = 0
    bad = {}
    for axis, c in ((1, "u"), (2, "v"), (3, "w")):
        cc, hh = G[c + "_codes"], G["h" + c]
        uT, vT, wT, visT, rp = momentum_fields(axis)
        f1 = adi_first_rhs(cc, *hh, G["s1_" + c], uT, vT, wT, visT, rp, G["tau"])
        for direction, vt in ((1, uT), (2, vT), (3, wT)):
            a, b, cf = adi_line_coeffs(direction, cc, *hh, vt, visT, G["tau"])
            nb = 0
            for cells in sectors(cc, direction):
                M, o = int(lm[call]), int(off[call])
                fl = 0 if cc[cells[0]] in (3, 7) else 1
                fr = 0 if cc[cells[-1]] in (3, 7) else 1
                assert M == len(cells) - 1 + fl + fr, "line layout differs from the sector scan"
                for r in range(1 + fl, M - fr):
                    cell = cells[r - fl]
                    if (G["line_a"][o + r], G["line_b"][o + r], G["line_c"][o + r]) != (a[cell], b[cell], cf[cell]):
                        nb += 1
                    if direction == 1 and G["line_f"][o + r] != f1[cell]:
                        nb += 1
                call += 1
            bad[(axis, direction)] = nb
    return bad, call


def conc_codes(G):
    return conc_mask(G["p_codes"], [G[c + "_codes"] for c in "uvw"])


def conc_line_mismatches(G, transfer, adi_upwind_coeffs, adi_first_rhs_upwind):
    """Compares the captured step-2 line systems of the concentration equation
    (SolveTransferEquation_ with schemeType 1 and diffusion 0, the calls after
    the three momentum equations') with the upwind coefficients built from
    `transfer` = (uTr, vTr, wTr, rpTr) on the concentration grid: a, b, c of
    every Actual row in all three sweeps, f of the first.  Returns
    ({direction: mismatching rows}, {direction: rows}, index after the last
    call used)."""
    lm = G["line_m"]
    off = np.concatenate([[0], np.cumsum(lm + 1)])
    call = sum(len(sectors(G[c + "_codes"], d)) for c in "uvw" for d in (1, 2, 3))
    cc, hh = conc_codes(G), G["hp"]
    uT, vT, wT, rp = transfer
    f1 = adi_first_rhs_upwind(cc, *hh, G["s1_cnc"], uT, vT, wT, 0.0, rp, G["tau"])
    bad, rows = {}, {}
    for direction, vt in ((1, uT), (2, vT), (3, wT)):
        a, b, cf = adi_upwind_coeffs(direction, cc, *hh, vt, 0.0, G["tau"])
        nb = nr = 0
        for cells in sectors(cc, direction):
            M, o = int(lm[call]), int(off[call])
            fl = 0 if cc[cells[0]] in (3, 7) else 1
            fr = 0 if cc[cells[-1]] in (3, 7) else 1
            assert M == len(cells) - 1 + fl + fr, "line layout differs from the sector scan"
            for r in range(1 + fl, M - fr):
                cell = cells[r - fl]
                nr += 1
                if (G["line_a"][o + r], G["line_b"][o + r], G["line_c"][o + r]) != (a[cell], b[cell], cf[cell]):
                    nb += 1
                if direction == 1 and G["line_f"][o + r] != f1[cell]:
                    nb += 1
            call += 1
        bad[direction], rows[direction] = nb, nr
    return bad, rows, call
