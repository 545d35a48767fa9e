// The time-step passes on either side of the pressure solve
// (TVPProblem::SolveBySplitting):
//
//  xf_pressure_rhs      right-hand side of the pressure equation,
//                       XProblem.cpp:5474-5512;
//  xf_velocity_correct  projection of one staggered velocity component,
//                       XProblem.cpp:5598-5777;
//  xf_divergence_max    the "control balance" check, XProblem.cpp:5782-5829;
//  xf_momentum_rhs      transfer velocities, face viscosity and right-hand
//                       side of one velocity equation, XProblem.cpp:5088-5419;
//  xf_conc_transfer     transfer velocities and right-hand side of the
//                       concentration equation, XProblem.cpp:5886-5935.
//
// Staggered boxes follow the reference's grids (XStatement.h:127-135): with the
// pressure box n1 x n2 x n3, the u box is (n1-1) x n2 x n3, v is n1 x (n2-1) x n3
// and w is n1 x n2 x (n3-1), all C order; each velocity box's own grid carries
// the separations the reference reads (hxU, hyV, hzW).  One thread per cell, the
// reference's expressions and operation order (FP64, no contraction): results
// are bit-identical to its loops.
//
// The reference throws at the first offending cell of its loop; here every
// offending cell reports its index to a per-kind minimum (atomicMin) in the
// context scratch, and the host turns the first one in the reference's loop
// order into the status and message.
#include <math.h>

#include "xf_common.cuh"

enum { PC_FICTIVE = 0, PC_ACTUAL = 1, PC_DEFINED = 3, PC_PREDEFINED = 4, PC_NORMAL = 5, PC_PRENORMAL = 6,
       PC_EQUATION = 7, PC_PREEQUATION = 8 };

// Error kinds, each the minimum offending cell in iscalars[CHK0 + kind].
enum { CHK0 = 48, E_RANGE = 0, E_NOTIMPL_P, E_UNKNOWN, E_DEFINED, E_PREDEF_NONE, E_PREDEF_MANY, E_PREDEF_VALUE,
       E_NOTIMPL_V, E_NOTIMPL_EQ, E_NOTIMPL_C, E_RANGE_C, E_COUNT };
constexpr long long NO_CELL = 0x7f7f7f7f7f7f7f7fLL;   // cudaMemset byte 0x7f
constexpr int SL_STEP = 8;                              // reduction slot of xf_divergence_max (and SL_STEP + 1)

__device__ __forceinline__ void report(DevScratch* S, int kind, long long cell) {
  atomicMin(&S->iscalars[CHK0 + kind], cell);
}

// a / b correctly rounded, from y = RN(1/b) (the grid's reciprocal tables,
// or 1/tau from the host).  q = RN(a y) lies within an ulp of a / b, the
// residual r = a - b q is exact (one FMA), and RN(q + r y) = RN(a / b):
// Markstein's theorem for FMA-based division (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990; also Muller et al., Handbook of Floating-Point
// Arithmetic, ch. 5).  Three FP64 operations instead of the IEEE division's
// reciprocal iteration, which matters at GB300's FP64 rate (1/58 of FP32).
// The theorem needs a normal, unclamped residual: a numerator or quotient
// outside [2^-950, 2^1000) in magnitude (zero, tiny, huge, not finite, or a
// divisor of 0 or infinity) takes the IEEE division itself.  Checked bit for
// bit against the IEEE division by xf_selftest_division.
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  const double q = a * y;
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu, eq = ((unsigned)__double2hiint(q) >> 20) & 0x7ffu;
  if (ea - (1023u - 950u) >= 1950u || eq - (1023u - 950u) >= 1950u) return a / b;
  const double r = fma(-b, q, a);
  return fma(r, y, q);
}

// (i, j, k) of flat cell c in a box with strides s1 = b2 b3, s2 = b3: 32-bit
// divisions for boxes below 2^32 cells, 64-bit ones (a software routine of
// about a hundred instructions each) above.
template <bool SMALL>
__device__ __forceinline__ void split3(int64_t c, int64_t s1, int64_t s2, int& i, int& j, int& k) {
  if (SMALL) {
    const unsigned cc = (unsigned)c, t1 = (unsigned)s1, t2 = (unsigned)s2;
    const unsigned ii = cc / t1, r = cc - ii * t1, jj = r / t2;
    i = (int)ii;
    j = (int)jj;
    k = (int)(r - jj * t2);
  } else {
    i = (int)(c / s1);
    j = (int)((c - i * s1) / s2);
    k = (int)(c - i * s1 - j * s2);
  }
}

// Launch of a kernel templated on SMALL (box below 2^32 cells).
#define XF_LAUNCH_BOX(kern, ncell, grid, block, ...)                                      \
  do {                                                                                    \
    if ((ncell) < (1ll << 32)) kern<true><<<(grid), (block), 0, ctx->stream>>>(__VA_ARGS__); \
    else kern<false><<<(grid), (block), 0, ctx->stream>>>(__VA_ARGS__);                    \
  } while (0)

template <bool SMALL>
__global__ void k_pressure_rhs(const uint8_t* __restrict__ code, int n1, int n2, int n3, const double* __restrict__ u,
                               const double* __restrict__ v, const double* __restrict__ w,
                               const double* __restrict__ hxU, const double* __restrict__ hyV,
                               const double* __restrict__ hzW, const double* __restrict__ rhxU,
                               const double* __restrict__ rhyV, const double* __restrict__ rhzW,
                               const double* __restrict__ rho, double tau, double rtau,
                               const double* __restrict__ border, double* __restrict__ rhs, DevScratch* S) {
  const int64_t n = (int64_t)n1 * n2 * n3;
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int64_t sv1 = (int64_t)(n2 - 1) * n3, sw1 = (int64_t)n2 * (n3 - 1), sw2 = n3 - 1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int m = code[c];
    if (m == PC_FICTIVE) {
      rhs[c] = 0;
    } else if (m == PC_ACTUAL) {
      int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
      if (i < 1 || i > n1 - 2 || j < 1 || j > n2 - 2 || k < 1 || k > n3 - 2) {
        report(S, E_RANGE, c);   // the reference would read outside the velocity boxes
        continue;
      }
      const int64_t cu = i * s1 + j * s2 + k;            // u box: (n1-1) x n2 x n3
      const int64_t cv = i * sv1 + j * s2 + k;           // v box: n1 x (n2-1) x n3
      const int64_t cw = i * sw1 + j * sw2 + k;          // w box: n1 x n2 x (n3-1)
      const double u_i_1 = u[cu - s1], u_i = u[cu];
      const double v_j_1 = v[cv - s2], v_j = v[cv];
      const double w_k_1 = w[cw - 1], w_k = w[cw];
      const double d = rho ? rho[c] : 1.0;
      const double div_ = d * d * div_rcp(u_i - u_i_1, hxU[i - 1], rhxU[i - 1]) +
                          div_rcp(v_j - v_j_1, hyV[j - 1], rhyV[j - 1]) + div_rcp(w_k - w_k_1, hzW[k - 1], rhzW[k - 1]);
      rhs[c] = -div_rcp(div_, tau, rtau);
    } else if (m == PC_PREDEFINED) {
      rhs[c] = border ? border[c] : 0.0;
    } else if (m == PC_PRENORMAL || m == PC_DEFINED || m == PC_NORMAL || m == PC_EQUATION || m == PC_PREEQUATION) {
      report(S, E_NOTIMPL_P, c);
    } else {
      report(S, E_UNKNOWN, c);
    }
  }
}

// Velocity correction, pass 1 (every cell but PreDefined ones): axis 1..3;
// the velocity box is b1 x b2 x b3, the pressure box has one more layer along
// the axis.
template <bool SMALL>
__global__ void k_vel_pass1(int axis, const uint8_t* __restrict__ code, int b1, int b2, int b3,
                            const double* __restrict__ prev, double* __restrict__ cur, const double* __restrict__ p,
                            const double* __restrict__ hP, const double* __restrict__ rhP,
                            const double* __restrict__ rho, double tau, const double* __restrict__ border,
                            DevScratch* S) {
  const int64_t n = (int64_t)b1 * b2 * b3;
  const int64_t s1 = (int64_t)b2 * b3, s2 = b3;
  const int p2 = axis == 2 ? b2 + 1 : b2, p3 = axis == 3 ? b3 + 1 : b3;
  const int64_t ps1 = (int64_t)p2 * p3, ps2 = p3;
  const int64_t pstep = axis == 1 ? ps1 : axis == 2 ? ps2 : 1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int m = code[c];
    if (m == PC_PREDEFINED) continue;
    if (m == PC_FICTIVE) {
      cur[c] = 0;
    } else if (m == PC_ACTUAL || m == PC_NORMAL || m == PC_EQUATION) {
      int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
      const int64_t cp = i * ps1 + j * ps2 + k;
      const int ih = axis == 1 ? i : axis == 2 ? j : k;
      const double gradP = div_rcp(p[cp + pstep] - p[cp], hP[ih], rhP[ih]);
      cur[c] = prev[c] - tau * gradP / (rho ? rho[cp] : 1.0);
    } else if (m == PC_DEFINED) {
      const double defVal = border ? border[c] : 0.0;
      if (prev[c] != defVal) report(S, E_DEFINED, c);
      cur[c] = defVal;
    } else if (m == PC_PRENORMAL || m == PC_PREEQUATION) {
      report(S, E_NOTIMPL_V, c);
    } else {
      report(S, E_UNKNOWN, c);
    }
  }
}

// Pass 2: PreDefined cells mirror their single Actual neighbour about the
// border value.
template <bool SMALL>
// (check = false: only the assignment, the closing border recalculation of
// the reference's ADI sweeps for PreDefined sector ends, XProblem.cpp:2996-3003)
__global__ void k_vel_pass2(const uint8_t* __restrict__ code, int b1, int b2, int b3, const double* __restrict__ prev,
                            double* __restrict__ cur, const double* __restrict__ border, DevScratch* S,
                            bool check = true) {
  const int64_t n = (int64_t)b1 * b2 * b3;
  const int64_t s1 = (int64_t)b2 * b3, s2 = b3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (code[c] != PC_PREDEFINED) continue;
    int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
    const double defVal = border ? border[c] : 0.0;
    int64_t nb = -1;
    int count = 0;
    for (int dir = 1; dir < 4; dir++)
      for (int sign = 0; sign < 2; sign++) {
        const int shift = -1 + sign * 2;
        const int ii = dir == 1 ? i + shift : i, jj = dir == 2 ? j + shift : j, kk = dir == 3 ? k + shift : k;
        if (ii >= 0 && ii < b1 && jj >= 0 && jj < b2 && kk >= 0 && kk < b3) {
          const int64_t q = ii * s1 + jj * s2 + kk;
          if (code[q] == PC_ACTUAL) {
            nb = q;
            count++;
          }
        }
      }
    if (count <= 0) { report(S, E_PREDEF_NONE, c); continue; }
    if (count > 1) { report(S, E_PREDEF_MANY, c); continue; }
    if (check && fabs(prev[c] - (2 * defVal - prev[nb])) > 1e-10) report(S, E_PREDEF_VALUE, c);
    cur[c] = 2 * defVal - cur[nb];
  }
}

// Control balance: first strict maximum of |div u| over Actual pressure cells.
template <bool SMALL>
__global__ void __launch_bounds__(RED_THREADS) k_div_max(const uint8_t* __restrict__ code, int n1, int n2, int n3,
                                                         const double* __restrict__ u, const double* __restrict__ v,
                                                         const double* __restrict__ w, const double* __restrict__ hxU,
                                                         const double* __restrict__ hyV,
                                                         const double* __restrict__ hzW,
                                                         const double* __restrict__ rhxU,
                                                         const double* __restrict__ rhyV,
                                                         const double* __restrict__ rhzW, DevScratch* S, int slot) {
  __shared__ AbsMax sh[32];
  __shared__ bool last;
  const int64_t n = (int64_t)n1 * n2 * n3;
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int64_t sv1 = (int64_t)(n2 - 1) * n3, sw1 = (int64_t)n2 * (n3 - 1), sw2 = n3 - 1;
  AbsMax best;
  best.v = 0.0;
  best.c = -1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (code[c] != PC_ACTUAL) continue;
    int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
    if (i < 1 || i > n1 - 2 || j < 1 || j > n2 - 2 || k < 1 || k > n3 - 2) {
      report(S, E_RANGE, c);   // the reference would read outside the velocity boxes
      continue;
    }
    const int64_t cu = i * s1 + j * s2 + k, cv = i * sv1 + j * s2 + k, cw = i * sw1 + j * sw2 + k;
    const double div = div_rcp(u[cu] - u[cu - s1], hxU[i - 1], rhxU[i - 1]) +
                       div_rcp(v[cv] - v[cv - s2], hyV[j - 1], rhyV[j - 1]) +
                       div_rcp(w[cw] - w[cw - 1], hzW[k - 1], rhzW[k - 1]);
    const double a = fabs(div);
    if (a > best.v) { best.v = a; best.c = c; }   // NaN never wins, as in the reference
  }
  AbsMax r = am_block(best, sh);
  if (threadIdx.x == 0) {
    S->partials[slot][blockIdx.x] = r.v;
    S->partials[slot + 1][blockIdx.x] = (double)r.c;
    __threadfence();
    unsigned int t = atomicAdd(&S->tickets[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  AbsMax q;
  q.v = 0.0;
  q.c = -1;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    AbsMax x;
    x.v = __ldcg(&S->partials[slot][b]);
    x.c = (long long)__ldcg(&S->partials[slot + 1][b]);
    q = am_combine(q, x);
  }
  q = am_block(q, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = q.c >= 0 ? q.v : 0.0;
    S->scalars[slot + 1] = (double)q.c;
    S->tickets[slot] = 0;
  }
}

// Momentum right-hand side, pass 1 (XProblem.cpp:5088-5305) with pass 2
// (:5310-5350) folded in: every cell of the component box b1 x b2 x b3 of
// velocity `axis`.  The staggered boxes have the pressure box's strides less
// one layer along their own axis; vis is the pressure box.
struct MomArgs {
  int axis, b1, b2, b3;
  const uint8_t* code;
  const uint8_t* nflag;
  const double *u, *v, *w, *vis, *border, *force;
  const double *hx, *hy, *hz;
  const double *rhhx, *rhhy, *rhhz;   // RN(2 / (h[i-1] + h[i])) per index
  double *uTr, *vTr, *wTr, *visTr, *rp;
  DevScratch* S;
};

template <bool SMALL>
__global__ void k_mom_transfer(MomArgs a) {
  const int64_t n = (int64_t)a.b1 * a.b2 * a.b3;
  const int64_t s1 = (int64_t)a.b2 * a.b3, s2 = a.b3;
  const int n2 = a.b2 + (a.axis == 2), n3 = a.b3 + (a.axis == 3);
  const int64_t us1 = (int64_t)n2 * n3, us2 = n3;
  const int64_t vs1 = (int64_t)(n2 - 1) * n3, vs2 = n3;
  const int64_t ws1 = (int64_t)n2 * (n3 - 1), ws2 = n3 - 1;
  const int64_t ps1 = (int64_t)n2 * n3, ps2 = n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int m = a.code[c];
    double ut = 0, vt = 0, wt = 0, vist = 0, r = 0;
    if (m == PC_FICTIVE) {
    } else if (m == PC_ACTUAL) {
      int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
      if (i < 1 || i > a.b1 - 2 || j < 1 || j > a.b2 - 2 || k < 1 || k > a.b3 - 2) {
        report(a.S, E_RANGE, c);   // the reference would read outside the boxes
        continue;
      }
      const int64_t cu = i * us1 + j * us2 + k, cv = i * vs1 + j * vs2 + k, cw = i * ws1 + j * ws2 + k;
      const int64_t cp = i * ps1 + j * ps2 + k;
      const double* u = a.u;
      const double* v = a.v;
      const double* w = a.w;
      if (a.axis == 1) {
        ut = u[cu];
        vt = (v[cv] + v[cv + vs1] + v[cv - vs2] + v[cv + vs1 - vs2]) / 4;
        wt = (w[cw] + w[cw + ws1] + w[cw - 1] + w[cw + ws1 - 1]) / 4;
        if (a.vis) vist = (a.vis[cp] + a.vis[cp + ps1]) / 2;
      } else if (a.axis == 2) {
        ut = (u[cu] + u[cu + us2] + u[cu - us1] + u[cu - us1 + us2]) / 4;
        vt = v[cv];
        wt = (w[cw] + w[cw + ws2] + w[cw - 1] + w[cw + ws2 - 1]) / 4;
        if (a.vis) vist = (a.vis[cp] + a.vis[cp + ps2]) / 2;
      } else {
        ut = (u[cu] + u[cu + 1] + u[cu - us1] + u[cu - us1 + 1]) / 4;
        vt = (v[cv] + v[cv + 1] + v[cv - vs2] + v[cv - vs2 + 1]) / 4;
        wt = w[cw];
        if (a.vis) vist = (a.vis[cp] + a.vis[cp + 1]) / 2;
      }
      r = a.force ? a.force[c] : 0.0;   // GetForce replaces the Actual rows' zero
    } else if (m == PC_DEFINED || m == PC_PREDEFINED) {
      r = a.border ? a.border[c] : 0.0;
    } else if (m == PC_NORMAL) {
      if (a.axis != 1 || a.nflag[c] != 1) { report(a.S, E_NOTIMPL_EQ, c); continue; }
      r = a.border ? a.border[c] : 0.0;
    } else if (m == PC_EQUATION || m == PC_PRENORMAL || m == PC_PREEQUATION) {
      report(a.S, E_NOTIMPL_V, c);
      continue;
    } else {
      report(a.S, E_UNKNOWN, c);
      continue;
    }
    a.uTr[c] = ut; a.vTr[c] = vt; a.wTr[c] = wt; a.visTr[c] = vist; a.rp[c] = r;
  }
}

// Pass 3 (XProblem.cpp:5352-5419): rp += dVis . (dVel + dU) on Actual cells.
template <bool SMALL>
__global__ void k_mom_viscous(MomArgs a) {
  const int64_t n = (int64_t)a.b1 * a.b2 * a.b3;
  const int64_t s1 = (int64_t)a.b2 * a.b3, s2 = a.b3;
  const int64_t st = a.axis == 1 ? s1 : a.axis == 2 ? s2 : 1;
  const double* velTr = a.axis == 1 ? a.uTr : a.axis == 2 ? a.vTr : a.wTr;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (a.code[c] != PC_ACTUAL) continue;
    int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
    const double ddx = a.hx[i] + a.hx[i - 1], ddy = a.hy[j] + a.hy[j - 1], ddz = a.hz[k] + a.hz[k - 1];
    // RN(1/(h[i-1] + h[i])) = RN(1/hh) / 2 exactly, hh = (h[i-1] + h[i]) / 2
    const double rdx = 0.5 * a.rhhx[i], rdy = 0.5 * a.rhhy[j], rdz = 0.5 * a.rhhz[k];
    const double dVisX = div_rcp(a.visTr[c + s1] - a.visTr[c - s1], ddx, rdx);
    const double dVisY = div_rcp(a.visTr[c + s2] - a.visTr[c - s2], ddy, rdy);
    const double dVisZ = div_rcp(a.visTr[c + 1] - a.visTr[c - 1], ddz, rdz);
    const double dd = a.axis == 1 ? ddx : a.axis == 2 ? ddy : ddz;
    const double rd = a.axis == 1 ? rdx : a.axis == 2 ? rdy : rdz;
    const double dU = div_rcp(a.uTr[c + st] - a.uTr[c - st], dd, rd);
    const double dV = div_rcp(a.vTr[c + st] - a.vTr[c - st], dd, rd);
    const double dW = div_rcp(a.wTr[c + st] - a.wTr[c - st], dd, rd);
    const double dVelX = div_rcp(velTr[c + s1] - velTr[c - s1], ddx, rdx);
    const double dVelY = div_rcp(velTr[c + s2] - velTr[c - s2], ddy, rdy);
    const double dVelZ = div_rcp(velTr[c + 1] - velTr[c - 1], ddz, rdz);
    a.rp[c] = a.rp[c] + (dVisX * (dVelX + dU) + dVisY * (dVelY + dV) + dVisZ * (dVelZ + dW));
  }
}

// ---------------------------------------------------------------------------
static bool is_f64(const xf_vec* v) { return v && v->dtype == XF_F64; }

static int check_staggered(xf_ctx* ctx, const xf_grid* gp, const xf_vec* u, const xf_vec* v, const xf_vec* w,
                           const char* who) {
  if (!is_f64(u) || !is_f64(v) || !is_f64(w)) return xf_fail(ctx, XF_ERR_ARG, "%s: u, v, w must be FP64 boxes", who);
  const xf_grid *gu = u->g, *gv = v->g, *gw = w->g;
  if (gu->ctx != ctx || gv->ctx != ctx || gw->ctx != ctx)
    return xf_fail(ctx, XF_ERR_ARG, "%s: boxes of another context", who);
  if (gu->n1 != gp->n1 - 1 || gu->n2 != gp->n2 || gu->n3 != gp->n3 || gv->n1 != gp->n1 || gv->n2 != gp->n2 - 1 ||
      gv->n3 != gp->n3 || gw->n1 != gp->n1 || gw->n2 != gp->n2 || gw->n3 != gp->n3 - 1)
    return xf_fail(ctx, XF_ERR_ARG,
                   "%s: staggered boxes must be (n1-1,n2,n3), (n1,n2-1,n3), (n1,n2,n3-1) for a %dx%dx%d pressure box",
                   who, gp->n1, gp->n2, gp->n3);
  return XF_OK;
}

static int clear_checks(xf_ctx* ctx) {
  XF_CUDA(ctx, cudaMemsetAsync(&ctx->scratch->iscalars[CHK0], 0x7f, E_COUNT * sizeof(long long), ctx->stream));
  return XF_OK;
}

static int read_checks(xf_ctx* ctx, long long* out) {
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->iscalars[CHK0], E_COUNT * sizeof(long long),
                               cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  memcpy(out, ctx->host_scalars, E_COUNT * sizeof(long long));
  return XF_OK;
}

// The first offending cell (in flat order) among `kinds`, or -1.
static int first_error(const long long* chk, const int* kinds, int nk, long long* cell) {
  int best = -1;
  *cell = NO_CELL;
  for (int t = 0; t < nk; t++)
    if (chk[kinds[t]] < *cell) {
      *cell = chk[kinds[t]];
      best = kinds[t];
    }
  return best;
}

static const char* check_message(int kind) {
  switch (kind) {
    case E_RANGE: return "an Actual pressure cell on the box face (the reference reads outside the velocity boxes)";
    case E_NOTIMPL_P: return "Method is not implemented for this border point type of pressure";
    case E_UNKNOWN: return "Unknown point mask type";
    case E_DEFINED: return "Defined border condition checking error";
    case E_PREDEF_NONE: return "PreDefined border condition checking error - actual values count <= 0";
    case E_PREDEF_MANY: return "PreDefined border condition checking error - actual values count > 1";
    case E_PREDEF_VALUE: return "PreDefined border condition checking error - value incorrect";
    case E_NOTIMPL_V: return "Method is not implemented for this point border type of velocity";
    case E_NOTIMPL_C: return "Method is not implemented for this point border type of concentration";
    case E_RANGE_C: return "an Actual concentration cell on the box face (the reference reads outside the velocity boxes)";
    case E_NOTIMPL_EQ:
      return "Method is not implemented for this point border type of velocity and this equation number and this "
             "normal vector";
    default: return "unknown";
  }
}

static int fail_at(xf_ctx* ctx, const xf_grid* g, int kind, long long cell, const char* who) {
  const int i = (int)(cell / g->s1), j = (int)((cell - i * g->s1) / g->s2), k = (int)(cell % g->s2);
  const int st = (kind == E_DEFINED || kind == E_PREDEF_VALUE) ? XF_ERR_CHECK : XF_ERR_MASK;
  return xf_fail(ctx, st, "%s: %s at (%d, %d, %d)", who, check_message(kind), i, j, k);
}

static int same_box(const xf_vec* a, const xf_grid* g) {
  return a->g->n1 == g->n1 && a->g->n2 == g->n2 && a->g->n3 == g->n3;
}

extern "C" int xf_pressure_rhs(const xf_grid* gp, const xf_vec* u, const xf_vec* v, const xf_vec* w,
                               const xf_vec* density, double tau, const xf_vec* border, xf_vec* rhs) {
  if (!gp || !rhs) return XF_ERR_ARG;
  xf_ctx* ctx = gp->ctx;
  int st;
  if ((st = check_staggered(ctx, gp, u, v, w, "xf_pressure_rhs"))) return st;
  if (!is_f64(rhs) || !same_box(rhs, gp) || (density && (!is_f64(density) || !same_box(density, gp))) ||
      (border && (!is_f64(border) || !same_box(border, gp))))
    return xf_fail(ctx, XF_ERR_ARG, "xf_pressure_rhs: rhs, density and border must be FP64 pressure boxes");
  if (!(tau != 0)) return xf_fail(ctx, XF_ERR_ARG, "xf_pressure_rhs: tau must be nonzero");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((st = clear_checks(ctx))) return st;
  XF_LAUNCH_BOX(k_pressure_rhs, gp->ncell, grid_blocks(ctx, gp->ncell, 256), 256,
      gp->code, gp->n1, gp->n2, gp->n3, (const double*)u->data, (const double*)v->data, (const double*)w->data,
      u->g->hx, v->g->hy, w->g->hz, u->g->rhx, v->g->rhy, w->g->rhz,
      density ? (const double*)density->data : nullptr, tau, 1.0 / tau, border ? (const double*)border->data : nullptr,
      (double*)rhs->data, ctx->scratch);
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int kinds[] = {E_RANGE, E_NOTIMPL_P, E_UNKNOWN};
  const int bad = first_error(chk, kinds, 3, &cell);
  if (bad >= 0) return fail_at(ctx, gp, bad, cell, "xf_pressure_rhs");
  return XF_OK;
}

extern "C" int xf_velocity_correct(int axis, const xf_vec* vel_prev, const xf_vec* p, const xf_vec* density, double tau,
                                   const xf_vec* border, xf_vec* vel) {
  if (!vel_prev || !p || !vel) return XF_ERR_ARG;
  xf_ctx* ctx = vel->g->ctx;
  const xf_grid* gv = vel->g;
  const xf_grid* gp = p->g;
  if (axis < 1 || axis > 3) return xf_fail(ctx, XF_ERR_ARG, "xf_velocity_correct: axis must be 1, 2 or 3");
  if (!is_f64(vel_prev) || !is_f64(p) || !is_f64(vel) || !same_box(vel_prev, gv) ||
      (border && (!is_f64(border) || !same_box(border, gv))) ||
      (density && (!is_f64(density) || !same_box(density, gp))))
    return xf_fail(ctx, XF_ERR_ARG, "xf_velocity_correct: FP64 boxes of matching shapes expected");
  if (gp->n1 != gv->n1 + (axis == 1) || gp->n2 != gv->n2 + (axis == 2) || gp->n3 != gv->n3 + (axis == 3))
    return xf_fail(ctx, XF_ERR_ARG, "xf_velocity_correct: the pressure box must have one more layer along axis %d",
                   axis);
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  int st;
  if ((st = clear_checks(ctx))) return st;
  const double* hP = axis == 1 ? gp->hx : axis == 2 ? gp->hy : gp->hz;
  const double* rhP = axis == 1 ? gp->rhx : axis == 2 ? gp->rhy : gp->rhz;
  const int bl = grid_blocks(ctx, gv->ncell, 256);
  const double* bd = border ? (const double*)border->data : nullptr;
  XF_LAUNCH_BOX(k_vel_pass1, gv->ncell, bl, 256, axis, gv->code, gv->n1, gv->n2, gv->n3, (const double*)vel_prev->data,
                                           (double*)vel->data, (const double*)p->data, hP, rhP,
                                           density ? (const double*)density->data : nullptr, tau, bd, ctx->scratch);
  XF_LAUNCH_BOX(k_vel_pass2, gv->ncell, bl, 256, gv->code, gv->n1, gv->n2, gv->n3, (const double*)vel_prev->data,
                                           (double*)vel->data, bd, ctx->scratch);
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int pass1[] = {E_DEFINED, E_NOTIMPL_V, E_UNKNOWN};
  const int pass2[] = {E_PREDEF_NONE, E_PREDEF_MANY, E_PREDEF_VALUE};
  int bad = first_error(chk, pass1, 3, &cell);
  if (bad < 0) bad = first_error(chk, pass2, 3, &cell);
  if (bad >= 0) return fail_at(ctx, gv, bad, cell, "xf_velocity_correct");
  return XF_OK;
}

extern "C" int xf_divergence_max(const xf_grid* gp, const xf_vec* u, const xf_vec* v, const xf_vec* w, double* value,
                                 int32_t* ijk) {
  if (!gp || !value) return XF_ERR_ARG;
  xf_ctx* ctx = gp->ctx;
  int st;
  if ((st = check_staggered(ctx, gp, u, v, w, "xf_divergence_max"))) return st;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((st = clear_checks(ctx))) return st;
  const int bl = red_blocks(ctx, gp->ncell);
  XF_LAUNCH_BOX(k_div_max, gp->ncell, bl, RED_THREADS, gp->code, gp->n1, gp->n2, gp->n3, (const double*)u->data,
                                                 (const double*)v->data, (const double*)w->data, u->g->hx, v->g->hy,
                                                 w->g->hz, u->g->rhx, v->g->rhy, w->g->rhz, ctx->scratch, SL_STEP);
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->scalars[SL_STEP], 2 * sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const double val = ctx->host_scalars[0];
  const long long c = (long long)ctx->host_scalars[1];
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int kinds[] = {E_RANGE};
  const int bad = first_error(chk, kinds, 1, &cell);
  if (bad >= 0) return fail_at(ctx, gp, bad, cell, "xf_divergence_max");
  *value = val;
  if (ijk) {
    if (c < 0) {
      ijk[0] = ijk[1] = ijk[2] = -1;
    } else {
      ijk[0] = (int32_t)(c / gp->s1);
      ijk[1] = (int32_t)((c - ijk[0] * gp->s1) / gp->s2);
      ijk[2] = (int32_t)(c % gp->s2);
    }
  }
  return XF_OK;
}

extern "C" int xf_momentum_rhs(int axis, const xf_vec* u_prev, const xf_vec* v_prev, const xf_vec* w_prev,
                               const xf_vec* vis, const xf_vec* border, const xf_vec* force, xf_vec* u_tr,
                               xf_vec* v_tr, xf_vec* w_tr, xf_vec* vis_tr, xf_vec* rp) {
  if (!u_prev || !v_prev || !w_prev || !u_tr || !v_tr || !w_tr || !vis_tr || !rp) return XF_ERR_ARG;
  const xf_grid* gc = rp->g;   // the component's grid
  xf_ctx* ctx = gc->ctx;
  if (axis < 1 || axis > 3) return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: axis must be 1, 2 or 3");
  const xf_vec* outs[5] = {u_tr, v_tr, w_tr, vis_tr, rp};
  for (const xf_vec* o : outs)
    if (!is_f64(o) || o->g != gc)
      return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: outputs must be FP64 vectors of the component's grid");
  for (int q = 0; q < 5; q++)
    for (int r = q + 1; r < 5; r++)
      if (outs[q] == outs[r]) return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: outputs must be distinct");
  if ((border && (!is_f64(border) || !same_box(border, gc))) || (force && (!is_f64(force) || !same_box(force, gc))))
    return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: border and force must be FP64 component boxes");
  const int n1 = gc->n1 + (axis == 1), n2 = gc->n2 + (axis == 2), n3 = gc->n3 + (axis == 3);
  const xf_vec* vel[3] = {u_prev, v_prev, w_prev};
  for (int d = 0; d < 3; d++) {
    if (!is_f64(vel[d]) || vel[d]->g->ctx != ctx)
      return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: u, v, w must be FP64 boxes of this context");
    const xf_grid* g = vel[d]->g;
    if (g->n1 != n1 - (d == 0) || g->n2 != n2 - (d == 1) || g->n3 != n3 - (d == 2))
      return xf_fail(ctx, XF_ERR_ARG,
                     "xf_momentum_rhs: staggered boxes must be (n1-1,n2,n3), (n1,n2-1,n3), (n1,n2,n3-1) for the "
                     "%dx%dx%d pressure box of this component",
                     n1, n2, n3);
  }
  if (vis && (!is_f64(vis) || vis->g->n1 != n1 || vis->g->n2 != n2 || vis->g->n3 != n3))
    return xf_fail(ctx, XF_ERR_ARG, "xf_momentum_rhs: vis must be an FP64 pressure box");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  int st;
  if ((st = clear_checks(ctx))) return st;
  MomArgs a;
  a.axis = axis; a.b1 = gc->n1; a.b2 = gc->n2; a.b3 = gc->n3;
  a.code = gc->code; a.nflag = gc->nflag;
  a.u = (const double*)u_prev->data; a.v = (const double*)v_prev->data; a.w = (const double*)w_prev->data;
  a.vis = vis ? (const double*)vis->data : nullptr;
  a.border = border ? (const double*)border->data : nullptr;
  a.force = force ? (const double*)force->data : nullptr;
  a.hx = gc->hx; a.hy = gc->hy; a.hz = gc->hz;
  a.rhhx = gc->rhhx; a.rhhy = gc->rhhy; a.rhhz = gc->rhhz;
  a.uTr = (double*)u_tr->data; a.vTr = (double*)v_tr->data; a.wTr = (double*)w_tr->data;
  a.visTr = (double*)vis_tr->data; a.rp = (double*)rp->data;
  a.S = ctx->scratch;
  const int bl = grid_blocks(ctx, gc->ncell, 256);
  XF_LAUNCH_BOX(k_mom_transfer, gc->ncell, bl, 256, a);
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int kinds[] = {E_RANGE, E_NOTIMPL_V, E_NOTIMPL_EQ, E_UNKNOWN};
  const int bad = first_error(chk, kinds, 4, &cell);
  if (bad >= 0) return fail_at(ctx, gc, bad, cell, "xf_momentum_rhs");
  XF_LAUNCH_BOX(k_mom_viscous, gc->ncell, bl, 256, a);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// The concentration equation's transfer terms (TVPProblem::SolveBySplitting,
// XProblem.cpp:5886-5935) on the concentration grid (the pressure box):
// Actual points the averages of the two staggered velocities around them
// (u (n1-1) x n2 x n3, v n1 x (n2-1) x n3, w n1 x n2 x (n3-1)) and rp 0;
// PreDefined points zero velocities and, on the inlet face i = 0, the inlet
// value (ConcentrationInletCondition; NULL: 0); Fictive and PreNormal points
// zeros; every other code a throw of the reference.
template <bool SMALL>
__global__ void k_conc_transfer(const uint8_t* __restrict__ code, int n1, int n2, int n3,
                                const double* __restrict__ u, const double* __restrict__ v,
                                const double* __restrict__ w, const double* __restrict__ inlet,
                                double* __restrict__ uTr, double* __restrict__ vTr, double* __restrict__ wTr,
                                double* __restrict__ rpTr, DevScratch* S) {
  const int64_t n = (int64_t)n1 * n2 * n3;
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int64_t sv1 = (int64_t)(n2 - 1) * n3, sw1 = (int64_t)n2 * (n3 - 1), sw2 = n3 - 1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int m = code[c];
    double ut = 0, vt = 0, wt = 0, rp = 0;
    if (m == PC_ACTUAL) {
      int i, j, k;
      split3<SMALL>(c, s1, s2, i, j, k);
      if (i < 1 || i > n1 - 2 || j < 1 || j > n2 - 2 || k < 1 || k > n3 - 2) {
        report(S, E_RANGE_C, c);
        continue;
      }
      const int64_t cu = i * s1 + j * s2 + k, cv = i * sv1 + j * s2 + k, cw = i * sw1 + j * sw2 + k;
      ut = (u[cu - s1] + u[cu]) / 2;
      vt = (v[cv - s2] + v[cv]) / 2;
      wt = (w[cw - 1] + w[cw]) / 2;
    } else if (m == PC_PREDEFINED) {
      if (inlet && c < s1) rp = inlet[c];   // i == 0
    } else if (m == PC_DEFINED || m == PC_NORMAL || m == PC_EQUATION || m == PC_PREEQUATION) {
      report(S, E_NOTIMPL_C, c);
      continue;
    } else if (m != PC_FICTIVE && m != PC_PRENORMAL) {
      report(S, E_UNKNOWN, c);
      continue;
    }
    uTr[c] = ut;
    vTr[c] = vt;
    wTr[c] = wt;
    rpTr[c] = rp;
  }
}

extern "C" int xf_conc_transfer(const xf_grid* gc, const xf_vec* u, const xf_vec* v, const xf_vec* w,
                                const xf_vec* inlet, xf_vec* u_tr, xf_vec* v_tr, xf_vec* w_tr, xf_vec* rp) {
  if (!gc || !u_tr || !v_tr || !w_tr || !rp) return XF_ERR_ARG;
  xf_ctx* ctx = gc->ctx;
  int st;
  if ((st = check_staggered(ctx, gc, u, v, w, "xf_conc_transfer"))) return st;
  const xf_vec* outs[4] = {u_tr, v_tr, w_tr, rp};
  for (int q = 0; q < 4; q++) {
    if (!is_f64(outs[q]) || outs[q]->g != gc)
      return xf_fail(ctx, XF_ERR_ARG, "xf_conc_transfer: outputs must be FP64 vectors of the concentration grid");
    for (int r = q + 1; r < 4; r++)
      if (outs[q] == outs[r]) return xf_fail(ctx, XF_ERR_ARG, "xf_conc_transfer: outputs must be distinct");
  }
  if (inlet && (!is_f64(inlet) || !same_box(inlet, gc)))
    return xf_fail(ctx, XF_ERR_ARG, "xf_conc_transfer: inlet must be an FP64 box of the concentration grid");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((st = clear_checks(ctx))) return st;
  XF_LAUNCH_BOX(k_conc_transfer, gc->ncell, grid_blocks(ctx, gc->ncell, 256), 256, gc->code, gc->n1, gc->n2, gc->n3,
                (const double*)u->data, (const double*)v->data, (const double*)w->data,
                inlet ? (const double*)inlet->data : nullptr, (double*)u_tr->data, (double*)v_tr->data,
                (double*)w_tr->data, (double*)rp->data, ctx->scratch);
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int kinds[] = {E_RANGE_C, E_NOTIMPL_C, E_UNKNOWN};
  const int bad = first_error(chk, kinds, 3, &cell);
  if (bad >= 0) return fail_at(ctx, gc, bad, cell, "xf_conc_transfer");
  return XF_OK;
}

// ---------------------------------------------------------------------------
// Self-test of div_rcp against the IEEE division, bit for bit, over n hashed
// operand pairs (splitmix64 of seed and index): three quarters with the
// numerator's exponent within 2^+-60 and the divisor's within [2^-40, 2^10]
// (field differences over spacings and time steps), the rest with fully
// random bit patterns (zeros, subnormals, infinities and NaNs included).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__global__ void k_div_selftest(long long n, unsigned long long seed, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    unsigned long long ha = splitmix64(seed ^ (2ull * (unsigned long long)c)), hb = splitmix64(seed ^ (2ull * (unsigned long long)c + 1));
    if ((ha & 3ull) != 0) {   // exponents in the ranges of the step kernels' operands
      const unsigned long long ea = 1023ull - 60ull + ((ha >> 2) % 121ull), eb = 1023ull - 40ull + ((hb >> 2) % 51ull);
      ha = (ha & 0x800fffffffffffffull) | (ea << 52);
      hb = (hb & 0x800fffffffffffffull) | (eb << 52);
    }
    const double a = __longlong_as_double((long long)ha), b = __longlong_as_double((long long)hb);
    const double y = 1.0 / b;
    const double got = div_rcp(a, b, y), want = a / b;
    const bool same = __double_as_longlong(got) == __double_as_longlong(want) || (isnan(got) && isnan(want));
    if (!same) bad++;
  }
  if (bad) atomicAdd(mismatches, bad);
}

// Right-hand side of the implicit transfer equation that replaces the ADI
// sweeps of one velocity component (SolveTransferEquation__, XProblem.cpp:
// 5421 and 2784-3420): (1/tau) f_1 + rp on Actual points, the line systems'
// base term (XProblem.cpp:3192), and rp (the border value the momentum
// right-hand side put there) on the other active points, whose rows are the
// grid's border rows; inactive points keep f_1.
__global__ void k_transfer_rhs(const uint8_t* __restrict__ code, int64_t n, const double* __restrict__ f,
                               const double* __restrict__ rp, double itau, double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int m = code[c];
    double v = f[c];
    if (m == 1) v = itau * f[c] + rp[c];
    else if (m == 4 || m == 5 || m == 6 || m == 8) v = rp[c];
    out[c] = v;
  }
}

extern "C" int xf_transfer_rhs(const xf_vec* f_prev, const xf_vec* rp, double tau, xf_vec* out) {
  if (!f_prev || !rp || !out) return XF_ERR_ARG;
  const xf_grid* g = out->g;
  xf_ctx* ctx = g->ctx;
  if (!is_f64(f_prev) || !is_f64(rp) || !is_f64(out) || !same_box(f_prev, g) || !same_box(rp, g))
    return xf_fail(ctx, XF_ERR_ARG, "xf_transfer_rhs: FP64 boxes of one grid expected");
  if (!(tau != 0)) return xf_fail(ctx, XF_ERR_ARG, "xf_transfer_rhs: tau must be nonzero");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  k_transfer_rhs<<<grid_blocks(ctx, g->ncell, 256), 256, 0, ctx->stream>>>(
      g->code, g->ncell, (const double*)f_prev->data, (const double*)rp->data, 1.0 / tau, (double*)out->data);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// Defined points that end a line sector (an Actual neighbour along some axis)
// take their border value, as the ADI sweeps assign them (XProblem.cpp:
// 2975-2980 and the sector end after it).
template <bool SMALL>
__global__ void k_defined_ends(const uint8_t* __restrict__ code, int n1, int n2, int n3,
                               const double* __restrict__ border, double* __restrict__ vel) {
  const int64_t n = (int64_t)n1 * n2 * n3;
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (code[c] != PC_DEFINED) continue;
    int i, j, k;
    split3<SMALL>(c, s1, s2, i, j, k);
    const bool end = (i > 0 && code[c - s1] == PC_ACTUAL) || (i < n1 - 1 && code[c + s1] == PC_ACTUAL) ||
                     (j > 0 && code[c - s2] == PC_ACTUAL) || (j < n2 - 1 && code[c + s2] == PC_ACTUAL) ||
                     (k > 0 && code[c - 1] == PC_ACTUAL) || (k < n3 - 1 && code[c + 1] == PC_ACTUAL);
    if (end) vel[c] = border ? border[c] : 0.0;
  }
}

// The border values of an implicit transfer solve made exact, as the
// reference's ADI sweeps recalculate their sector ends (XProblem.cpp:
// 2975-3003): Defined sector ends take the border value, and every PreDefined
// point becomes 2 b - (its Actual neighbour), so that the velocity
// correction's border checks hold (exactly, and to rounding).
extern "C" int xf_border_recalc(const xf_vec* border, xf_vec* vel) {
  if (!vel) return XF_ERR_ARG;
  const xf_grid* g = vel->g;
  xf_ctx* ctx = g->ctx;
  if (!is_f64(vel) || (border && (!is_f64(border) || !same_box(border, g))))
    return xf_fail(ctx, XF_ERR_ARG, "xf_border_recalc: FP64 boxes of one grid expected");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  int st;
  if ((st = clear_checks(ctx))) return st;
  XF_LAUNCH_BOX(k_defined_ends, g->ncell, grid_blocks(ctx, g->ncell, 256), 256, g->code, g->n1, g->n2, g->n3,
                border ? (const double*)border->data : nullptr, (double*)vel->data);
  XF_LAUNCH_BOX(k_vel_pass2, g->ncell, grid_blocks(ctx, g->ncell, 256), 256, g->code, g->n1, g->n2, g->n3,
                (const double*)vel->data, (double*)vel->data, border ? (const double*)border->data : nullptr,
                ctx->scratch, false);
  long long chk[E_COUNT], cell;
  if ((st = read_checks(ctx, chk))) return st;
  const int kinds[] = {E_PREDEF_NONE, E_PREDEF_MANY};
  const int bad = first_error(chk, kinds, 2, &cell);
  if (bad >= 0) return fail_at(ctx, g, bad, cell, "xf_border_recalc");
  return XF_OK;
}

// A zero-gradient (outflow) face: each PreDefined point on face (axis, side)
// takes the current value of its Actual neighbour across the face as its
// border value, so the next step's semi-sum row makes the face value follow
// the interior (lagged by one step).
__global__ void k_border_follow(const uint8_t* __restrict__ code, int n1, int n2, int n3, int axis, int side,
                                const double* __restrict__ vel, double* __restrict__ border) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int na = axis == 0 ? n1 : axis == 1 ? n2 : n3;
  const int la = axis == 0 ? n2 : n1, lb = axis == 2 ? n2 : n3;   // the face plane's two other axes
  const int64_t np = (int64_t)la * lb;
  const int f = side ? na - 1 : 0, inward = side ? -1 : 1;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np; q += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(q / lb), y = (int)(q - (int64_t)x * lb);
    int i, j, k;
    if (axis == 0) { i = f; j = x; k = y; }
    else if (axis == 1) { i = x; j = f; k = y; }
    else { i = x; j = y; k = f; }
    const int64_t c = i * s1 + j * s2 + k;
    if (code[c] != PC_PREDEFINED) continue;
    const int64_t nb = c + inward * (axis == 0 ? s1 : axis == 1 ? s2 : 1);
    if (code[nb] == PC_ACTUAL) border[c] = vel[nb];
  }
}

extern "C" int xf_border_follow(const xf_vec* vel, xf_vec* border, int axis, int side) {
  if (!vel || !border) return XF_ERR_ARG;
  const xf_grid* g = vel->g;
  xf_ctx* ctx = g->ctx;
  if (axis < 1 || axis > 3 || (side != 0 && side != 1))
    return xf_fail(ctx, XF_ERR_ARG, "xf_border_follow: axis 1..3 and side 0 or 1 expected");
  if (!is_f64(vel) || !is_f64(border) || !same_box(border, g))
    return xf_fail(ctx, XF_ERR_ARG, "xf_border_follow: FP64 boxes of one grid expected");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t np = axis == 1 ? (int64_t)g->n2 * g->n3 : axis == 2 ? (int64_t)g->n1 * g->n3 : (int64_t)g->n1 * g->n2;
  k_border_follow<<<grid_blocks(ctx, np, 256), 256, 0, ctx->stream>>>(g->code, g->n1, g->n2, g->n3, axis - 1, side,
                                                                      (const double*)vel->data, (double*)border->data);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// A convective outflow on the high face of `axis` for the component normal to
// it: one block walks the face plane, advances each Defined outlet point's
// border value by an explicit upwind step of dv/dt + speed dv/dn = 0, sums
// the area-weighted outlet and inlet (low face) values and the outlet area in
// a fixed-order tree, then shifts the outlet so the two fluxes balance.
constexpr int OF_THREADS = 1024;

__device__ __forceinline__ double face_width(const double* __restrict__ h, int t, int n) {
  return (t >= 1 && t <= n - 2) ? (h[t - 1] + h[t]) / 2 : 0.0;   // the cell around node t
}

__global__ void __launch_bounds__(OF_THREADS)
    k_outflow_convective(const uint8_t* __restrict__ code, int n1, int n2, int n3, int axis,
                         const double* __restrict__ vel, double* __restrict__ border, const double* __restrict__ hx,
                         const double* __restrict__ hy, const double* __restrict__ hz, double speed_tau) {
  __shared__ double red[3][OF_THREADS];
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int na = axis == 0 ? n1 : axis == 1 ? n2 : n3;
  const int la = axis == 0 ? n2 : n1, lb = axis == 2 ? n2 : n3;   // the face plane's two other axes
  const double* ha = axis == 0 ? hy : hx;
  const double* hb = axis == 2 ? hy : hz;
  const double* hn = axis == 0 ? hx : axis == 1 ? hy : hz;
  const int64_t step = axis == 0 ? s1 : axis == 1 ? s2 : 1;
  const int64_t np = (int64_t)la * lb;
  const double c = speed_tau / hn[na - 2];   // Courant number across the face
  const int tid = threadIdx.x;
  double in_sum = 0, out_sum = 0, out_area = 0;
  for (int64_t q = tid; q < np; q += OF_THREADS) {
    const int x = (int)(q / lb), y = (int)(q - (int64_t)x * lb);
    int64_t c0;
    if (axis == 0) c0 = x * s2 + y;
    else if (axis == 1) c0 = x * s1 + y;
    else c0 = x * s1 + y * s2;
    const int64_t c1 = c0 + (int64_t)(na - 1) * step;
    const double w = face_width(ha, x, la) * face_width(hb, y, lb);
    if (code[c0] == PC_DEFINED) in_sum += w * border[c0];
    if (code[c1] == PC_DEFINED) {
      double v = border[c1];
      v = v - c * (v - vel[c1 - step]);
      border[c1] = v;
      out_sum += w * v;
      out_area += w;
    }
  }
  red[0][tid] = in_sum;
  red[1][tid] = out_sum;
  red[2][tid] = out_area;
  __syncthreads();
  for (int h = OF_THREADS / 2; h > 0; h >>= 1) {
    if (tid < h)
      for (int t = 0; t < 3; t++) red[t][tid] += red[t][tid + h];
    __syncthreads();
  }
  const double shift = red[2][0] > 0 ? (red[0][0] - red[1][0]) / red[2][0] : 0.0;
  for (int64_t q = tid; q < np; q += OF_THREADS) {   // each thread revisits its own points
    const int x = (int)(q / lb), y = (int)(q - (int64_t)x * lb);
    int64_t c0;
    if (axis == 0) c0 = x * s2 + y;
    else if (axis == 1) c0 = x * s1 + y;
    else c0 = x * s1 + y * s2;
    const int64_t c1 = c0 + (int64_t)(na - 1) * step;
    if (code[c1] == PC_DEFINED) border[c1] += shift;
  }
}

extern "C" int xf_outflow_convective(const xf_vec* vel, xf_vec* border, int axis, double speed, double tau) {
  if (!vel || !border) return XF_ERR_ARG;
  const xf_grid* g = vel->g;
  xf_ctx* ctx = g->ctx;
  if (axis < 1 || axis > 3) return xf_fail(ctx, XF_ERR_ARG, "xf_outflow_convective: axis 1..3 expected");
  if (!is_f64(vel) || !is_f64(border) || !same_box(border, g) || border->g != g)
    return xf_fail(ctx, XF_ERR_ARG, "xf_outflow_convective: FP64 vectors of one grid expected");
  const int na = axis == 1 ? g->n1 : axis == 2 ? g->n2 : g->n3;
  if (na < 3 || !(speed >= 0) || !(tau > 0))
    return xf_fail(ctx, XF_ERR_ARG, "xf_outflow_convective: a box of 3 layers or more, speed >= 0 and tau > 0");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  k_outflow_convective<<<1, OF_THREADS, 0, ctx->stream>>>(g->code, g->n1, g->n2, g->n3, axis - 1,
                                                          (const double*)vel->data, (double*)border->data, g->hx,
                                                          g->hy, g->hz, speed * tau);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_selftest_division(xf_ctx* ctx, long long n, unsigned long long seed, long long* mismatches) {
  if (!ctx || !mismatches || n < 0) return XF_ERR_ARG;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  unsigned long long* d = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&d, sizeof(unsigned long long), ctx->stream));
  XF_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  k_div_selftest<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(n, seed, d);
  unsigned long long h = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFreeAsync(d, ctx->stream);
  if (e != cudaSuccess) return xf_fail(ctx, XF_ERR_CUDA, "xf_selftest_division: %s", cudaGetErrorString(e));
  *mismatches = (long long)h;
  return XF_OK;
}
