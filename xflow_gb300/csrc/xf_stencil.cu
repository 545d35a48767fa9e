// Operators (T3dLaplaceOperator, T3dVariableDivergentedOperator) and the
// masked matvec y |= A(x) (+/- s) of TRnRelease3dSpace::
// LocalReleaseAssignSpeedLinearCombination(op) (XSpace.cpp:3013-3217).
//
// Kernel layout (plane march): a thread owns one (j, k) column of the box and
// walks a chunk of i-planes, keeping x[i-1], x[i], x[i+1] in registers and
// prefetching plane i+2 while it computes plane i.  Consecutive threads own
// consecutive k, so every plane access is coalesced; the j+-1 / k+-1
// neighbours are re-reads of lines the neighbouring threads just fetched (L1/L2).
#include <atomic>
#include <type_traits>

#include "xf_control.cuh"
#include "xf_stencil.cuh"

template <>
StencilGrid<double> make_stencil_grid<double>(const xf_grid* g, const double* rho) {
  StencilGrid<double> s;
  s.kind = g->kind; s.brow_of = g->brow_of; s.brow_nrm = g->brow_nrm;
  s.hx = g->hx; s.hy = g->hy; s.hz = g->hz;
  s.cxm = g->cxm; s.cxp = g->cxp; s.cym = g->cym; s.cyp = g->cyp; s.czm = g->czm; s.czp = g->czp;
  s.rhx = g->rhx; s.rhy = g->rhy; s.rhz = g->rhz; s.rhhx = g->rhhx; s.rhhy = g->rhhy; s.rhhz = g->rhhz;
  s.rho = rho;
  s.n1 = g->n1; s.n2 = g->n2; s.n3 = g->n3; s.s1 = (int)g->s1; s.s2 = (int)g->s2;
  return s;
}
template <>
StencilGrid<float> make_stencil_grid<float>(const xf_grid* g, const float* rho) {
  StencilGrid<float> s;
  s.kind = g->kind; s.brow_of = g->brow_of; s.brow_nrm = g->brow_nrm;
  s.hx = g->fhx; s.hy = g->fhy; s.hz = g->fhz;
  s.cxm = g->fxm; s.cxp = g->fxp; s.cym = g->fym; s.cyp = g->fyp; s.czm = g->fzm; s.czp = g->fzp;
  s.rhx = g->frhx; s.rhy = g->frhy; s.rhz = g->frhz; s.rhhx = g->frhhx; s.rhhy = g->frhhy; s.rhhz = g->frhhz;
  s.rho = rho;
  s.n1 = g->n1; s.n2 = g->n2; s.n3 = g->n3; s.s1 = (int)g->s1; s.s2 = (int)g->s2;
  return s;
}

constexpr int MV_THREADS = 256;

// y |= A(x) + sign*s (negated when neg), written to y (T) and/or y32 (float);
// fused FP64 dots (w, v) -> slot_w and (v, v) -> slot_w+1; the last block to
// finish runs the solver control step `ctl`.
template <typename T>
struct MatvecArgs {
  StencilGrid<T> g;
  const T* __restrict__ x;
  T* __restrict__ y;
  float* __restrict__ y32;
  const T* __restrict__ s;
  const T* __restrict__ w;
  const double* __restrict__ diag;
  int sign, neg, zero_inactive, dot_w, dot_self;
  int slot_w, ctl, gate, chunk;
  DevScratch* S;
};

// Laplace Actual row on register-resident x[i-1], x[i], x[i+1].
template <typename T, bool USE_D>
__device__ __forceinline__ T march_lap(const StencilGrid<T>& g, const MatvecArgs<T>& a, int c, int i, uint8_t kb,
                                       T xm, T xc, T xp, T xjm, T xjp, T xkm, T xkp, T cym, T cyp, T czm, T czp) {
  const T cxm = g.cxm[i], cxp = g.cxp[i];
  if (USE_D) {
    // FP64: y = D x_c - sum_n c_n x_n  (one DMUL and six DFMA per row)
    const T kpx = (kb & K_PX) ? cxp : T(0), kmx = (kb & K_MX) ? cxm : T(0);
    const T kpy = (kb & K_PY) ? cyp : T(0), kmy = (kb & K_MY) ? cym : T(0);
    const T kpz = (kb & K_PZ) ? czp : T(0), kmz = (kb & K_MZ) ? czm : T(0);
    T acc = (T)a.diag[c] * xc;
    acc = fma(-kpx, xp, acc);
    acc = fma(-kmx, xm, acc);
    acc = fma(-kpy, xjp, acc);
    acc = fma(-kmy, xjm, acc);
    acc = fma(-kpz, xkp, acc);
    acc = fma(-kmz, xkm, acc);
    return acc;
  } else {
    // FP32: the reference's difference form, c * (x_n - x_c)
    const T tpx = (kb & K_PX) ? cxp * (xp - xc) : T(0);
    const T tmx = (kb & K_MX) ? cxm * (xc - xm) : T(0);
    const T tpy = (kb & K_PY) ? cyp * (xjp - xc) : T(0);
    const T tmy = (kb & K_MY) ? cym * (xc - xjm) : T(0);
    const T tpz = (kb & K_PZ) ? czp * (xkp - xc) : T(0);
    const T tmz = (kb & K_MZ) ? czm * (xc - xkm) : T(0);
    return -(((tpx - tmx) + (tpy - tmy)) + (tpz - tmz));
  }
}

// The fast FP64 advection-diffusion rows stream ten arrays a cell: four
// blocks an SM (at most 64 registers) keep enough loads in flight.
template <typename T, int OP, bool EXACT, bool USE_D>
__global__ void __launch_bounds__(MV_THREADS, (OP == XF_OP_ADVDIFF && !EXACT) ? 4 : 1) k_matvec(MatvecArgs<T> a) {
  __shared__ double sh[32];
  __shared__ bool last;
  // Solver kernels turn into no-ops once the solve is done (or, when gated,
  // while no true-residual replacement is pending).
  if (a.ctl != CTL_NONE && (a.S->iscalars[I_DONE] || (a.gate && !a.S->iscalars[I_NEEDREP]))) return;
  const StencilGrid<T>& g = a.g;
  const int P = g.n2 * g.n3;
  const int p = blockIdx.x * MV_THREADS + threadIdx.x;
  const int i0 = blockIdx.y * a.chunk;
  const int i1 = min(g.n1, i0 + a.chunk);
  DotAcc<T> dw, ds;
  if (p < P) {
    const int j = p / g.n3, k = p - j * g.n3;
    // side offsets clamped to stay inside the box (only used by interior rows)
    const int okm = k > 0 ? -1 : 0, okp = k < g.n3 - 1 ? 1 : 0;
    const int ojm = j > 0 ? -g.n3 : 0, ojp = j < g.n2 - 1 ? g.n3 : 0;
    const bool fast = (OP == XF_OP_LAPLACE) && !EXACT;
    T cym = 0, cyp = 0, czm = 0, czp = 0;
    if (fast) { cym = g.cym[j]; cyp = g.cyp[j]; czm = g.czm[k]; czp = g.czp[k]; }
    const T* __restrict__ x = a.x;
    int c = i0 * P + p;
    T xm = i0 > 0 ? x[c - P] : T(0);
    T xc = x[c];
    T xp = i0 + 1 < g.n1 ? x[c + P] : T(0);
    uint8_t kc = g.kind[c];
    for (int i = i0; i < i1; i++, c += P) {
      const T xpp = i + 2 < g.n1 ? x[c + 2 * P] : T(0);
      const uint8_t kn = i + 1 < g.n1 ? g.kind[c + P] : (uint8_t)0;
      const T xjm = x[c + ojm], xjp = x[c + ojp], xkm = x[c + okm], xkp = x[c + okp];
      const int row = row_of(kc);
      if (row == ROW_NONE) {
        if (a.zero_inactive) {
          if (a.y) a.y[c] = T(0);
          if (a.y32) a.y32[c] = 0.f;
        }
      } else {
        T v;
        if (fast && row == ROW_ACTUAL) v = march_lap<T, USE_D>(g, a, c, i, kc, xm, xc, xp, xjm, xjp, xkm, xkp, cym, cyp, czm, czp);
        else v = apply_row<T, OP, EXACT>(g, x, i, j, k, c, kc);
        if (a.sign > 0) v = v + a.s[c];
        else if (a.sign < 0) v = v - a.s[c];
        if (a.neg) v = -v;
        if (a.dot_w) dw.add(a.w[c], v);
        if (a.dot_self) ds.add(v, v);
        if (a.y) a.y[c] = v;
        if (a.y32) a.y32[c] = (float)v;
      }
      xm = xc; xc = xp; xp = xpp; kc = kn;
    }
  }
  if (a.dot_w || a.dot_self || a.ctl != CTL_NONE) {
    double vals[2] = {dw.value(), ds.value()};
    if (publish_partials<2>(a.S, a.slot_w, vals, sh, &last)) {
      double tw = finish_partials(a.S, a.slot_w, sh);
      double ts = finish_partials(a.S, a.slot_w + 1, sh);
      if (threadIdx.x == 0) {
        if (a.dot_w) a.S->scalars[a.slot_w] = tw;
        if (a.dot_self) a.S->scalars[a.slot_w + 1] = ts;
        a.S->tickets[a.slot_w] = 0;
        control_step(a.S, a.ctl);
      }
    }
  }
}

// The advection fields of an XF_OP_ADVDIFF operator in a stencil grid.
template <typename T>
static void set_ad_fields(StencilGrid<T>& s, const xf_op* op) {
  constexpr bool D64 = std::is_same<T, double>::value;
  s.adv0 = D64 ? (const T*)op->adv64[0] : (const T*)op->adv32[0];
  s.adv1 = D64 ? (const T*)op->adv64[1] : (const T*)op->adv32[1];
  s.adv2 = D64 ? (const T*)op->adv64[2] : (const T*)op->adv32[2];
  s.ad_itau = (T)(1 / op->ad_tau);
  s.ad_D = (T)op->ad_D;
  s.adDf = !op->adD_set ? nullptr : D64 ? (const T*)op->adD64 : (const T*)op->adD32;
  s.ad_conv = (op->ad_flags & XF_ADV_CONVECTIVE) ? T(1) : T(0);
  s.ad_diff = (op->ad_flags & XF_ADV_DIFFUSIVE) ? T(1) : T(0);
  s.ad_upwind = (op->ad_flags & XF_ADV_UPWIND) ? 1 : 0;
  s.adc = (D64 && op->adc_valid) ? (const T*)op->adc64 : nullptr;
  s.adc_n = op->g->ncell;
}

// Per-axis factors of the fast coefficients, 5 per node m of each axis (the
// halves folded in): 0.5/hx2, 0.5/h, 0.5 h/hxhxh, 0.5 hx2/hxhxh, 0.5 h_1/hxhxh
// with h_1 = h[m-1], h = h[m], hx2 = h_1 + h, hxhxh = h_1 h hx2 / 2 (the exact
// rows' quantities; nodes 0 and n-1, which carry no Actual row, get 0).
__global__ void k_ad_axis(const double* __restrict__ h, int n, double* __restrict__ t) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    double r2 = 0, rh = 0, dA = 0, dB = 0, dC = 0;
    if (m >= 1 && m <= n - 2) {
      const double h_1 = h[m - 1], hh = h[m], hx2 = h_1 + hh, hxhxh = h_1 * hh * hx2 / 2;
      r2 = 0.5 / hx2;
      rh = 0.5 / hh;
      dA = 0.5 * hh / hxhxh;
      dB = 0.5 * hx2 / hxhxh;
      dC = 0.5 * h_1 / hxhxh;
    }
    t[5 * m] = r2; t[5 * m + 1] = rh; t[5 * m + 2] = dA; t[5 * m + 3] = dB; t[5 * m + 4] = dC;
  }
}

// A, B, C of one direction from the axis factors (central or upwind), as the
// exact rows define them but with products for the divisions.
__device__ __forceinline__ void ad_coef_fast(const double* __restrict__ t, double vd, double D, double conv,
                                             double diff, bool upwind, double& A, double& B, double& C) {
  const double dA = diff * (-D * t[2]), dB = diff * (D * t[3]), dC = diff * (-D * t[4]);
  if (!upwind) {
    A = conv * (-vd * t[0]) + dA;
    B = dB;
    C = conv * (vd * t[0]) + dC;
  } else if (vd < 0) {
    A = dA;
    B = conv * (-vd * t[1]) + dB;
    C = conv * (vd * t[1]) + dC;
  } else {
    A = conv * (-vd * t[1]) + dA;
    B = conv * (vd * t[1]) + dB;
    C = dC;
  }
}

// The border rows in the same seven-coefficient form (centre, x-, x+, y-,
// y+, z-, z+): a semi-sum row takes 1/2 of itself and of its neighbour
// against the normal (the last nonzero normal component decides, as the row
// does); a normal-difference row with an axis-aligned normal is
// n_a (f_c - f_{c-1}) / h (normal +) or n_a (f_{c+1} - f_c) / h (normal -),
// its 4-point face averages collapsing to single cells.  A normal-difference
// row with an oblique normal reaches beyond the seven points: NaN in the
// centre sends it to the general row.
__device__ void ad_border_coeffs(const StencilGrid<double>& g, int64_t c, int row, double q[7]) {
  for (int t = 0; t < 7; t++) q[t] = 0.0;
  const int b = g.brow_of[c];
  const double nrm[3] = {g.brow_nrm[3 * b], g.brow_nrm[3 * b + 1], g.brow_nrm[3 * b + 2]};
  if (row == ROW_PREDEF) {
    int ax = -1;
    for (int a = 0; a < 3; a++)
      if (nrm[a] != 0) ax = a;
    if (ax < 0) return;   // no normal: the row is 0
    q[0] = 0.5;
    q[1 + 2 * ax + (nrm[ax] > 0 ? 0 : 1)] = 0.5;
    return;
  }
  int ax = -1, cnt = 0;
  for (int a = 0; a < 3; a++)
    if (nrm[a] != 0) { ax = a; cnt++; }
  if (cnt == 0) return;   // the row is 0
  if (cnt > 1) { q[0] = __longlong_as_double(0x7ff8000000000000ll); return; }
  const int i = (int)(c / g.s1), j = (int)((c - (int64_t)i * g.s1) / g.s2), k = (int)(c % g.s2);
  const int m = ax == 0 ? i : ax == 1 ? j : k;
  const double* h = ax == 0 ? g.hx : ax == 1 ? g.hy : g.hz;
  const double na = nrm[ax];
  if (na > 0) {
    const double r = na / h[m - 1];
    q[0] = r;
    q[1 + 2 * ax] = -r;
  } else {
    const double r = na / h[m];
    q[0] = -r;
    q[2 + 2 * ax] = r;
  }
}

// The FP64 coefficient table of the fast rows: for Actual rows a centre
// coefficient 1/tau + B_x + B_y + B_z and the six neighbour coefficients;
// border rows as ad_border_coeffs.
__global__ void k_ad_coeffs(StencilGrid<double> g, int64_t n, const double* __restrict__ tx,
                            const double* __restrict__ ty, const double* __restrict__ tz, double* __restrict__ out) {
  const bool up = g.ad_upwind != 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int row = row_of(g.kind[c]);
    if (row == ROW_NONE) continue;
    if (row != ROW_ACTUAL) {
      double q[7];
      ad_border_coeffs(g, c, row, q);
      for (int t = 0; t < 7; t++) out[t * n + c] = q[t];
      continue;
    }
    const int i = (int)(c / g.s1), j = (int)((c - (int64_t)i * g.s1) / g.s2), k = (int)(c % g.s2);
    const double D = g.adDf ? g.adDf[c] : g.ad_D;
    double Ax, Bx, Cx, Ay, By, Cy, Az, Bz, Cz;
    ad_coef_fast(tx + 5 * i, g.adv0[c], D, g.ad_conv, g.ad_diff, up, Ax, Bx, Cx);
    ad_coef_fast(ty + 5 * j, g.adv1[c], D, g.ad_conv, g.ad_diff, up, Ay, By, Cy);
    ad_coef_fast(tz + 5 * k, g.adv2[c], D, g.ad_conv, g.ad_diff, up, Az, Bz, Cz);
    out[c] = g.ad_itau + Bx + By + Bz;
    out[n + c] = Ax;
    out[2 * n + c] = Cx;
    out[3 * n + c] = Ay;
    out[4 * n + c] = Cy;
    out[5 * n + c] = Az;
    out[6 * n + c] = Cz;
  }
}

// The fast FP64 advection-diffusion apply as a flat grid-stride kernel: a
// thread takes cell after cell (the row reads its seven coefficients and its
// neighbours directly, so the plane march buys nothing), at full occupancy.
// Border rows read the table too (their semi-sums and axis-aligned normal
// differences are seven-point rows), so a warp that holds a face cell does
// not wait on the general border row; only oblique normal differences take
// it.  Same dots and control step as k_matvec.
constexpr int AD_THREADS = 256;
// The border rows, out of line: they are few, and inlined they would set the
// register budget of the whole loop.
__device__ __noinline__ double ad_border_row(const StencilGrid<double>& g, const double* __restrict__ x, int64_t c,
                                             int row) {
  const int64_t s1 = g.s1, s2 = g.s2;
  const int i = (int)(c / s1), j = (int)((c - (int64_t)i * s1) / s2), k = (int)(c % s2);
  return boundary_row<double, false>(g, x, i, j, k, (int)c, row);
}

__global__ void __launch_bounds__(AD_THREADS, 4) k_ad_fast(MatvecArgs<double> a) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (a.ctl != CTL_NONE && (a.S->iscalars[I_DONE] || (a.gate && !a.S->iscalars[I_NEEDREP]))) return;
  const StencilGrid<double>& g = a.g;
  const int64_t s1 = g.s1, s2 = g.s2, n = (int64_t)g.n1 * s1, nn = g.adc_n;
  const double* __restrict__ x = a.x;
  DotAcc<double> dw, ds;
  for (int64_t c = blockIdx.x * (int64_t)AD_THREADS + threadIdx.x; c < n; c += (int64_t)gridDim.x * AD_THREADS) {
    const int row = row_of(g.kind[c]);
    if (row == ROW_NONE) {
      if (a.zero_inactive) {
        if (a.y) a.y[c] = 0.0;
        if (a.y32) a.y32[c] = 0.f;
      }
      continue;
    }
    double v;
    const double* __restrict__ q = g.adc + c;
    const double q0 = q[0];
    if (row == ROW_ACTUAL) {   // interior: all six neighbours are inside the box
      v = q0 * x[c];
      v = fma(q[nn], x[c - s1], v);
      v = fma(q[2 * nn], x[c + s1], v);
      v = fma(q[3 * nn], x[c - s2], v);
      v = fma(q[4 * nn], x[c + s2], v);
      v = fma(q[5 * nn], x[c - 1], v);
      v = fma(q[6 * nn], x[c + 1], v);
    } else if (q0 == q0) {   // a border row from the table: it reads only its nonzero neighbours
      const int64_t off[6] = {-s1, s1, -s2, s2, -1, 1};
      v = q0 * x[c];
#pragma unroll
      for (int t = 0; t < 6; t++) {
        const double qt = q[(t + 1) * nn];
        if (qt != 0) v = fma(qt, x[c + off[t]], v);
      }
    } else {   // an oblique normal difference
      v = ad_border_row(g, x, c, row);
    }
    if (a.sign > 0) v = v + a.s[c];
    else if (a.sign < 0) v = v - a.s[c];
    if (a.neg) v = -v;
    if (a.dot_w) dw.add(a.w[c], v);
    if (a.dot_self) ds.add(v, v);
    if (a.y) a.y[c] = v;
    if (a.y32) a.y32[c] = (float)v;
  }
  if (a.dot_w || a.dot_self || a.ctl != CTL_NONE) {
    double vals[2] = {dw.value(), ds.value()};
    if (publish_partials<2>(a.S, a.slot_w, vals, sh, &last)) {
      double tw = finish_partials(a.S, a.slot_w, sh);
      double ts = finish_partials(a.S, a.slot_w + 1, sh);
      if (threadIdx.x == 0) {
        if (a.dot_w) a.S->scalars[a.slot_w] = tw;
        if (a.dot_self) a.S->scalars[a.slot_w + 1] = ts;
        a.S->tickets[a.slot_w] = 0;
        control_step(a.S, a.ctl);
      }
    }
  }
}

// A unit probe at the row's own cell: a border row evaluated on it is the
// row's diagonal coefficient.
struct UnitProbe {
  __device__ __forceinline__ double operator()(int a, int b, int d) const { return (a | b | d) == 0 ? 1.0 : 0.0; }
};

// Inverse row diagonals of the fast rows (Actual: the table's centre; border
// rows: the row on a unit probe), 0 off the active set and where a diagonal
// is 0.
__global__ void k_ad_jacobi(StencilGrid<double> g, int64_t n, const double* __restrict__ table,
                            double* __restrict__ dinv) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int row = row_of(g.kind[c]);
    double d = 0;
    if (row == ROW_ACTUAL) {
      d = table[c];
    } else if (row != ROW_NONE) {
      const int i = (int)(c / g.s1), j = (int)((c - (int64_t)i * g.s1) / g.s2), k = (int)(c % g.s2);
      d = boundary_row_acc<double, false>(g, UnitProbe{}, i, j, k, (int)c, row);
    }
    dinv[c] = d != 0 ? 1.0 / d : 0.0;
  }
}

// The Laplace operator's inverse row diagonals (Actual: the fast row's
// diagonal; border rows: the row on a unit probe), 0 off the active set.
__global__ void k_lap_jacobi(StencilGrid<double> g, int64_t n, const double* __restrict__ diag,
                             double* __restrict__ dinv) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int row = row_of(g.kind[c]);
    double d = 0;
    if (row == ROW_ACTUAL) {
      d = diag[c];
    } else if (row != ROW_NONE) {
      const int i = (int)(c / g.s1), j = (int)((c - (int64_t)i * g.s1) / g.s2), k = (int)(c % g.s2);
      d = boundary_row_acc<double, false>(g, UnitProbe{}, i, j, k, (int)c, row);
    }
    dinv[c] = d != 0 ? 1.0 / d : 0.0;
  }
}

// The inverse row diagonals of a Laplace or advection-diffusion operator
// (the latter refreshed by xf_op_ready), for Jacobi-preconditioned BiCGStab.
int xf_op_jacobi(const xf_op* op, const double** dinv) {
  xf_ctx* ctx = op->g->ctx;
  if (op->kind == XF_OP_ADVDIFF && op->adc_valid && op->adj64) {
    *dinv = op->adj64;
    return XF_OK;
  }
  if (op->kind != XF_OP_LAPLACE)
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: Jacobi BiCGStab takes a Laplace or advection-diffusion operator");
  const int64_t n = op->g->ncell;
  if (!op->lap_jac_valid) {
    if (!op->adj64 && cudaMalloc(&op->adj64, n * 8) != cudaSuccess) {
      cudaGetLastError();
      return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    }
    StencilGrid<double> s = make_stencil_grid<double>(op->g, nullptr);
    k_lap_jacobi<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(s, n, op->g->diag, op->adj64);
    XF_CUDA(ctx, cudaGetLastError());
    op->lap_jac_valid = 1;
  }
  *dinv = op->adj64;
  return XF_OK;
}

template <typename T>
static void launch_matvec(const xf_op* op, const T* rho, const MvReq<T>& q) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  MatvecArgs<T> a;
  a.g = make_stencil_grid<T>(g, rho);
  a.x = q.x; a.y = q.y; a.y32 = q.y32; a.s = q.s; a.w = q.w; a.diag = g->diag;
  a.sign = q.sign; a.neg = q.neg; a.zero_inactive = q.zero_inactive;
  a.dot_w = q.w != nullptr; a.dot_self = q.dot_self;
  a.slot_w = q.slot; a.ctl = q.ctl; a.gate = q.gate;
  a.S = ctx->scratch;
  const int P = g->n2 * g->n3;
  const int bx = (P + MV_THREADS - 1) / MV_THREADS;
  // plane chunk: ~16 planes per block, fewer chunks if the partial-sum table
  // would overflow
  int chunk = 16;
  while ((int64_t)bx * ((g->n1 + chunk - 1) / chunk) > RED_MAX_BLOCKS) chunk *= 2;
  a.chunk = chunk;
  dim3 grid(bx, (g->n1 + chunk - 1) / chunk);
  const bool use_d = std::is_same<T, double>::value && op->kind == XF_OP_LAPLACE && !q.exact;
  if (op->kind == XF_OP_ADVDIFF) {
    set_ad_fields<T>(a.g, op);
    if constexpr (std::is_same<T, double>::value) {
      if (!q.exact && a.g.adc) {
        k_ad_fast<<<grid_blocks(ctx, g->ncell, AD_THREADS), AD_THREADS, 0, ctx->stream>>>(a);
        return;
      }
    }
    if (q.exact) k_matvec<T, XF_OP_ADVDIFF, true, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
    else k_matvec<T, XF_OP_ADVDIFF, false, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
    return;
  }
  if (op->kind == XF_OP_LAPLACE) {
    if (q.exact) k_matvec<T, XF_OP_LAPLACE, true, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
    else if (use_d) k_matvec<T, XF_OP_LAPLACE, false, true><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
    else k_matvec<T, XF_OP_LAPLACE, false, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
  } else {
    if (q.exact) k_matvec<T, XF_OP_VARDIV, true, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
    else k_matvec<T, XF_OP_VARDIV, false, false><<<grid, MV_THREADS, 0, ctx->stream>>>(a);
  }
}

void xf_pack_mv64(const xf_op* op, const MvReq<double>& q);
void xf_pack_free(PackData* P);

void xf_mv64(const xf_op* op, const MvReq<double>& q) {
  if (op->kind == XF_OP_PACK) xf_pack_mv64(op, q);
  else launch_matvec<double>(op, op->rho, q);
}
// (packed operators are FP64 only: the callers refuse FP32 with them)
void xf_mv32(const xf_op* op, const MvReq<float>& q) { launch_matvec<float>(op, op->rho32, q); }

// Used by the C-ABI helpers: plain apply with an optional dot into slot.
void xf_apply_f64(const xf_op* op, const double* x, double* y, const double* s, int sign, bool exact,
                  bool zero_inactive, const double* w, int slot) {
  MvReq<double> q;
  q.x = x; q.y = y; q.s = s; q.sign = sign; q.exact = exact; q.zero_inactive = zero_inactive; q.w = w; q.slot = slot;
  xf_mv64(op, q);
}
void xf_apply_f32(const xf_op* op, const float* x, float* y, const float* s, int sign, bool zero_inactive,
                  const float* w, int slot) {
  MvReq<float> q;
  q.x = x; q.y = y; q.s = s; q.sign = sign; q.zero_inactive = zero_inactive; q.w = w; q.slot = slot;
  xf_mv32(op, q);
}

// ---------------------------------------------------------------------------
extern "C" int xf_op_create(xf_grid* g, int kind, xf_op** out) {
  if (!g || !out || (kind != XF_OP_LAPLACE && kind != XF_OP_VARDIV && kind != XF_OP_ADVDIFF))
    return xf_fail(g ? g->ctx : nullptr, XF_ERR_ARG, "xf_op_create: bad arguments");
  *out = nullptr;
  int64_t bad = -1;
  int st = xf_grid_check(g, kind, &bad);
  if (st != XF_OK) {
    const int i = (int)(bad / g->s1), j = (int)((bad / g->s2) % g->n2), k = (int)(bad % g->n3);
    return xf_fail(g->ctx, XF_ERR_MASK,
                   "operator %d is not defined at cell (%d,%d,%d): the reference throws or reads outside its arrays there",
                   kind, i, j, k);
  }
  static std::atomic<unsigned long long> serials{0};
  xf_op* op = new xf_op();
  op->g = g; op->kind = kind; op->rho = nullptr; op->rho32 = nullptr; op->rho_set = 0;
  op->serial = ++serials;
  if (kind == XF_OP_VARDIV) {
    xf_ctx* ctx = g->ctx;
    if (cudaMalloc(&op->rho, g->ncell * 8) != cudaSuccess || cudaMalloc(&op->rho32, g->ncell * 4) != cudaSuccess) {
      cudaGetLastError();
      xf_op_destroy(op);
      return xf_fail(ctx, XF_ERR_NOMEM, "xf_op_create: density allocation failed");
    }
    // The reference dereferences a null density until withDensity is called
    // (XOperator.h:422); here the operator refuses to apply until it is set.
    cudaMemsetAsync(op->rho, 0, g->ncell * 8, ctx->stream);
    cudaMemsetAsync(op->rho32, 0, g->ncell * 4, ctx->stream);
  }
  *out = op;
  return XF_OK;
}

extern "C" int xf_op_destroy(xf_op* op) {
  if (!op) return XF_ERR_ARG;
  cudaSetDevice(op->g->ctx->device);
  cudaStreamSynchronize(op->g->ctx->stream);
  if (op->rho) cudaFree(op->rho);
  if (op->rho32) cudaFree(op->rho32);
  for (int d = 0; d < 3; d++) {
    if (op->adv64[d]) cudaFree(op->adv64[d]);
    if (op->adv32[d]) cudaFree(op->adv32[d]);
  }
  if (op->adD64) cudaFree(op->adD64);
  if (op->adD32) cudaFree(op->adD32);
  if (op->adc64) cudaFree(op->adc64);
  if (op->adj64) cudaFree(op->adj64);
  if (op->pack) xf_pack_free(op->pack);
  if (op->host_x) xf_vec_destroy(op->host_x);
  if (op->host_b) xf_vec_destroy(op->host_b);
  delete op;
  return XF_OK;
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) b[c] = (float)a[c];
}

extern "C" int xf_op_set_density(xf_op* op, const double* host_rho) {
  if (!op || !host_rho) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  if (op->kind != XF_OP_VARDIV) return xf_fail(ctx, XF_ERR_STATE, "xf_op_set_density: not a variable-density operator");
  const int64_t n = op->g->ncell;
  XF_CUDA(ctx, cudaMemcpyAsync(op->rho, host_rho, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  k_d2f<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(op->rho, op->rho32, n);
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  op->rho_set = 1;
  return XF_OK;
}

extern "C" int xf_op_set_advection(xf_op* op, const xf_vec* u, const xf_vec* v, const xf_vec* w, double tau,
                                   double diff_coef, int flags) {
  if (!op) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  if (op->kind != XF_OP_ADVDIFF) return xf_fail(ctx, XF_ERR_STATE, "xf_op_set_advection: not an advection-diffusion operator");
  if (!(tau != 0) || (flags & ~(XF_ADV_CONVECTIVE | XF_ADV_DIFFUSIVE | XF_ADV_UPWIND)))
    return xf_fail(ctx, XF_ERR_ARG, "xf_op_set_advection: tau must be nonzero and flags XF_ADV_*");
  const xf_vec* vel[3] = {u, v, w};
  for (int d = 0; d < 3; d++)
    if (vel[d] && (vel[d]->g != op->g || vel[d]->dtype != XF_F64))
      return xf_fail(ctx, XF_ERR_STATE, "xf_op_set_advection: velocities must be FP64 boxes of the operator's grid");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t n = op->g->ncell;
  op->adc_valid = 0;
  const int64_t nax = 5 * ((int64_t)op->g->n1 + op->g->n2 + op->g->n3);   // per-axis factors after the table
  if ((!op->adc64 && cudaMalloc(&op->adc64, (7 * n + nax) * 8) != cudaSuccess) ||
      (!op->adj64 && cudaMalloc(&op->adj64, n * 8) != cudaSuccess)) {
    cudaGetLastError();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_op_set_advection: allocation");
  }
  for (int d = 0; d < 3; d++) {
    if (!op->adv64[d] && (cudaMalloc(&op->adv64[d], n * 8) != cudaSuccess ||
                          cudaMalloc(&op->adv32[d], n * 4) != cudaSuccess)) {
      cudaGetLastError();
      return xf_fail(ctx, XF_ERR_NOMEM, "xf_op_set_advection: allocation");
    }
    if (vel[d]) XF_CUDA(ctx, cudaMemcpyAsync(op->adv64[d], vel[d]->data, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    else XF_CUDA(ctx, cudaMemsetAsync(op->adv64[d], 0, n * 8, ctx->stream));
    k_d2f<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(op->adv64[d], op->adv32[d], n);
  }
  XF_CUDA(ctx, cudaGetLastError());
  op->ad_tau = tau;
  op->ad_D = diff_coef;
  op->ad_flags = flags;
  op->adv_set = 1;
  return XF_OK;
}

extern "C" int xf_op_set_diffusion_field(xf_op* op, const xf_vec* d) {
  if (!op) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  if (op->kind != XF_OP_ADVDIFF)
    return xf_fail(ctx, XF_ERR_STATE, "xf_op_set_diffusion_field: not an advection-diffusion operator");
  op->adc_valid = 0;
  if (!d) {
    op->adD_set = 0;
    return XF_OK;
  }
  if (d->g != op->g || d->dtype != XF_F64)
    return xf_fail(ctx, XF_ERR_STATE, "xf_op_set_diffusion_field: an FP64 box of the operator's grid expected");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t n = op->g->ncell;
  if (!op->adD64 && (cudaMalloc(&op->adD64, n * 8) != cudaSuccess || cudaMalloc(&op->adD32, n * 4) != cudaSuccess)) {
    cudaGetLastError();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_op_set_diffusion_field: allocation");
  }
  XF_CUDA(ctx, cudaMemcpyAsync(op->adD64, d->data, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  k_d2f<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(op->adD64, op->adD32, n);
  XF_CUDA(ctx, cudaGetLastError());
  op->adD_set = 1;
  return XF_OK;
}

int xf_op_ready(const xf_op* op) {
  if (op->kind == XF_OP_ADVDIFF && !op->adv_set)
    return xf_fail(op->g->ctx, XF_ERR_STATE, "advection-diffusion operator used before xf_op_set_advection");
  if (op->kind == XF_OP_ADVDIFF && !op->adc_valid && op->adc64) {   // refresh the coefficient table
    xf_ctx* ctx = op->g->ctx;
    XF_CUDA(ctx, cudaSetDevice(ctx->device));
    const xf_grid* g = op->g;
    StencilGrid<double> s = make_stencil_grid<double>(g, nullptr);
    op->adc_valid = 0;
    set_ad_fields<double>(s, op);
    const int64_t n = g->ncell;
    double* tx = op->adc64 + 7 * n;   // the axis factors sit after the table
    double* ty = tx + 5 * g->n1;
    double* tz = ty + 5 * g->n2;
    k_ad_axis<<<1, 256, 0, ctx->stream>>>(g->hx, g->n1, tx);
    k_ad_axis<<<1, 256, 0, ctx->stream>>>(g->hy, g->n2, ty);
    k_ad_axis<<<1, 256, 0, ctx->stream>>>(g->hz, g->n3, tz);
    k_ad_coeffs<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(s, n, tx, ty, tz, op->adc64);
    k_ad_jacobi<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(s, n, op->adc64, op->adj64);
    XF_CUDA(ctx, cudaGetLastError());
    op->adc_valid = 1;
  }
  if (op->kind == XF_OP_VARDIV && !op->rho_set)
    return xf_fail(op->g->ctx, XF_ERR_STATE, "variable-density operator used before xf_op_set_density");
  return XF_OK;
}

static int check_vec(const xf_op* op, const xf_vec* v, const char* what) {
  if (!v) return xf_fail(op->g->ctx, XF_ERR_ARG, "%s: null vector", what);
  if (v->g != op->g) return xf_fail(op->g->ctx, XF_ERR_STATE, "%s: vector of another grid", what);
  return XF_OK;
}

extern "C" int xf_matvec(xf_op* op, const xf_vec* x, xf_vec* y, const xf_vec* s, int sign, int flags,
                         const xf_vec* opt_w, double* opt_dot) {
  if (!op) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  int st;
  if ((st = check_vec(op, x, "xf_matvec x")) || (st = check_vec(op, y, "xf_matvec y"))) return st;
  if (sign != 0 && (st = check_vec(op, s, "xf_matvec s"))) return st;
  if (x == y) return xf_fail(ctx, XF_ERR_ARG, "xf_matvec: x and y must differ");
  if ((st = xf_op_ready(op))) return st;
  if (x->dtype != y->dtype || (sign != 0 && s->dtype != x->dtype))
    return xf_fail(ctx, XF_ERR_STATE, "xf_matvec: mixed dtypes");
  const bool exact = (flags & XF_EXACT) != 0;
  if (exact && x->dtype != XF_F64) return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_matvec: XF_EXACT needs FP64 vectors");
  if (op->kind == XF_OP_PACK && x->dtype != XF_F64)
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_matvec: packed operators are FP64");
  const xf_vec* w = opt_dot ? (opt_w ? opt_w : x) : nullptr;
  if (w && (st = check_vec(op, w, "xf_matvec w"))) return st;
  if (w && w->dtype != x->dtype) return xf_fail(ctx, XF_ERR_STATE, "xf_matvec: dot partner dtype");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int slot = 0;
  if (x->dtype == XF_F64)
    xf_apply_f64(op, (const double*)x->data, (double*)y->data, s ? (const double*)s->data : nullptr, sign, exact,
                 (flags & XF_ZERO_INACTIVE) != 0, w ? (const double*)w->data : nullptr, slot);
  else
    xf_apply_f32(op, (const float*)x->data, (float*)y->data, s ? (const float*)s->data : nullptr, sign,
                 (flags & XF_ZERO_INACTIVE) != 0, w ? (const float*)w->data : nullptr, slot);
  XF_CUDA(ctx, cudaGetLastError());
  if (opt_dot) {
    XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->scalars[slot], 8, cudaMemcpyDeviceToHost, ctx->stream));
    XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *opt_dot = ctx->host_scalars[0];
  }
  return XF_OK;
}
