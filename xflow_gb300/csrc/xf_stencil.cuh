// Device-side row evaluation of the reference operators.
//
//  * exact_*  : the reference's own expressions and operation order
//               (T3dLaplaceOperator::operator(), XOperator.cpp:938-1129;
//               T3dVariableDivergentedOperator::operator(), :1901-2233).
//               With --fmad=false these are bit-identical to the CPU in FP64.
//  * fast_*   : the same rows with the divisions folded into per-index
//               coefficients (c?p = 1/(h[i]*hh), c?m = 1/(h[i-1]*hh),
//               hh = (h[i-1]+h[i])/2), used on the solver hot path.
#pragma once
#include "xf_common.cuh"

template <typename T>
struct StencilGrid {
  const uint8_t* __restrict__ kind;
  const int32_t* __restrict__ brow_of;
  const double* __restrict__ brow_nrm;
  const T* __restrict__ hx;   // separations (exact / boundary rows)
  const T* __restrict__ hy;
  const T* __restrict__ hz;
  const T* __restrict__ cxm; const T* __restrict__ cxp;
  const T* __restrict__ cym; const T* __restrict__ cyp;
  const T* __restrict__ czm; const T* __restrict__ czp;
  const T* __restrict__ rhx; const T* __restrict__ rhy; const T* __restrict__ rhz;
  const T* __restrict__ rhhx; const T* __restrict__ rhhy; const T* __restrict__ rhhz;
  const T* __restrict__ rho;  // density box (VARDIV) or null
  // ADVDIFF: advecting velocity per direction, 1/tau, D and the two flags as 0/1
  const T* __restrict__ adv0; const T* __restrict__ adv1; const T* __restrict__ adv2;
  const T* __restrict__ adDf;   // per-cell D of the variable-viscosity form, or null
  // the Actual rows' seven coefficients of the fast form (centre, then the
  // x-, x+, y-, y+, z-, z+ neighbours; SoA with stride adc_n), precomputed
  // from the fields above, or null
  const T* __restrict__ adc;
  int64_t adc_n;
  T ad_itau, ad_D, ad_conv, ad_diff;
  int ad_upwind;   // the first-order upwind form of the convective term
  int n1, n2, n3;
  int s1, s2;
};

// Laplace Actual row, reference order (XOperator.cpp:971-1019).
template <typename T>
__device__ __forceinline__ T exact_lap_actual(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k,
                                              int c, uint8_t kb) {
  const int s1 = g.s1, s2 = g.s2;
  T hx_2X = (g.hx[i - 1] + g.hx[i]) / T(2);
  T hx_2Y = (g.hy[j - 1] + g.hy[j]) / T(2);
  T hx_2Z = (g.hz[k - 1] + g.hz[k]) / T(2);
  T fc = f[c];
  T f_i_1 = (fc - f[c - s1]) / (g.hx[i - 1]);
  T f_i = (f[c + s1] - fc) / (g.hx[i]);
  T f_j_1 = (fc - f[c - s2]) / (g.hy[j - 1]);
  T f_j = (f[c + s2] - fc) / (g.hy[j]);
  T f_k_1 = (fc - f[c - 1]) / (g.hz[k - 1]);
  T f_k = (f[c + 1] - fc) / (g.hz[k]);
  if (!(kb & K_MX)) f_i_1 = 0;
  if (!(kb & K_PX)) f_i = 0;
  if (!(kb & K_MY)) f_j_1 = 0;
  if (!(kb & K_PY)) f_j = 0;
  if (!(kb & K_MZ)) f_k_1 = 0;
  if (!(kb & K_PZ)) f_k = 0;
  return -((f_i - f_i_1) / hx_2X + (f_j - f_j_1) / hx_2Y + (f_k - f_k_1) / hx_2Z);
}

// Variable-density Actual row, reference order (XOperator.cpp:1933-2025).
template <typename T>
__device__ __forceinline__ T exact_vd_actual(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k,
                                             int c, uint8_t kb) {
  const int s1 = g.s1, s2 = g.s2;
  const T* __restrict__ rho = g.rho;
  T h_1X = g.hx[i - 1], hX = g.hx[i];
  T h_1Y = g.hy[j - 1], hY = g.hy[j];
  T h_1Z = g.hz[k - 1], hZ = g.hz[k];
  T hx_2X = (g.hx[i - 1] + g.hx[i]) / T(2);
  T hx_2Y = (g.hy[j - 1] + g.hy[j]) / T(2);
  T hx_2Z = (g.hz[k - 1] + g.hz[k]) / T(2);
  T fc = f[c], rc = rho[c];
  T f_i_1 = rho[c - s1] * (fc - f[c - s1]) / (h_1X);
  T f_i = rho[c + s1] * (f[c + s1] - fc) / (hX);
  T f_j_1 = rho[c - s2] * (fc - f[c - s2]) / (h_1Y);
  T f_j = rho[c + s2] * (f[c + s2] - fc) / (hY);
  T f_k_1 = rho[c - 1] * (fc - f[c - 1]) / (h_1Z);
  T f_k = rho[c + 1] * (f[c + 1] - fc) / (hZ);
  T d_i = (rho[c + s1] - rc) / (h_1X);
  T d_j = (rho[c + s2] - rc) / (h_1Y);
  T d_k = (rho[c + 1] - rc) / (h_1Z);
  if (!(kb & K_MX)) f_i_1 = 0;
  if (!(kb & K_PX)) { f_i = 0; d_i = 0; }
  if (!(kb & K_MY)) f_j_1 = 0;
  if (!(kb & K_PY)) { f_j = 0; d_j = 0; }
  if (!(kb & K_MZ)) f_k_1 = 0;
  if (!(kb & K_PZ)) { f_k = 0; d_k = 0; }
  T laplace_p = ((f_i - f_i_1) / hx_2X + (f_j - f_j_1) / hx_2Y + (f_k - f_k_1) / hx_2Z);
  T divergence_density = d_i + d_j + d_k;
  return -(rc * laplace_p - divergence_density * fc);
}

// PreDefined (semi-sum, XOperator.cpp:1034-1069) and PreNormal
// (XOperator.cpp:1070-1119; variable-density tail :2210-2221) rows.  `F`
// returns the argument at offset (di, dj, dk) from the row's cell, so the same
// formulas serve global-memory and shared-memory-staged callers.
template <typename T, bool VARDIV, class F>
__device__ __forceinline__ T boundary_row_acc(const StencilGrid<T>& g, const F& FF, int i, int j, int k, int c,
                                              int row) {
  const int s1 = g.s1, s2 = g.s2;
  const int b = g.brow_of[c];
  const double nxd = g.brow_nrm[3 * b], nyd = g.brow_nrm[3 * b + 1], nzd = g.brow_nrm[3 * b + 2];
  if (row == ROW_PREDEF) {
    T semiSum = 0;
    if (nxd > 0) semiSum = (FF(0, 0, 0) + FF(-1, 0, 0)) / T(2);
    else if (nxd < 0) semiSum = (FF(1, 0, 0) + FF(0, 0, 0)) / T(2);
    if (nyd > 0) semiSum = (FF(0, 0, 0) + FF(0, -1, 0)) / T(2);
    else if (nyd < 0) semiSum = (FF(0, 1, 0) + FF(0, 0, 0)) / T(2);
    if (nzd > 0) semiSum = (FF(0, 0, 0) + FF(0, 0, -1)) / T(2);
    else if (nzd < 0) semiSum = (FF(0, 0, 1) + FF(0, 0, 0)) / T(2);
    return semiSum;
  }
  const T nx = (T)nxd, ny = (T)nyd, nz = (T)nzd;
  int sI = 0, sI1 = 0, sJ = 0, sJ1 = 0, sK = 0, sK1 = 0;
  T hxl = 1, hyl = 1, hzl = 1;
  if (nxd > 0) { sI = 0; sI1 = -1; hxl = g.hx[i - 1]; } else if (nxd < 0) { sI = 1; sI1 = 0; hxl = g.hx[i]; }
  if (nyd > 0) { sJ = 0; sJ1 = -1; hyl = g.hy[j - 1]; } else if (nyd < 0) { sJ = 1; sJ1 = 0; hyl = g.hy[j]; }
  if (nzd > 0) { sK = 0; sK1 = -1; hzl = g.hz[k - 1]; } else if (nzd < 0) { sK = 1; sK1 = 0; hzl = g.hz[k]; }
  T fl = (FF(sI, 0, 0) + FF(sI, sJ, 0) + FF(sI, 0, sK) + FF(sI, sJ, sK)) / T(4);
  T fl_1 = (FF(sI1, 0, 0) + FF(sI1, sJ, 0) + FF(sI1, 0, sK) + FF(sI1, sJ, sK)) / T(4);
  T dfx = (fl - fl_1) / hxl;
  fl = (FF(0, sJ, 0) + FF(sI, sJ, 0) + FF(0, sJ, sK) + FF(sI, sJ, sK)) / T(4);
  fl_1 = (FF(0, sJ1, 0) + FF(sI, sJ1, 0) + FF(0, sJ1, sK) + FF(sI, sJ1, sK)) / T(4);
  T dfy = (fl - fl_1) / hyl;
  fl = (FF(0, 0, sK) + FF(sI, 0, sK) + FF(0, sJ, sK) + FF(sI, sJ, sK)) / T(4);
  fl_1 = (FF(0, 0, sK1) + FF(sI, 0, sK1) + FF(0, sJ, sK1) + FF(sI, sJ, sK1)) / T(4);
  T dfz = (fl - fl_1) / hzl;
  if (!VARDIV) return dfx * nx + dfy * ny + dfz * nz;
  const T* __restrict__ rho = g.rho;
  T d_x = rho[c + s1] - rho[c] / (g.hx[i - 1]);
  T d_y = rho[c + s2] - rho[c] / (g.hy[j - 1]);
  T d_z = rho[c + 1] - rho[c] / (g.hz[k - 1]);
  T laplace_p = dfx * nx + dfy * ny + dfz * nz;
  T divergence_density = d_x + d_y + d_z;
  return rho[c] * laplace_p - divergence_density * FF(0, 0, 0);
}

template <typename T>
struct GlobalAcc {
  const T* __restrict__ f;
  int c, s1, s2;
  __device__ __forceinline__ T operator()(int a, int b, int d) const { return f[c + a * s1 + b * s2 + d]; }
};

template <typename T, bool VARDIV>
__device__ __forceinline__ T boundary_row(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k,
                                          int c, int row) {
  GlobalAcc<T> acc{f, c, g.s1, g.s2};
  return boundary_row_acc<T, VARDIV>(g, acc, i, j, k, c, row);
}

template <typename T>
__device__ __forceinline__ T sel(bool b, T v) { return b ? v : T(0); }

// Laplace Actual row, coefficient form.
template <typename T>
__device__ __forceinline__ T fast_lap_actual(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k,
                                             int c, uint8_t kb) {
  const int s1 = g.s1, s2 = g.s2;
  const T fc = f[c];
  const T tpx = sel<T>(kb & K_PX, g.cxp[i] * (f[c + s1] - fc));
  const T tmx = sel<T>(kb & K_MX, g.cxm[i] * (fc - f[c - s1]));
  const T tpy = sel<T>(kb & K_PY, g.cyp[j] * (f[c + s2] - fc));
  const T tmy = sel<T>(kb & K_MY, g.cym[j] * (fc - f[c - s2]));
  const T tpz = sel<T>(kb & K_PZ, g.czp[k] * (f[c + 1] - fc));
  const T tmz = sel<T>(kb & K_MZ, g.czm[k] * (fc - f[c - 1]));
  return -(((tpx - tmx) + (tpy - tmy)) + (tpz - tmz));
}

// Variable-density Actual row, coefficient form.
template <typename T>
__device__ __forceinline__ T fast_vd_actual(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k,
                                            int c, uint8_t kb) {
  const int s1 = g.s1, s2 = g.s2;
  const T* __restrict__ rho = g.rho;
  const T fc = f[c], rc = rho[c];
  const T rpx = rho[c + s1], rpy = rho[c + s2], rpz = rho[c + 1];
  const T f_i = sel<T>(kb & K_PX, rpx * (f[c + s1] - fc) * g.rhx[i]);
  const T f_i_1 = sel<T>(kb & K_MX, rho[c - s1] * (fc - f[c - s1]) * g.rhx[i - 1]);
  const T f_j = sel<T>(kb & K_PY, rpy * (f[c + s2] - fc) * g.rhy[j]);
  const T f_j_1 = sel<T>(kb & K_MY, rho[c - s2] * (fc - f[c - s2]) * g.rhy[j - 1]);
  const T f_k = sel<T>(kb & K_PZ, rpz * (f[c + 1] - fc) * g.rhz[k]);
  const T f_k_1 = sel<T>(kb & K_MZ, rho[c - 1] * (fc - f[c - 1]) * g.rhz[k - 1]);
  const T d_i = sel<T>(kb & K_PX, (rpx - rc) * g.rhx[i - 1]);
  const T d_j = sel<T>(kb & K_PY, (rpy - rc) * g.rhy[j - 1]);
  const T d_k = sel<T>(kb & K_PZ, (rpz - rc) * g.rhz[k - 1]);
  const T lap = (f_i - f_i_1) * g.rhhx[i] + (f_j - f_j_1) * g.rhhy[j] + (f_k - f_k_1) * g.rhhz[k];
  return -(rc * lap - (d_i + d_j + d_k) * fc);
}

// Advection-diffusion Actual row: per direction the reference's ADI line
// coefficients (XProblem.cpp:1236-1238) in its operation order, summed over
// x, y, z after (1/tau) f_c.  Neighbour values are read as they are (the
// solver keeps inactive cells at 0).
template <typename T>
__device__ __forceinline__ void ad_coef(const T* __restrict__ h, int m, T vd, T D, T conv, T diff, T& A, T& B, T& C) {
  const T h_1 = h[m - 1], hh = h[m];
  const T hx2 = h[m - 1] + h[m];
  const T hxhxh = h[m - 1] * h[m] * (h[m - 1] + h[m]) / T(2);
  A = conv * (T(0.5) * (-vd / hx2)) + diff * (T(0.5) * (-(D)*hh / hxhxh));
  B = diff * (T(0.5) * (D)*hx2 / hxhxh);
  C = conv * (T(0.5) * (vd / hx2)) + diff * (T(0.5) * (-(D)*h_1 / hxhxh));
}

// The upwind form (schemeType 1 of SolveTransferEquation_, XProblem.cpp:
// 1828-1843): the convective term takes the upstream neighbour over h[m];
// the centre coefficient is the convective term plus the diffusive one.
template <typename T>
__device__ __forceinline__ void ad_coef_upwind(const T* __restrict__ h, int m, T vd, T D, T conv, T diff, T& A, T& B,
                                               T& C) {
  const T h_1 = h[m - 1], hh = h[m];
  const T hx2 = h[m - 1] + h[m];
  const T hxhxh = h[m - 1] * h[m] * (h[m - 1] + h[m]) / T(2);
  const T Bd = diff * (T(0.5) * (D)*hx2 / hxhxh);
  T Bc;
  if (vd < T(0)) {
    A = diff * (T(0.5) * (-(D)*hh / hxhxh));
    Bc = conv * (T(0.5) * (-vd / hh));
    C = conv * (T(0.5) * (vd / hh)) + diff * (T(0.5) * (-(D)*h_1 / hxhxh));
  } else {
    A = conv * (T(0.5) * (-vd / hh)) + diff * (T(0.5) * (-(D)*hh / hxhxh));
    Bc = conv * (T(0.5) * (vd / hh));
    C = diff * (T(0.5) * (-(D)*h_1 / hxhxh));
  }
  B = Bc + Bd;
}

// The nine coefficients of the Actual row at (i, j, k): A, B, C along x, y, z.
template <typename T>
__device__ __forceinline__ void ad_coefs(const StencilGrid<T>& g, int i, int j, int k, int c, T* q) {
  const T D = g.adDf ? g.adDf[c] : g.ad_D;   // diffCoefVar[i][j][k] (XProblem.cpp:3204) or the constant
  if (g.ad_upwind) {
    ad_coef_upwind<T>(g.hx, i, g.adv0[c], D, g.ad_conv, g.ad_diff, q[0], q[1], q[2]);
    ad_coef_upwind<T>(g.hy, j, g.adv1[c], D, g.ad_conv, g.ad_diff, q[3], q[4], q[5]);
    ad_coef_upwind<T>(g.hz, k, g.adv2[c], D, g.ad_conv, g.ad_diff, q[6], q[7], q[8]);
  } else {
    ad_coef<T>(g.hx, i, g.adv0[c], D, g.ad_conv, g.ad_diff, q[0], q[1], q[2]);
    ad_coef<T>(g.hy, j, g.adv1[c], D, g.ad_conv, g.ad_diff, q[3], q[4], q[5]);
    ad_coef<T>(g.hz, k, g.adv2[c], D, g.ad_conv, g.ad_diff, q[6], q[7], q[8]);
  }
}

// EXACT: (1/tau) f_c, then per direction A f[m-1] + B f_c + C f[m+1], the
// reference's operation order (19 FP64 operations and 15 divisions a row).
// Otherwise, from the table when there is one: the centre coefficient
// 1/tau + B_x + B_y + B_z and six FMAs (7 FP64 operations: GB300's FP64 rate
// bounds this row, not its bytes).
template <typename T, bool EXACT>
__device__ __forceinline__ T ad_actual(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k, int c) {
  const int s1 = g.s1, s2 = g.s2;
  const T fc = f[c];
  if (!EXACT && g.adc) {
    const T* __restrict__ q = g.adc + c;
    const int64_t n = g.adc_n;
    T res = q[0] * fc;
    res = fma(q[n], f[c - s1], res);
    res = fma(q[2 * n], f[c + s1], res);
    res = fma(q[3 * n], f[c - s2], res);
    res = fma(q[4 * n], f[c + s2], res);
    res = fma(q[5 * n], f[c - 1], res);
    res = fma(q[6 * n], f[c + 1], res);
    return res;
  }
  T q[9];
  ad_coefs<T>(g, i, j, k, c, q);
  T res = g.ad_itau * fc;
  res = res + (q[0] * f[c - s1] + q[1] * fc + q[2] * f[c + s1]);
  res = res + (q[3] * f[c - s2] + q[4] * fc + q[5] * f[c + s2]);
  res = res + (q[6] * f[c - 1] + q[7] * fc + q[8] * f[c + 1]);
  return res;
}

// One row of A applied to f at cell c of kind kb (row != ROW_NONE).
template <typename T, int OP, bool EXACT>
__device__ __forceinline__ T apply_row(const StencilGrid<T>& g, const T* __restrict__ f, int i, int j, int k, int c,
                                       uint8_t kb) {
  const int row = row_of(kb);
  if (row == ROW_ACTUAL) {
    if (OP == XF_OP_ADVDIFF) return ad_actual<T, EXACT>(g, f, i, j, k, c);
    if (OP == XF_OP_LAPLACE) return EXACT ? exact_lap_actual<T>(g, f, i, j, k, c, kb) : fast_lap_actual<T>(g, f, i, j, k, c, kb);
    return EXACT ? exact_vd_actual<T>(g, f, i, j, k, c, kb) : fast_vd_actual<T>(g, f, i, j, k, c, kb);
  }
  return boundary_row<T, OP == XF_OP_VARDIV>(g, f, i, j, k, c, row);
}

template <typename T>
StencilGrid<T> make_stencil_grid(const xf_grid* g, const T* rho);
