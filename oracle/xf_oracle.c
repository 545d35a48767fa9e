/* Test infrastructure only: CPU restatement of the reference's pressure-path
 * arithmetic.  See xf_oracle.h.  Parity of this restatement is pinned by
 * tests/test_oracle_golden.py against fixtures produced by the reference's
 * own compiled classes (tests/golden/make_golden.py).
 *
 * With xfo_set_threads(1) every loop runs in the reference's i->j->k order
 * with the reference's operation order (bit-exact operator and vector
 * algebra).  More threads parallelise the cell loops for the timed CPU
 * baseline; reductions then sum per-thread partials (not bit-exact).
 */
#define _GNU_SOURCE
#include "xf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void xfo_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int xfo_get_threads(void) { return g_threads; }

enum { FICT = 0, ACT = 1, DEF = 3, PREDEF = 4, NORM = 5, PRENORM = 6, EQU = 7, PREEQU = 8 };

/* XProblem.cpp:4155-4182: grid codes -> space mask. */
void xfo_space_mask(const int32_t* codes, int64_t ncell, uint8_t* smask) {
  for (int64_t c = 0; c < ncell; c++) {
    int m = codes[c];
    smask[c] = (m == ACT || m == PREDEF || m == NORM || m == PRENORM || m == PREEQU) ? 1 : 0;
  }
}

/* XSpaceModel.cpp:383-406: Rn numbering, 1-based, i->j->k order. */
int64_t xfo_rn_map(const uint8_t* smask, int n1, int n2, int n3, int32_t* inv_box, int32_t* fwd_ijk) {
  int64_t num = 0;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        int64_t c = ((int64_t)i * n2 + j) * n3 + k;
        if (smask[c] > 0) {
          num++;
          if (inv_box) inv_box[c] = (int32_t)num;
          if (fwd_ijk) { fwd_ijk[3 * (num - 1)] = i; fwd_ijk[3 * (num - 1) + 1] = j; fwd_ijk[3 * (num - 1) + 2] = k; }
        } else if (inv_box) {
          inv_box[c] = 0;
        }
      }
  return num;
}

/* Every check the reference makes while evaluating an active row
 * (XOperator.cpp:971-1123, 1933-2227), plus index-range checks for reads the
 * reference would make outside its arrays.  Returns XFO_ERR_MASK and the first
 * offending cell. */
int xfo_validate(int op, const int32_t* codes, const double* normals, int n1, int n2, int n3, int64_t* bad) {
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        int64_t c = ((int64_t)i * n2 + j) * n3 + k;
        int m = codes[c];
        int known = (m == FICT || m == ACT || m == DEF || m == PREDEF || m == NORM || m == PRENORM || m == EQU || m == PREEQU);
        int interior = i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 2;
        int ok = 1;
        if (!known) ok = 0;
        else if (m == NORM || m == PREEQU) ok = 0;
        else if (m == ACT) ok = interior;
        else if (m == PREDEF || m == PRENORM) {
          double nx = normals[3 * c], ny = normals[3 * c + 1], nz = normals[3 * c + 2];
          if (nx == 0 && ny == 0 && nz == 0) ok = 0;
          else if (m == PREDEF) {
            if (nx != 0) ok = (ny == 0 && nz == 0 && fabs(nx) == 1);
            else if (ny != 0) ok = (nx == 0 && nz == 0 && fabs(ny) == 1);
            else ok = (nx == 0 && ny == 0 && fabs(nz) == 1);
            if (ok) {
              int di = nx > 0 ? -1 : nx < 0 ? 1 : 0, dj = ny > 0 ? -1 : ny < 0 ? 1 : 0, dk = nz > 0 ? -1 : nz < 0 ? 1 : 0;
              ok = i + di >= 0 && i + di < n1 && j + dj >= 0 && j + dj < n2 && k + dk >= 0 && k + dk < n3;
            }
          } else {
            int lo_i = nx > 0 ? -1 : 0, hi_i = nx < 0 ? 1 : 0;
            int lo_j = ny > 0 ? -1 : 0, hi_j = ny < 0 ? 1 : 0;
            int lo_k = nz > 0 ? -1 : 0, hi_k = nz < 0 ? 1 : 0;
            ok = i + lo_i >= 0 && i + hi_i < n1 && j + lo_j >= 0 && j + hi_j < n2 && k + lo_k >= 0 && k + hi_k < n3;
            if (op == XFO_OP_VARDIV) ok = ok && interior;
          }
        }
        if (!ok) { if (bad) *bad = c; return XFO_ERR_MASK; }
      }
  return XFO_OK;
}

typedef struct {
  int n1, n2, n3;
  int64_t s1, s2;
  const int32_t* codes;
  const double* nrm;
  const double *hx, *hy, *hz, *rho;
} xfo_grid;

/* T3dLaplaceOperator::operator(), XOperator.cpp:938-1129 (Actual, PreDefined,
 * PreNormal branches). */
static double lap_row(const xfo_grid* g, const double* f, int i, int j, int k) {
  const int64_t s1 = g->s1, s2 = g->s2;
  const int64_t c = i * s1 + j * s2 + k;
  const int m = g->codes[c];
  const int32_t* mask = g->codes;
  if (m == ACT) {
    double hx_2X = (g->hx[i - 1] + g->hx[i]) / 2;
    double hx_2Y = (g->hy[j - 1] + g->hy[j]) / 2;
    double hx_2Z = (g->hz[k - 1] + g->hz[k]) / 2;
    double f_i_1 = (f[c] - f[c - s1]) / (g->hx[i - 1]);
    double f_i = (f[c + s1] - f[c]) / (g->hx[i]);
    double f_j_1 = (f[c] - f[c - s2]) / (g->hy[j - 1]);
    double f_j = (f[c + s2] - f[c]) / (g->hy[j]);
    double f_k_1 = (f[c] - f[c - 1]) / (g->hz[k - 1]);
    double f_k = (f[c + 1] - f[c]) / (g->hz[k]);
    if (mask[c - s1] == FICT) f_i_1 = 0;
    if (mask[c + s1] == FICT) f_i = 0;
    if (mask[c - s2] == FICT) f_j_1 = 0;
    if (mask[c + s2] == FICT) f_j = 0;
    if (mask[c - 1] == FICT) f_k_1 = 0;
    if (mask[c + 1] == FICT) f_k = 0;
    return -((f_i - f_i_1) / hx_2X + (f_j - f_j_1) / hx_2Y + (f_k - f_k_1) / hx_2Z);
  }
  const double nx = g->nrm[3 * c], ny = g->nrm[3 * c + 1], nz = g->nrm[3 * c + 2];
  if (m == PREDEF) {
    double semiSum = 0;
    if (nx > 0) semiSum = (f[c] + f[c - s1]) / 2;
    else if (nx < 0) semiSum = (f[c + s1] + f[c]) / 2;
    if (ny > 0) semiSum = (f[c] + f[c - s2]) / 2;
    else if (ny < 0) semiSum = (f[c + s2] + f[c]) / 2;
    if (nz > 0) semiSum = (f[c] + f[c - 1]) / 2;
    else if (nz < 0) semiSum = (f[c + 1] + f[c]) / 2;
    return semiSum;
  }
  /* PreNormal */
  int sI = 0, sI1 = 0, sJ = 0, sJ1 = 0, sK = 0, sK1 = 0;
  double hxl = 1, hyl = 1, hzl = 1;
  if (nx > 0) { sI = 0; sI1 = -1; hxl = g->hx[i - 1]; } else if (nx < 0) { sI = 1; sI1 = 0; hxl = g->hx[i]; }
  if (ny > 0) { sJ = 0; sJ1 = -1; hyl = g->hy[j - 1]; } else if (ny < 0) { sJ = 1; sJ1 = 0; hyl = g->hy[j]; }
  if (nz > 0) { sK = 0; sK1 = -1; hzl = g->hz[k - 1]; } else if (nz < 0) { sK = 1; sK1 = 0; hzl = g->hz[k]; }
#define F(a, b, d) f[(int64_t)(i + (a)) * s1 + (int64_t)(j + (b)) * s2 + (k + (d))]
  double fl = (F(sI, 0, 0) + F(sI, sJ, 0) + F(sI, 0, sK) + F(sI, sJ, sK)) / 4;
  double fl_1 = (F(sI1, 0, 0) + F(sI1, sJ, 0) + F(sI1, 0, sK) + F(sI1, sJ, sK)) / 4;
  double dfx = (fl - fl_1) / hxl;
  fl = (F(0, sJ, 0) + F(sI, sJ, 0) + F(0, sJ, sK) + F(sI, sJ, sK)) / 4;
  fl_1 = (F(0, sJ1, 0) + F(sI, sJ1, 0) + F(0, sJ1, sK) + F(sI, sJ1, sK)) / 4;
  double dfy = (fl - fl_1) / hyl;
  fl = (F(0, 0, sK) + F(sI, 0, sK) + F(0, sJ, sK) + F(sI, sJ, sK)) / 4;
  fl_1 = (F(0, 0, sK1) + F(sI, 0, sK1) + F(0, sJ, sK1) + F(sI, sJ, sK1)) / 4;
  double dfz = (fl - fl_1) / hzl;
#undef F
  if (g->rho == NULL) return dfx * nx + dfy * ny + dfz * nz;
  /* T3dVariableDivergentedOperator PreNormal tail, XOperator.cpp:2211-2221,
   * including its precedence (rho[i+1] - rho[i]/h). */
  const double* rho = g->rho;
  double d_x = rho[c + s1] - rho[c] / (g->hx[i - 1]);
  double d_y = rho[c + s2] - rho[c] / (g->hy[j - 1]);
  double d_z = rho[c + 1] - rho[c] / (g->hz[k - 1]);
  double laplace_p = dfx * nx + dfy * ny + dfz * nz;
  double divergence_density = d_x + d_y + d_z;
  return rho[c] * laplace_p - divergence_density * f[c];
}

/* T3dVariableDivergentedOperator::operator() Actual branch, XOperator.cpp:1933-2026. */
static double vardiv_actual(const xfo_grid* g, const double* f, int i, int j, int k) {
  const int64_t s1 = g->s1, s2 = g->s2;
  const int64_t c = i * s1 + j * s2 + k;
  const int32_t* mask = g->codes;
  const double* rho = g->rho;
  double h_1X = g->hx[i - 1], hX = g->hx[i];
  double h_1Y = g->hy[j - 1], hY = g->hy[j];
  double h_1Z = g->hz[k - 1], hZ = g->hz[k];
  double hx_2X = (g->hx[i - 1] + g->hx[i]) / 2;
  double hx_2Y = (g->hy[j - 1] + g->hy[j]) / 2;
  double hx_2Z = (g->hz[k - 1] + g->hz[k]) / 2;
  double f_i_1 = rho[c - s1] * (f[c] - f[c - s1]) / (h_1X);
  double f_i = rho[c + s1] * (f[c + s1] - f[c]) / (hX);
  double f_j_1 = rho[c - s2] * (f[c] - f[c - s2]) / (h_1Y);
  double f_j = rho[c + s2] * (f[c + s2] - f[c]) / (hY);
  double f_k_1 = rho[c - 1] * (f[c] - f[c - 1]) / (h_1Z);
  double f_k = rho[c + 1] * (f[c + 1] - f[c]) / (hZ);
  double d_i = (rho[c + s1] - rho[c]) / (h_1X);
  double d_j = (rho[c + s2] - rho[c]) / (h_1Y);
  double d_k = (rho[c + 1] - rho[c]) / (h_1Z);
  if (mask[c - s1] == FICT) f_i_1 = 0;
  if (mask[c + s1] == FICT) { f_i = 0; d_i = 0; }
  if (mask[c - s2] == FICT) f_j_1 = 0;
  if (mask[c + s2] == FICT) { f_j = 0; d_j = 0; }
  if (mask[c - 1] == FICT) f_k_1 = 0;
  if (mask[c + 1] == FICT) { f_k = 0; d_k = 0; }
  double laplace_p = ((f_i - f_i_1) / hx_2X + (f_j - f_j_1) / hx_2Y + (f_k - f_k_1) / hx_2Z);
  double divergence_density = d_i + d_j + d_k;
  return -(rho[c] * laplace_p - divergence_density * f[c]);
}

static double row(int op, const xfo_grid* g, const double* f, int i, int j, int k) {
  int64_t c = i * g->s1 + j * g->s2 + k;
  if (op == XFO_OP_VARDIV && g->codes[c] == ACT) return vardiv_actual(g, f, i, j, k);
  return lap_row(g, f, i, j, k);
}

static int active(const int32_t* codes, int64_t c) {
  int m = codes[c];
  return m == ACT || m == PREDEF || m == NORM || m == PRENORM || m == PREEQU;
}

/* TRnRelease3dSpace::LocalReleaseAssignSpeedLinearCombination(op),
 * XSpace.cpp:3013-3217: y = A x (+/- s) on cells with space mask > 0. */
int xfo_apply(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
              const double* hz, const double* density, int n1, int n2, int n3, const double* x,
              const double* s, int sign, double* y) {
  int64_t bad;
  if (xfo_validate(op, codes, normals, n1, n2, n3, &bad) != XFO_OK) return XFO_ERR_MASK;
  xfo_grid g = {n1, n2, n3, (int64_t)n2 * n3, n3, codes, normals, hx, hy, hz, op == XFO_OP_VARDIV ? density : NULL};
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        int64_t c = ((int64_t)i * n2 + j) * n3 + k;
        if (!active(codes, c)) continue;
        double v = row(op, &g, x, i, j, k);
        if (sign > 0) v = v + s[c];
        else if (sign < 0) v = v - s[c];
        y[c] = v;
      }
  return XFO_OK;
}

/* XSpace.cpp:2489-3010: z = p1*s1 + p2*s2 on active cells. */
void xfo_lincomb(double p1, const double* s1, double p2, const double* s2, const uint8_t* smask, int64_t n,
                 double* z) {
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t c = 0; c < n; c++)
    if (smask[c] > 0) {
      double a = s1 ? p1 * s1[c] : 0.0;
      z[c] = s2 ? a + p2 * s2[c] : a;
    }
}

/* XSpace.cpp:3261-3342 (sequential accumulation). */
double xfo_dot(const double* a, const double* b, const uint8_t* smask, int64_t n) {
  double res = 0;
  if (g_threads == 1) {
    for (int64_t c = 0; c < n; c++)
      if (smask[c] > 0) res = res + a[c] * b[c];
    return res;
  }
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(+ : res)
  for (int64_t c = 0; c < n; c++)
    if (smask[c] > 0) res = res + a[c] * b[c];
  return res;
}

/* XSpace.cpp:3219-3259 + 1205-1217: sqrtl of the masked sum of squares. */
double xfo_norm(const double* a, const uint8_t* smask, int64_t n) {
  double res = 0;
  for (int64_t c = 0; c < n; c++)
    if (smask[c] > 0) res = res + a[c] * a[c];
  return (double)sqrtl(res);
}

/* XSpace.cpp:3428-3487 (type 1): first strict maximum of |a| in i->j->k order;
 * Rn index 1 when nothing beats 0. */
double xfo_absmax(const double* a, const uint8_t* smask, const int32_t* inv, int64_t n, int32_t* rn) {
  double res = 0;
  int32_t idx = 1;
  for (int64_t c = 0; c < n; c++)
    if (smask[c] > 0) {
      double v = fabs(a[c]);
      if (v > res) { res = v; idx = inv[c]; }
    }
  if (rn) *rn = idx;
  return res;
}

/* ------------------------------------------------------------------------ */
typedef struct {
  int op;
  xfo_grid g;
  uint8_t* smask;
  int64_t n;
} sys_t;

static int sys_init(sys_t* S, int op, const int32_t* codes, const double* normals, const double* hx,
                    const double* hy, const double* hz, const double* density, int n1, int n2, int n3) {
  int64_t bad;
  if (xfo_validate(op, codes, normals, n1, n2, n3, &bad) != XFO_OK) return XFO_ERR_MASK;
  S->op = op;
  xfo_grid g = {n1, n2, n3, (int64_t)n2 * n3, n3, codes, normals, hx, hy, hz, op == XFO_OP_VARDIV ? density : NULL};
  S->g = g;
  S->n = (int64_t)n1 * n2 * n3;
  S->smask = (uint8_t*)malloc(S->n);
  xfo_space_mask(codes, S->n, S->smask);
  return XFO_OK;
}

static void apply(sys_t* S, const double* x, const double* s, int sign, double* y) {
  xfo_grid* g = &S->g;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int i = 0; i < g->n1; i++)
    for (int j = 0; j < g->n2; j++)
      for (int k = 0; k < g->n3; k++) {
        int64_t c = ((int64_t)i * g->n2 + j) * g->n3 + k;
        if (!S->smask[c]) continue;
        double v = row(S->op, g, x, i, j, k);
        if (sign > 0) v = v + s[c];
        else if (sign < 0) v = v - s[c];
        y[c] = v;
      }
}

/* (A x, y) through LocalReleaseInnerproduct(op), XSpace.cpp:3344-3419. */
static double dot_op(sys_t* S, const double* x, const double* y) {
  xfo_grid* g = &S->g;
  double res = 0;
  if (g_threads == 1) {
    for (int i = 0; i < g->n1; i++)
      for (int j = 0; j < g->n2; j++)
        for (int k = 0; k < g->n3; k++) {
          int64_t c = ((int64_t)i * g->n2 + j) * g->n3 + k;
          if (S->smask[c]) res = res + y[c] * row(S->op, g, x, i, j, k);
        }
    return res;
  }
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(+ : res)
  for (int i = 0; i < g->n1; i++)
    for (int j = 0; j < g->n2; j++)
      for (int k = 0; k < g->n3; k++) {
        int64_t c = ((int64_t)i * g->n2 + j) * g->n3 + k;
        if (S->smask[c]) res = res + y[c] * row(S->op, g, x, i, j, k);
      }
  return res;
}

static double* zeros(int64_t n) { return (double*)calloc((size_t)n, sizeof(double)); }
static double* copyv(const double* a, int64_t n) {
  double* p = (double*)malloc((size_t)n * sizeof(double));
  memcpy(p, a, (size_t)n * sizeof(double));
  return p;
}
static void massign(double* dst, const double* src, const uint8_t* m, int64_t n) {
  for (int64_t c = 0; c < n; c++)
    if (m[c]) dst[c] = src[c];
}

/* TSLAE::SolveByConjugateGradients, XSLAE.cpp:56-157 (three-term form, true
 * residual every iteration, ||r||_2 <= eps absolute). */
int xfo_cg_reference(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                     const double* hz, const double* density, int n1, int n2, int n3, const double* x0,
                     const double* b, double eps, int maxit, double* result, xfo_stats* st) {
  sys_t S;
  if (sys_init(&S, op, codes, normals, hx, hy, hz, density, n1, n2, n3)) return XFO_ERR_MASK;
  const int64_t n = S.n;
  const uint8_t* m = S.smask;
  if (eps <= 0) eps = 1e-5;
  memcpy(result, x0, (size_t)n * sizeof(double));
  for (int64_t c = 0; c < n; c++) if (m[c]) result[c] = 0; /* *fResult |= 0 */
  double* xk_1 = copyv(x0, n);
  double* rk_1 = zeros(n);
  apply(&S, xk_1, b, -1, rk_1);
  double rk_1Xrk_1 = xfo_dot(rk_1, rk_1, m, n);
  massign(result, xk_1, m, n);
  st->iterations = 0; st->status = 0; st->resid = sqrt(rk_1Xrk_1);
  if (rk_1Xrk_1 != 0) {
    double tauk = rk_1Xrk_1 / dot_op(&S, rk_1, rk_1);
    double* xk = copyv(x0, n);
    xfo_lincomb(1.0, xk_1, -tauk, rk_1, m, n, xk);
    double* rk = zeros(n);
    apply(&S, xk, b, -1, rk);
    double rkXrk = xfo_dot(rk, rk, m, n);
    massign(result, xk, m, n);
    if (rkXrk != 0) {
      double alfak = 1;
      int it = 0;
      double epsCur = (double)sqrtl(rkXrk);
      while (epsCur > eps) {
        if (maxit > 0 && it >= maxit) { st->status = 13; break; }
        it++;
        double tauk1 = rkXrk / dot_op(&S, rk, rk);
        double alfak1 = 1 - (1 / alfak) * (tauk1 / tauk) * (rkXrk / rk_1Xrk_1);
        alfak1 = 1 / alfak1;
        xfo_lincomb(alfak1, xk, (1 - alfak1), xk_1, m, n, result);
        xfo_lincomb(1.0, result, -(tauk1 * alfak1), rk, m, n, result);
        massign(xk_1, xk, m, n);
        massign(rk_1, rk, m, n);
        rk_1Xrk_1 = rkXrk;
        tauk = tauk1;
        alfak = alfak1;
        massign(xk, result, m, n);
        apply(&S, xk, b, -1, rk);
        rkXrk = xfo_dot(rk, rk, m, n);
        epsCur = (double)sqrtl(rkXrk);
      }
      st->iterations = it;
      st->resid = epsCur;
    }
    free(xk); free(rk);
  }
  free(xk_1); free(rk_1); free(S.smask);
  return XFO_OK;
}

/* TSLAE::SolveByBiConjugateGradientsStab, XSLAE.cpp:667-768 (warm start,
 * ||r||_inf <= eps). */
int xfo_bicgstab_reference(int op, const int32_t* codes, const double* normals, const double* hx,
                           const double* hy, const double* hz, const double* density, int n1, int n2, int n3,
                           const double* x0, const double* b, double eps, int maxit, double* result,
                           xfo_stats* st) {
  sys_t S;
  if (sys_init(&S, op, codes, normals, hx, hy, hz, density, n1, n2, n3)) return XFO_ERR_MASK;
  const int64_t n = S.n;
  const uint8_t* m = S.smask;
  if (eps <= 0) eps = 1e-5;
  int32_t idx;
  int32_t* inv = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  xfo_rn_map(m, n1, n2, n3, inv, NULL);
  memcpy(result, x0, (size_t)n * sizeof(double));
  for (int64_t c = 0; c < n; c++) if (m[c]) result[c] = 0;
  double* Un = copyv(x0, n);
  double *tmp1 = zeros(n), *tmp2 = zeros(n), *Rn = zeros(n), *sRn = zeros(n);
  double *Pn = zeros(n), *Pn1 = zeros(n), *Vn = zeros(n), *Sn = zeros(n), *Tn = zeros(n);
  apply(&S, Un, NULL, 0, Rn);
  xfo_lincomb(1.0, b, -1.0, Rn, m, n, Rn);
  massign(sRn, Rn, m, n);
  double pn = 1., an = 1., bn = 1., wn = 1., pn1;
  int it = 0;
  double norm = xfo_absmax(Rn, m, inv, n, &idx);
  st->status = 0;
  while (norm > eps) {
    if (maxit > 0 && it >= maxit) { st->status = 13; break; }
    it++;
    pn1 = xfo_dot(sRn, Rn, m, n);
    bn = (pn1 / pn) * (an / wn);
    xfo_lincomb(wn, Vn, 0, NULL, m, n, Pn1);
    xfo_lincomb(1.0, Pn, -1.0, Pn1, m, n, Pn1);
    xfo_lincomb(bn, Pn1, 0, NULL, m, n, Pn1);
    xfo_lincomb(1.0, Rn, 1.0, Pn1, m, n, Pn1);
    apply(&S, Pn1, NULL, 0, Vn);
    an = pn1 / xfo_dot(sRn, Vn, m, n);
    xfo_lincomb(an, Vn, 0, NULL, m, n, Sn);
    xfo_lincomb(1.0, Rn, -1.0, Sn, m, n, Sn);
    apply(&S, Sn, NULL, 0, Tn);
    wn = xfo_dot(Tn, Sn, m, n) / xfo_dot(Tn, Tn, m, n);
    xfo_lincomb(an, Pn1, 0, NULL, m, n, tmp1);
    xfo_lincomb(1.0, tmp1, wn, Sn, m, n, tmp2);
    xfo_lincomb(1.0, Un, 1.0, tmp2, m, n, Un);
    xfo_lincomb(wn, Tn, 0, NULL, m, n, Rn);
    xfo_lincomb(1.0, Sn, -1.0, Rn, m, n, Rn);
    pn = pn1;
    massign(Pn, Pn1, m, n);
    norm = xfo_absmax(Rn, m, inv, n, &idx);
  }
  massign(result, Un, m, n);
  st->iterations = it;
  st->resid = norm;
  free(Un); free(tmp1); free(tmp2); free(Rn); free(sRn); free(Pn); free(Pn1); free(Vn); free(Sn); free(Tn);
  free(inv); free(S.smask);
  return XFO_OK;
}

/* TSLAE::SolveByMinimalResiduals, XSLAE.cpp:350-414 (||r||_2 <= eps). */
int xfo_minres_reference(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                         const double* hz, const double* density, int n1, int n2, int n3, const double* x0,
                         const double* b, double eps, int maxit, double* result, xfo_stats* st) {
  sys_t S;
  if (sys_init(&S, op, codes, normals, hx, hy, hz, density, n1, n2, n3)) return XFO_ERR_MASK;
  const int64_t n = S.n;
  const uint8_t* m = S.smask;
  if (eps <= 0) eps = 1e-7;
  memcpy(result, x0, (size_t)n * sizeof(double));
  for (int64_t c = 0; c < n; c++) if (m[c]) result[c] = 0;
  double* xk = copyv(x0, n);
  double *rk = zeros(n), *Ark = zeros(n);
  apply(&S, xk, b, -1, rk);
  double rkXrk = xfo_dot(rk, rk, m, n);
  massign(result, xk, m, n);
  int it = 0;
  double epsCur = sqrt(rkXrk);
  st->status = 0;
  if (rkXrk != 0) {
    epsCur = (double)sqrtl(rkXrk);
    while (epsCur > eps) {
      if (maxit > 0 && it >= maxit) { st->status = 13; break; }
      it++;
      apply(&S, rk, NULL, 0, Ark);
      double alfa = (-1) * xfo_dot(Ark, rk, m, n) / xfo_dot(Ark, Ark, m, n);
      xfo_lincomb(1.0, xk, alfa, rk, m, n, xk);
      apply(&S, xk, b, -1, rk);
      rkXrk = xfo_dot(rk, rk, m, n);
      epsCur = (double)sqrtl(rkXrk);
    }
  }
  massign(result, xk, m, n);
  st->iterations = it;
  st->resid = epsCur;
  free(xk); free(rk); free(Ark); free(S.smask);
  return XFO_OK;
}

/* Laplace grids whose active cells are all Actual (XOperator.cpp:994-1019)
 * and interior: the flux-form rows of lap_row, written as straight-line code
 * over k (each row the same divisions and roundings as lap_row; Fictive
 * neighbours select a zero flux), y = 0 on other cells, and (p, y) summed on
 * the way.  One OpenMP team over i planes; the k loop vectorises (IEEE
 * division in every lane). */
static int all_actual_interior(const sys_t* S) {
  if (S->op != XFO_OP_LAPLACE) return 0;
  const xfo_grid* g = &S->g;
  for (int i = 0; i < g->n1; i++)
    for (int j = 0; j < g->n2; j++)
      for (int k = 0; k < g->n3; k++) {
        const int64_t c = ((int64_t)i * g->n2 + j) * g->n3 + k;
        if (!S->smask[c]) continue;
        if (g->codes[c] != ACT) return 0;
        if (i == 0 || j == 0 || k == 0 || i == g->n1 - 1 || j == g->n2 - 1 || k == g->n3 - 1) return 0;
      }
  return 1;
}

static double lap_actual_sweep(const sys_t* S, const double* f, double* y, const double* hz2) {
  const xfo_grid* g = &S->g;
  const int n1 = g->n1, n2 = g->n2, n3 = g->n3;
  const int64_t s1 = g->s1, s2 = g->s2;
  const int32_t* mask = g->codes;
  double pq = 0;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(+ : pq) if (g_threads > 1)
  for (int i = 0; i < n1; i++) {
    for (int j = 0; j < n2; j++) {
      const int64_t row0 = (int64_t)i * s1 + (int64_t)j * s2;
      if (i == 0 || j == 0 || i == n1 - 1 || j == n2 - 1) {
        for (int k = 0; k < n3; k++) y[row0 + k] = 0;
        continue;
      }
      const double hxm = g->hx[i - 1], hxp = g->hx[i], hym = g->hy[j - 1], hyp = g->hy[j];
      const double hx_2X = (hxm + hxp) / 2, hx_2Y = (hym + hyp) / 2;
      const double* hz = g->hz;
      y[row0] = 0;
      y[row0 + n3 - 1] = 0;
      double acc = 0;
#pragma omp simd reduction(+ : acc)
      for (int k = 1; k < n3 - 1; k++) {
        const int64_t c = row0 + k;
        double f_i_1 = (f[c] - f[c - s1]) / hxm;
        double f_i = (f[c + s1] - f[c]) / hxp;
        double f_j_1 = (f[c] - f[c - s2]) / hym;
        double f_j = (f[c + s2] - f[c]) / hyp;
        double f_k_1 = (f[c] - f[c - 1]) / hz[k - 1];
        double f_k = (f[c + 1] - f[c]) / hz[k];
        f_i_1 = mask[c - s1] == FICT ? 0.0 : f_i_1;
        f_i = mask[c + s1] == FICT ? 0.0 : f_i;
        f_j_1 = mask[c - s2] == FICT ? 0.0 : f_j_1;
        f_j = mask[c + s2] == FICT ? 0.0 : f_j;
        f_k_1 = mask[c - 1] == FICT ? 0.0 : f_k_1;
        f_k = mask[c + 1] == FICT ? 0.0 : f_k;
        const double v = -((f_i - f_i_1) / hx_2X + (f_j - f_j_1) / hx_2Y + (f_k - f_k_1) / hz2[k]);
        const double yv = mask[c] == ACT ? v : 0.0;
        y[c] = yv;
        acc += f[c] * yv;
      }
      pq += acc;
    }
  }
  return pq;
}

/* Plain Hestenes-Stiefel CG with a relative-residual stop: the FP64 CPU
 * counterpart of the GPU's plain FP64 CG (not a reference routine; the
 * reference's CG is the three-term form above).  Its rows are the reference
 * operator's (lap_row / row); on all-Actual Laplace grids the fused sweep
 * above computes them with (p, A p), and the vector update computes (r, r). */
int xfo_cg_plain(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                 const double* hz, const double* density, int n1, int n2, int n3, const double* x0,
                 const double* b, double rtol, int maxit, double* result, xfo_stats* st) {
  sys_t S;
  if (sys_init(&S, op, codes, normals, hx, hy, hz, density, n1, n2, n3)) return XFO_ERR_MASK;
  const int64_t n = S.n;
  const uint8_t* m = S.smask;
  const int fast = all_actual_interior(&S);
  double* hz2 = (double*)calloc((size_t)n3, sizeof(double));
  for (int k = 1; k < n3 - 1; k++) hz2[k] = (hz[k - 1] + hz[k]) / 2;
  memcpy(result, x0, (size_t)n * sizeof(double));
  double *r = zeros(n), *p = zeros(n), *q = zeros(n);
  apply(&S, result, b, -1, r); /* r = A x - b */
  xfo_lincomb(-1.0, r, 0, NULL, m, n, r);
  double bb = xfo_dot(b, b, m, n);
  double rr = xfo_dot(r, r, m, n);
  massign(p, r, m, n);
  int it = 0;
  st->status = 0;
  double thr = rtol * rtol * bb;
  while (rr > thr) {
    if (maxit > 0 && it >= maxit) { st->status = 13; break; }
    it++;
    double pq;
    if (fast) {
      pq = lap_actual_sweep(&S, p, q, hz2);
    } else {
      apply(&S, p, NULL, 0, q);
      pq = xfo_dot(p, q, m, n);
    }
    const double alpha = rr / pq;
    double rr_new = 0;
#pragma omp parallel for simd num_threads(g_threads) schedule(static) reduction(+ : rr_new) if (g_threads > 1)
    for (int64_t c = 0; c < n; c++) {
      const double mk = m[c] ? 1.0 : 0.0;
      const double xn = result[c] + alpha * p[c];
      const double rn = r[c] - alpha * q[c];
      result[c] = m[c] ? xn : result[c];
      r[c] = m[c] ? rn : r[c];
      rr_new += mk * (rn * rn);
    }
    const double beta = rr_new / rr;
    rr = rr_new;
#pragma omp parallel for simd num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (int64_t c = 0; c < n; c++) p[c] = m[c] ? r[c] + beta * p[c] : p[c];
  }
  st->iterations = it;
  st->resid = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  free(r); free(p); free(q); free(hz2); free(S.smask);
  return XFO_OK;
}

/* TSLAE::SolveByScalarRunning, XSLAE.cpp:416-445. */
void xfo_thomas(int M, double* u, const double* a, const double* b, const double* c, const double* f) {
  double* A = (double*)malloc(sizeof(double) * (M + 1));
  double* B = (double*)malloc(sizeof(double) * (M + 1));
  A[0] = 0;
  B[0] = u[0];
  A[M] = B[M] = 0;
  for (int m = 1; m < M; m++) {
    A[m] = (-c[m]) / (a[m] * A[m - 1] + b[m]);
    B[m] = (f[m] - a[m] * B[m - 1]) / (a[m] * A[m - 1] + b[m]);
  }
  for (int m = M - 1; m > 0; m--) u[m] = A[m] * u[m + 1] + B[m];
  free(A);
  free(B);
}

/* ------------------------------------------------------------------------ */
#define IB_RANGE 3

/* TImmersedBoundaryProblem::Index(grid, coord, type, axis, 3, 3), XProblem.cpp:8931-8967. */
static int ib_index(double coord, double step, int nend, int type, int axis) {
  int index = (int)floor((coord + (type != axis ? 0.5 * step : 0)) / step);
  if (index > (nend - 1) - IB_RANGE) index = (nend - 1) - IB_RANGE;
  if (index < IB_RANGE) index = IB_RANGE;
  return index;
}
/* Coord(grid, index, type, axis), XProblem.cpp:8988-9006. */
static double ib_coord(int index, double step, int type, int axis) {
  return index * step - (type != axis ? 0.5 * step : 0);
}
/* OptimalDirichlet, XProblem.cpp:9008-9032 (cosine delta). */
static double ib_delta(double distance, double h) {
  if (distance < 2 * h) return 1.0 / (4 * h) * (1 + cos(M_PI * distance / (2 * h)));
  return 0;
}

/* TImmersedBoundaryProblem::Interpolate, XProblem.cpp:8620-8791. h0 holds
 * Separation[0] of the three separators; the box has n-1 intervals per axis. */
void xfo_ib_interpolate(const double* vel, int n1, int n2, int n3, const double* h0, int axis, int nn,
                        const double* pos, double* node_vel) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const double cb = h0[axis - 1] * h0[axis - 1] * h0[axis - 1];
  for (int q = 0; q < nn; q++) {
    double px = pos[3 * q], py = pos[3 * q + 1], pz = pos[3 * q + 2];
    int xi = ib_index(px, h0[0], n1 - 1, 1, axis);
    int yi = ib_index(py, h0[1], n2 - 1, 2, axis);
    int zi = ib_index(pz, h0[2], n3 - 1, 3, axis);
    double acc = 0;
    for (int i = xi - IB_RANGE; i <= xi + IB_RANGE; ++i)
      for (int j = yi - IB_RANGE; j <= yi + IB_RANGE; ++j)
        for (int k = zi - IB_RANGE; k <= zi + IB_RANGE; ++k) {
          double wx = ib_delta(fabs(px - ib_coord(i, h0[0], 1, axis)), h0[0]);
          double wy = ib_delta(fabs(py - ib_coord(j, h0[1], 2, axis)), h0[1]);
          double wz = ib_delta(fabs(pz - ib_coord(k, h0[2], 3, axis)), h0[2]);
          acc += (vel[i * s1 + j * s2 + k] * wx * wy * wz) * cb;
        }
    node_vel[q] = acc;
  }
}

/* UpdateBoundaryPosition, XProblem.cpp:8858-8894. */
void xfo_ib_update(int nn, int axis, double tau, const double* node_vel, double* pos) {
  for (int q = 0; q < nn; q++) pos[3 * q + axis - 1] += node_vel[q] * tau;
}

/* ComputeBoundaryForces, XProblem.cpp:8436-8547, with the node laws of
 * XImmersedBoundary.cpp:654-757.  params = {stiffness, stretchingStiffness,
 * bendingStiffness, area}.  Runs in node order (the reference's loop with one
 * thread; with several it races on neighbours' forces). */
void xfo_ib_forces(int nn, int axis, const double* pos, const double* ref, const int32_t* kind,
                   const int32_t* next, const int32_t* prev, const double* dist0, const double* curv0,
                   const double* node_stiff, const double* params, double* force) {
  const int a = axis - 1;
  const double stiffness = params[0], kst = params[1], kbend = params[2], area = params[3];
  for (int q = 0; q < nn; q++) force[q] = 0;
  for (int q = 0; q < nn; q++) {
    double sf = 0, bf = 0, tf = 0;
    int nx = next[q], pv = prev[q];
    int kd = kind[q];
    if ((kd == 0 || kd == 2 || kd == 4) && nx >= 0) {
      double DX = pos[3 * q] - pos[3 * nx], DY = pos[3 * q + 1] - pos[3 * nx + 1], DZ = pos[3 * q + 2] - pos[3 * nx + 2];
      double distance = sqrt(DX * DX + DY * DY + DZ * DZ);
      double distance_axis = pos[3 * q + a] - pos[3 * nx + a];
      double k = kd == 2 ? node_stiff[q] : kst;
      sf = k * (distance - dist0[q]) * distance_axis / distance;
    }
    if (kd == 0 && nx >= 0 && pv >= 0) {
      double curv = pos[3 * nx + a] - 2 * pos[3 * q + a] + pos[3 * pv + a];
      bf = kbend * (curv0[3 * q + a] - curv);
    }
    if (kd == 1 || kd == 4) tf = stiffness * (pos[3 * q + a] - ref[3 * q + a]);
    if (kd == 2) tf = node_stiff[q] * (pos[3 * q + a] - ref[3 * q + a]);
    force[q] += -(sf + 2 * bf + tf) * area;
    if (nx >= 0) force[nx] += (sf + bf) * area;
    if (pv >= 0) force[pv] += bf * area;
  }
}

/* SpreadForce, XProblem.cpp:8550-8617 (arithmetic only; the FIXED-node mask
 * rewrite is not part of it). fbox must already hold the zeroed force. */
void xfo_ib_spread(double* fbox, int n1, int n2, int n3, const double* h0, int axis, int nn, const double* pos,
                   const double* force) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  for (int q = 0; q < nn; q++) {
    double px = pos[3 * q], py = pos[3 * q + 1], pz = pos[3 * q + 2];
    int xi = ib_index(px, h0[0], n1 - 1, 1, axis);
    int yi = ib_index(py, h0[1], n2 - 1, 2, axis);
    int zi = ib_index(pz, h0[2], n3 - 1, 3, axis);
    for (int i = xi - IB_RANGE; i <= xi + IB_RANGE; ++i)
      for (int j = yi - IB_RANGE; j <= yi + IB_RANGE; ++j)
        for (int k = zi - IB_RANGE; k <= zi + IB_RANGE; ++k) {
          double wx = ib_delta(fabs(px - ib_coord(i, h0[0], 1, axis)), h0[0]);
          double wy = ib_delta(fabs(py - ib_coord(j, h0[1], 2, axis)), h0[1]);
          double wz = ib_delta(fabs(pz - ib_coord(k, h0[2], 3, axis)), h0[2]);
          fbox[i * s1 + j * s2 + k] += (force[q] * wx * wy * wz);
        }
  }
}

/* ------------------------------------------------------------------------ */
/* Pressure right-hand side, XProblem.cpp:5474-5512.  Point codes as XMask.h:
 * 0 Fictive, 1 Actual, 3 Defined, 4 PreDefined, 5 Normal, 6 PreNormal,
 * 7 Equation, 8 PreEquation.  An Actual cell on the box face would read
 * outside the velocity boxes in the reference: reported as XFO_ERR_MASK. */
int xfo_pressure_rhs(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                     const double* w, const double* hxU, const double* hyV, const double* hzW, const double* density,
                     double tau, const double* border, double* rhs, int64_t* bad) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int64_t sv1 = (int64_t)(n2 - 1) * n3, sw1 = (int64_t)n2 * (n3 - 1), sw2 = n3 - 1;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t c = i * s1 + j * s2 + k;
        const int mijk = codes[c];
        if (mijk == 0) {
          rhs[c] = 0;
        } else if (mijk == 1) {
          if (i < 1 || i > n1 - 2 || j < 1 || j > n2 - 2 || k < 1 || k > n3 - 2) {
            *bad = c;
            return XFO_ERR_MASK;
          }
          double u_i_1 = u[(i - 1) * s1 + j * s2 + k], u_i = u[i * s1 + j * s2 + k];
          double v_j_1 = v[i * sv1 + (j - 1) * s2 + k], v_j = v[i * sv1 + j * s2 + k];
          double w_k_1 = w[i * sw1 + j * sw2 + k - 1], w_k = w[i * sw1 + j * sw2 + k];
          double d = density ? density[c] : 1.0;
          double div_ = d * d * ((u_i - u_i_1) / hxU[i - 1]) + ((v_j - v_j_1) / hyV[j - 1]) +
                        ((w_k - w_k_1) / hzW[k - 1]);
          rhs[c] = -(div_ / tau);
        } else if (mijk == 4) {
          rhs[c] = border ? border[c] : 0.0;
        } else {   /* not implemented for this border type / unknown code: the reference throws */
          *bad = c;
          return XFO_ERR_MASK;
        }
      }
  return XFO_OK;
}

/* Velocity correction of one component, XProblem.cpp:5598-5777: pass 1 over
 * every cell but PreDefined, pass 2 over PreDefined cells. */
int xfo_velocity_correct(int axis, const int32_t* codes, int b1, int b2, int b3, const double* prev, const double* p,
                         const double* hP, const double* density, double tau, const double* border, double* cur,
                         int64_t* bad) {
  const int64_t s1 = (int64_t)b2 * b3, s2 = b3;
  const int p2 = axis == 2 ? b2 + 1 : b2, p3 = axis == 3 ? b3 + 1 : b3;
  const int64_t ps1 = (int64_t)p2 * p3, ps2 = p3;
  for (int pass = 1; pass < 3; pass++)
    for (int i = 0; i < b1; i++)
      for (int j = 0; j < b2; j++)
        for (int k = 0; k < b3; k++) {
          const int64_t c = i * s1 + j * s2 + k;
          const int mijk = codes[c];
          if (pass == 1 && mijk == 4) continue;
          if (pass == 2 && mijk != 4) continue;
          if (mijk == 0) {
            cur[c] = 0;
          } else if (mijk == 1 || mijk == 5 || mijk == 7) {
            const int64_t cp = i * ps1 + j * ps2 + k;
            double gradP;
            if (axis == 1) gradP = (p[cp + ps1] - p[cp]) / hP[i];
            else if (axis == 2) gradP = (p[cp + ps2] - p[cp]) / hP[j];
            else gradP = (p[cp + 1] - p[cp]) / hP[k];
            cur[c] = prev[c] - tau * gradP / (density ? density[cp] : 1.0);
          } else if (mijk == 3) {
            double defVal = border ? border[c] : 0.0;
            if (prev[c] != defVal) {
              *bad = c;
              return XFO_ERR_CHECK;
            }
            cur[c] = defVal;
          } else if (mijk == 4) {
            double defVal = border ? border[c] : 0.0;
            int64_t nb = -1;
            int count = 0;
            for (int dir = 1; dir < 4; dir++)
              for (int sign = 0; sign < 2; sign++) {
                int shift = -1 + sign * 2;
                int ii = i, jj = j, kk = k;
                if (dir == 1) ii = i + shift;
                else if (dir == 2) jj = j + shift;
                else kk = k + shift;
                if (ii >= 0 && ii < b1 && jj >= 0 && jj < b2 && kk >= 0 && kk < b3 &&
                    codes[ii * s1 + jj * s2 + kk] == 1) {
                  nb = ii * s1 + jj * s2 + kk;
                  count++;
                }
              }
            if (count != 1) {
              *bad = c;
              return XFO_ERR_MASK;
            }
            double check = fabs(prev[c] - (2 * defVal - prev[nb]));
            if (check > 1e-10) {
              *bad = c;
              return XFO_ERR_CHECK;
            }
            cur[c] = 2 * defVal - cur[nb];
          } else {
            *bad = c;
            return XFO_ERR_MASK;
          }
        }
  return XFO_OK;
}

/* Control balance, XProblem.cpp:5782-5829. */
double xfo_divergence_max(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                          const double* w, const double* hxU, const double* hyV, const double* hzW, int32_t* ijk) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  const int64_t sv1 = (int64_t)(n2 - 1) * n3, sw1 = (int64_t)n2 * (n3 - 1), sw2 = n3 - 1;
  double divMaxValue = 0;
  ijk[0] = ijk[1] = ijk[2] = -1;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        if (codes[i * s1 + j * s2 + k] != 1) continue;
        double div = ((u[i * s1 + j * s2 + k] - u[(i - 1) * s1 + j * s2 + k]) / hxU[i - 1]) +
                     ((v[i * sv1 + j * s2 + k] - v[i * sv1 + (j - 1) * s2 + k]) / hyV[j - 1]) +
                     ((w[i * sw1 + j * sw2 + k] - w[i * sw1 + j * sw2 + k - 1]) / hzW[k - 1]);
        if (fabs(div) > divMaxValue) {
          divMaxValue = fabs(div);
          ijk[0] = i;
          ijk[1] = j;
          ijk[2] = k;
        }
      }
  return divMaxValue;
}

/* Momentum right-hand side of velocity component `axis` (1 u, 2 v, 3 w) on
 * its own b1 x b2 x b3 box, TVPProblem::SolveBySplitting, XProblem.cpp:
 * 5088-5419.  Pass 1 (:5088-5305), per cell in i -> j -> k order: Fictive
 * cells zero everything; Actual cells take the transfer velocities averaged
 * onto the component's nodes (:5108-5133), the face viscosity (the mean of the
 * two pressure-box values straddling the node) and rp = 0; Defined and
 * PreDefined cells zero the transfer fields and take rp = border; Normal cells
 * do the same for axis 1 with a normal along x only (:5157-5170) and throw
 * otherwise; Equation, PreNormal, PreEquation and unknown codes throw.  Pass 2
 * (:5310-5350): rp = force on Actual cells (GetForce; NULL is the base class's
 * zero force).  Pass 3 (:5352-5419): on Actual cells rp += dVis . (dVel + dU),
 * central differences over (h[m] + h[m-1]) of the pass-1 fields.  Boxes: u
 * (n1-1) x n2 x n3, v n1 x (n2-1) x n3, w n1 x n2 x (n3-1), vis n1 x n2 x n3
 * for the pressure box n1 x n2 x n3; hx/hy/hz are the component grid's
 * separations.  Returns XFO_OK, or XFO_ERR_MASK with the first throwing cell
 * (or an Actual cell on the box face, where the reference reads outside its
 * arrays) in *bad. */
int xfo_momentum_rhs(int axis, const int32_t* codes, const double* normals, int b1, int b2, int b3,
                     const double* u, const double* v, const double* w, const double* vis, const double* hx,
                     const double* hy, const double* hz, const double* border, const double* force, double* uTr,
                     double* vTr, double* wTr, double* visTr, double* rp, int64_t* bad) {
  if (axis < 1 || axis > 3) return XFO_ERR_ARG;
  const int n2 = b2 + (axis == 2), n3 = b3 + (axis == 3);   /* the pressure box's last two extents */
  const int64_t s1 = (int64_t)b2 * b3, s2 = b3;
  /* strides of the u, v, w and pressure boxes */
  const int64_t us1 = (int64_t)n2 * n3, us2 = n3;
  const int64_t vs1 = (int64_t)(n2 - 1) * n3, vs2 = n3;
  const int64_t ws1 = (int64_t)n2 * (n3 - 1), ws2 = n3 - 1;
  const int64_t ps1 = (int64_t)n2 * n3, ps2 = n3;
#define U_(i, j, k) u[(int64_t)(i) * us1 + (int64_t)(j) * us2 + (k)]
#define V_(i, j, k) v[(int64_t)(i) * vs1 + (int64_t)(j) * vs2 + (k)]
#define W_(i, j, k) w[(int64_t)(i) * ws1 + (int64_t)(j) * ws2 + (k)]
#define P_(i, j, k) vis[(int64_t)(i) * ps1 + (int64_t)(j) * ps2 + (k)]
  for (int i = 0; i < b1; i++)
    for (int j = 0; j < b2; j++)
      for (int k = 0; k < b3; k++) {
        const int64_t c = i * s1 + j * s2 + k;
        const int mijk = codes[c];
        if (mijk == 0) {
          uTr[c] = 0; vTr[c] = 0; wTr[c] = 0; rp[c] = 0; visTr[c] = 0;
        } else if (mijk == 1) {
          if (i < 1 || i > b1 - 2 || j < 1 || j > b2 - 2 || k < 1 || k > b3 - 2) {
            *bad = c;
            return XFO_ERR_MASK;
          }
          if (axis == 1) {
            uTr[c] = U_(i, j, k);
            vTr[c] = (V_(i, j, k) + V_(i + 1, j, k) + V_(i, j - 1, k) + V_(i + 1, j - 1, k)) / 4;
            wTr[c] = (W_(i, j, k) + W_(i + 1, j, k) + W_(i, j, k - 1) + W_(i + 1, j, k - 1)) / 4;
            visTr[c] = vis ? (P_(i, j, k) + P_(i + 1, j, k)) / 2 : 0.0;
          } else if (axis == 2) {
            uTr[c] = (U_(i, j, k) + U_(i, j + 1, k) + U_(i - 1, j, k) + U_(i - 1, j + 1, k)) / 4;
            vTr[c] = V_(i, j, k);
            wTr[c] = (W_(i, j, k) + W_(i, j + 1, k) + W_(i, j, k - 1) + W_(i, j + 1, k - 1)) / 4;
            visTr[c] = vis ? (P_(i, j, k) + P_(i, j + 1, k)) / 2 : 0.0;
          } else {
            uTr[c] = (U_(i, j, k) + U_(i, j, k + 1) + U_(i - 1, j, k) + U_(i - 1, j, k + 1)) / 4;
            vTr[c] = (V_(i, j, k) + V_(i, j, k + 1) + V_(i, j - 1, k) + V_(i, j - 1, k + 1)) / 4;
            wTr[c] = W_(i, j, k);
            visTr[c] = vis ? (P_(i, j, k) + P_(i, j, k + 1)) / 2 : 0.0;
          }
          rp[c] = 0;
        } else if (mijk == 3 || mijk == 4) {
          uTr[c] = 0; vTr[c] = 0; wTr[c] = 0; visTr[c] = 0;
          rp[c] = border ? border[c] : 0.0;
        } else if (mijk == 5) {
          const double nx = normals ? normals[3 * c] : 0.0, ny = normals ? normals[3 * c + 1] : 0.0,
                       nz = normals ? normals[3 * c + 2] : 0.0;
          uTr[c] = 0; vTr[c] = 0; wTr[c] = 0; visTr[c] = 0;
          if (axis != 1 || nx == 0 || ny != 0 || nz != 0) {
            *bad = c;
            return XFO_ERR_MASK;
          }
          rp[c] = border ? border[c] : 0.0;
        } else {   /* Equation, PreNormal, PreEquation: not implemented; else unknown */
          *bad = c;
          return XFO_ERR_MASK;
        }
      }
#undef U_
#undef V_
#undef W_
#undef P_
  for (int64_t c = 0; c < (int64_t)b1 * b2 * b3; c++)
    if (codes[c] == 1) rp[c] = force ? force[c] : 0.0;
  for (int i = 0; i < b1; i++)
    for (int j = 0; j < b2; j++)
      for (int k = 0; k < b3; k++) {
        const int64_t c = i * s1 + j * s2 + k;
        if (codes[c] != 1) continue;
        const double ddx = hx[i] + hx[i - 1], ddy = hy[j] + hy[j - 1], ddz = hz[k] + hz[k - 1];
        const double dVisX = (visTr[c + s1] - visTr[c - s1]) / ddx;
        const double dVisY = (visTr[c + s2] - visTr[c - s2]) / ddy;
        const double dVisZ = (visTr[c + 1] - visTr[c - 1]) / ddz;
        const int64_t st = axis == 1 ? s1 : axis == 2 ? s2 : 1;
        const double dd = axis == 1 ? ddx : axis == 2 ? ddy : ddz;
        const double dU = (uTr[c + st] - uTr[c - st]) / dd;
        const double dV = (vTr[c + st] - vTr[c - st]) / dd;
        const double dW = (wTr[c + st] - wTr[c - st]) / dd;
        const double* velTr = axis == 1 ? uTr : axis == 2 ? vTr : wTr;
        const double dVelX = (velTr[c + s1] - velTr[c - s1]) / ddx;
        const double dVelY = (velTr[c + s2] - velTr[c - s2]) / ddy;
        const double dVelZ = (velTr[c + 1] - velTr[c - 1]) / ddz;
        rp[c] = rp[c] + (dVisX * (dVelX + dU) + dVisY * (dVelY + dV) + dVisZ * (dVelZ + dW));
      }
  return XFO_OK;
}

/* ------------------------------------------------------------------------ */
/* T1dPackOperator (XOperator.cpp:1135-1350) over the Rn space of the
 * operator's grid.  Column j of A is A(e_j) evaluated by the operator itself
 * (xfo_apply), read on the rows of j's activity-table entry (the cell, then
 * its space neighbours at i-1, i+1, j-1, j+1, k-1, k+1:
 * T3dLaplaceOperator::ConstructActivityTables, XOperator.cpp:837-936) and kept
 * where nonzero; that is the transposed storage.  Row i of the original
 * storage looks its entries up in the columns of i's activity-table entry, in
 * that order (:1290-1322).  ptr has R+1 entries, cols/vals up to 7R; returns
 * nnz, or -1 on a grid the operator rejects. */
static int pack_pattern(const uint8_t* sm, const int32_t* inv, int n1, int n2, int n3, int i, int j, int k,
                        int32_t* out) {
  const int di[7] = {0, -1, 1, 0, 0, 0, 0}, dj[7] = {0, 0, 0, -1, 1, 0, 0}, dk[7] = {0, 0, 0, 0, 0, -1, 1};
  int cnt = 0;
  for (int s = 0; s < 7; s++) {
    int a = i + di[s], b = j + dj[s], c = k + dk[s];
    if (a < 0 || a >= n1 || b < 0 || b >= n2 || c < 0 || c >= n3) continue;
    int64_t q = ((int64_t)a * n2 + b) * n3 + c;
    if (sm[q]) out[cnt++] = inv[q] - 1;
  }
  return cnt;
}

int64_t xfo_pack_build(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                       const double* hz, const double* density, int n1, int n2, int n3, int32_t* a_ptr,
                       int32_t* a_cols, double* a_vals, int32_t* t_ptr, int32_t* t_cols, double* t_vals) {
  const int64_t n = (int64_t)n1 * n2 * n3;
  uint8_t* sm = (uint8_t*)malloc((size_t)n);
  xfo_space_mask(codes, n, sm);
  int32_t* inv = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  int32_t* fwd = (int32_t*)malloc((size_t)n * 3 * sizeof(int32_t));
  const int64_t R = xfo_rn_map(sm, n1, n2, n3, inv, fwd);
  double* e = (double*)calloc((size_t)n, sizeof(double));
  double* y = (double*)calloc((size_t)n, sizeof(double));
  int32_t pat[7];
  int64_t nnz = 0;
  t_ptr[0] = 0;
  for (int64_t col = 0; col < R; col++) {
    const int i = fwd[3 * col], j = fwd[3 * col + 1], k = fwd[3 * col + 2];
    const int64_t c = ((int64_t)i * n2 + j) * n3 + k;
    e[c] = 1;
    if (xfo_apply(op, codes, normals, hx, hy, hz, density, n1, n2, n3, e, NULL, 0, y) != XFO_OK) {
      nnz = -1;
      break;
    }
    e[c] = 0;
    const int cnt = pack_pattern(sm, inv, n1, n2, n3, i, j, k, pat);
    for (int s = 0; s < cnt; s++) {
      const int row = pat[s];
      const int64_t rc = ((int64_t)fwd[3 * row] * n2 + fwd[3 * row + 1]) * n3 + fwd[3 * row + 2];
      if (y[rc] != 0) {
        t_cols[nnz] = row;
        t_vals[nnz] = y[rc];
        nnz++;
      }
    }
    t_ptr[col + 1] = (int32_t)nnz;
  }
  if (nnz >= 0) {
    int64_t m = 0;
    a_ptr[0] = 0;
    for (int64_t row = 0; row < R; row++) {
      const int cnt = pack_pattern(sm, inv, n1, n2, n3, fwd[3 * row], fwd[3 * row + 1], fwd[3 * row + 2], pat);
      for (int s = 0; s < cnt; s++) {
        const int col = pat[s];
        double value = 0;
        for (int q = t_ptr[col]; q < t_ptr[col + 1]; q++)
          if (t_cols[q] == row) { value = t_vals[q]; break; }
        if (value != 0) {
          a_cols[m] = col;
          a_vals[m] = value;
          m++;
        }
      }
      a_ptr[row + 1] = (int32_t)m;
    }
  }
  free(sm); free(inv); free(fwd); free(e); free(y);
  return nnz;
}

/* T1dPackOperator::operator() (XOperator.cpp:1550-1571): the row dot in
 * storage order. */
void xfo_pack_apply(int64_t R, const int32_t* ptr, const int32_t* cols, const double* vals, const double* x,
                    double* y) {
  for (int64_t r = 0; r < R; r++) {
    double res = 0;
    for (int q = ptr[r]; q < ptr[r + 1]; q++) res = res + (vals[q]) * (x[cols[q]]);
    y[r] = res;
  }
}

static double dot1(const double* a, const double* b, int64_t R) {
  double res = 0;
  for (int64_t i = 0; i < R; i++) res = res + a[i] * b[i];
  return res;
}

/* TSLAE::SolveByBiConjugateGradients (XSLAE.cpp:159-348) on a packed system:
 * x starts at 0 whatever x0 holds (:171); stop when ||r||_2 <= eps (1e-8 when
 * eps <= 0, :166); a zero beta numerator or denominator is the reference's
 * throw (XFO_ERR_CHECK here, :274-275). */
int xfo_bicg_reference(int64_t R, const int32_t* a_ptr, const int32_t* a_cols, const double* a_vals,
                       const int32_t* t_ptr, const int32_t* t_cols, const double* t_vals, const double* b, double eps,
                       int maxit, double* result, xfo_stats* st) {
  if (eps <= 0) eps = 1e-8;
  double *xk = zeros(R), *xk_new = zeros(R), *rk = zeros(R), *rt = zeros(R), *rk_new = zeros(R);
  double *rt_new = zeros(R), *pk = zeros(R), *pt = zeros(R), *pk_new = zeros(R), *pt_new = zeros(R);
  double* Ap = zeros(R);
  int status = XFO_OK;
  xfo_pack_apply(R, a_ptr, a_cols, a_vals, xk, rk);
  for (int64_t i = 0; i < R; i++) rk[i] = rk[i] - b[i];        /* rk |= A(xk) - b */
  for (int64_t i = 0; i < R; i++) rt[i] = (-1) * rk[i];        /* rt |= (-1)*rk   */
  for (int64_t i = 0; i < R; i++) rk[i] = rt[i];
  memcpy(pk, rk, (size_t)R * 8);
  memcpy(pt, rt, (size_t)R * 8);
  double rkXrk = dot1(rk, rk, R);
  double epsCur = sqrt(rkXrk);
  int it = 0;
  st->status = 0;
  while (epsCur > eps) {
    if (maxit > 0 && it >= maxit) { st->status = 13; break; }
    ++it;
    double alpha1 = dot1(rk, rt, R);
    xfo_pack_apply(R, a_ptr, a_cols, a_vals, pk, Ap);
    double alpha2 = dot1(Ap, pt, R);
    double alpha = alpha1 / alpha2;
    for (int64_t i = 0; i < R; i++) xk_new[i] = xk[i] + alpha * pk[i];
    for (int64_t i = 0; i < R; i++) rk_new[i] = (-alpha) * Ap[i] + rk[i];
    xfo_pack_apply(R, t_ptr, t_cols, t_vals, pt, rt_new);
    for (int64_t i = 0; i < R; i++) rt_new[i] = (-alpha) * rt_new[i] + rt[i];
    double beta1 = dot1(rk_new, rt_new, R);
    double beta2 = dot1(rk, rt, R);
    if (beta1 == 0 || beta2 == 0) { status = XFO_ERR_CHECK; break; }
    double beta = beta1 / beta2;
    for (int64_t i = 0; i < R; i++) pk_new[i] = rk_new[i] + beta * pk[i];
    for (int64_t i = 0; i < R; i++) pt_new[i] = rt_new[i] + beta * pt[i];
    memcpy(xk, xk_new, (size_t)R * 8);
    memcpy(rk, rk_new, (size_t)R * 8);
    memcpy(rt, rt_new, (size_t)R * 8);
    memcpy(pk, pk_new, (size_t)R * 8);
    memcpy(pt, pt_new, (size_t)R * 8);
    rkXrk = dot1(rk, rk, R);
    epsCur = sqrt(rkXrk);
  }
  memcpy(result, xk, (size_t)R * 8);
  st->iterations = it;
  st->resid = epsCur;
  free(xk); free(xk_new); free(rk); free(rt); free(rk_new); free(rt_new); free(pk); free(pt); free(pk_new);
  free(pt_new); free(Ap);
  return status;
}

/* ------------------------------------------------------------------------ */
/* Implicit advection-diffusion operator of the momentum / transport
 * equations: on Actual cells the sum over x, y, z of the reference's ADI line
 * coefficients (THydrodynamicsProblem, XProblem.cpp:1236-1238), after
 * (1/tau) f_c, in the reference's operation order; PreDefined / PreNormal rows
 * as the Laplace operator's.  vel[d] is the advecting component along d at the
 * cell; flags bit 0 convective, bit 1 diffusive. */
/* One direction's implicit line coefficients of the split transfer equation
 * at an Actual point, central scheme (SolveTransferEquation__,
 * XProblem.cpp:3179-3184, schemeType 0) without the 1/tau of B. */
static void ad_coeffs(const double* h, int m, double vd, double D, double conv, double diff, double* A, double* B,
                      double* C) {
  double h_1 = h[m - 1], hh = h[m];
  double hx2 = h[m - 1] + h[m];
  double hxhxh = h[m - 1] * h[m] * (h[m - 1] + h[m]) / 2;
  *A = conv * (0.5 * (-vd / hx2)) + diff * (0.5 * (-(D)*hh / hxhxh));
  *B = diff * (0.5 * (D)*hx2 / hxhxh);
  *C = conv * (0.5 * (vd / hx2)) + diff * (0.5 * (-(D)*h_1 / hxhxh));
}

/* The upwind form of the same coefficients (SolveTransferEquation_, schemeType
 * 1, XProblem.cpp:1828-1843: the concentration's scheme), the 1/tau of b
 * excluded: the convective term takes the upstream neighbour by the sign of
 * vd, with the spacing hx[m] on either side as the reference writes it.  B is
 * returned as its two terms (convective, diffusive) so that b = 1/tau + Bc + Bd
 * can be formed in the reference's order. */
static void ad_coeffs_upwind(const double* h, int m, double vd, double D, double conv, double diff, double* A,
                             double* Bc, double* Bd, double* C) {
  double h_1 = h[m - 1], hh = h[m];
  double hx2 = h[m - 1] + h[m];
  double hxhxh = h[m - 1] * h[m] * (h[m - 1] + h[m]) / 2;
  if (vd < 0) {
    *A = diff * (0.5 * (-(D)*hh / hxhxh));
    *Bc = conv * (0.5 * (-vd / hh));
    *C = conv * (0.5 * (vd / hh)) + diff * (0.5 * (-(D)*h_1 / hxhxh));
  } else {
    *A = conv * (0.5 * (-vd / hh)) + diff * (0.5 * (-(D)*hh / hxhxh));
    *Bc = conv * (0.5 * (vd / hh));
    *C = diff * (0.5 * (-(D)*h_1 / hxhxh));
  }
  *Bd = diff * (0.5 * (D)*hx2 / hxhxh);
}

static double ad_dir(const double* h, int m, double vd, double D, double conv, double diff, double fm, double fc,
                     double fp) {
  double A, B, C;
  ad_coeffs(h, m, vd, D, conv, diff, &A, &B, &C);
  return A * fm + B * fc + C * fp;
}
static double ad_dir_upwind(const double* h, int m, double vd, double D, double conv, double diff, double fm,
                            double fc, double fp) {
  double A, Bc, Bd, C;
  ad_coeffs_upwind(h, m, vd, D, conv, diff, &A, &Bc, &Bd, &C);
  return A * fm + (Bc + Bd) * fc + C * fp;
}

/* The concentration's upwind line coefficients at every Actual point
 * (SolveTransferEquation_ with schemeType 1, XProblem.cpp:1828-1843): a,
 * b = 1/tau + convective + diffusive part (in the reference's order), c;
 * other points untouched. */
void xfo_adi_upwind_coeffs(int dir, const int32_t* codes, int n1, int n2, int n3, const double* hx,
                           const double* hy, const double* hz, const double* vecTr, double D, double tau, double* a,
                           double* b, double* c) {
  const double* h = dir == 1 ? hx : dir == 2 ? hy : hz;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
        if (codes[q] != ACT) continue;
        const int m = dir == 1 ? i : dir == 2 ? j : k;
        double A, Bc, Bd, C;
        ad_coeffs_upwind(h, m, vecTr[q], D, 1.0, 1.0, &A, &Bc, &Bd, &C);
        a[q] = A;
        b[q] = 1 / tau + Bc + Bd;
        c[q] = C;
      }
}

/* The concentration equation's transfer terms on its grid (the loop of
 * TVPProblem::SolveBySplitting, XProblem.cpp:5886-5935): Actual points take
 * the averages of the two staggered velocities around them, PreDefined
 * points on the inlet face (i = 0) the inlet value (inlet[] or 0), every
 * other term 0.  Returns 0; 1 at the first point of a type the reference
 * throws on, 2 at an Actual point on the box face (*bad its flat index). */
int xfo_conc_transfer(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                      const double* w, const double* inlet, double* uTr, double* vTr, double* wTr, double* rpTr,
                      int64_t* bad) {
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
        const int m = codes[q];
        uTr[q] = vTr[q] = wTr[q] = rpTr[q] = 0;
        if (m == ACT) {
          if (i < 1 || i > n1 - 2 || j < 1 || j > n2 - 2 || k < 1 || k > n3 - 2) {
            *bad = q;   /* the reference would read outside the velocity boxes */
            return 2;
          }
          /* u box (n1-1) x n2 x n3, v n1 x (n2-1) x n3, w n1 x n2 x (n3-1) */
          const double* ub = u + ((int64_t)(i - 1) * n2 + j) * n3 + k;
          const double* vb = v + ((int64_t)i * (n2 - 1) + (j - 1)) * n3 + k;
          const double* wb = w + ((int64_t)i * n2 + j) * (n3 - 1) + (k - 1);
          uTr[q] = (ub[0] + ub[(int64_t)n2 * n3]) / 2;
          vTr[q] = (vb[0] + vb[n3]) / 2;
          wTr[q] = (wb[0] + wb[1]) / 2;
        } else if (m == 4) {   /* PreDefined */
          if (i == 0 && inlet) rpTr[q] = inlet[q];
        } else if (m != 0 && m != 6) {
          *bad = q;
          return 1;
        }
      }
  return 0;
}

/* The line systems of the split transfer equation as the reference builds
 * them for every Actual point of a box (SolveTransferEquation__,
 * XProblem.cpp:3149-3190 and 3192-3276, central scheme): for direction
 * dir (1 x, 2 y, 3 z) the coefficients a, b = 1/tau + (diffusion part), c
 * with vecTr the transfer velocity along dir and D the point's diffusion
 * coefficient (diffCoefVar); and, for the x lines of the first splitting
 * step (the only sweep whose right-hand side reads f_1 alone), the
 * right-hand side f.  Other points are left untouched. */
void xfo_adi_line_coeffs(int dir, const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                         const double* hz, const double* vecTr, const double* D, double tau, double* a, double* b,
                         double* c) {
  const double* h = dir == 1 ? hx : dir == 2 ? hy : hz;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
        if (codes[q] != ACT) continue;
        const int m = dir == 1 ? i : dir == 2 ? j : k;
        double A, B, C;
        ad_coeffs(h, m, vecTr[q], D[q], 1.0, 1.0, &A, &B, &C);
        a[q] = A;
        b[q] = 1 / tau + B;
        c[q] = C;
      }
}

void xfo_adi_first_rhs(const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                       const double* hz, const double* f_1, const double* u, const double* v, const double* w,
                       const double* D, const double* rp, double tau, double* f) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
        if (codes[q] != ACT) continue;
        const double hX = hx[i], h_1X = hx[i - 1], hx2X = hx[i - 1] + hx[i];
        const double hxhxhX = hx[i - 1] * hx[i] * (hx[i - 1] + hx[i]) / 2;
        const double hY = hy[j], h_1Y = hy[j - 1], hx2Y = hy[j - 1] + hy[j];
        const double hxhxhY = hy[j - 1] * hy[j] * (hy[j - 1] + hy[j]) / 2;
        const double hZ = hz[k], h_1Z = hz[k - 1], hx2Z = hz[k - 1] + hz[k];
        const double hxhxhZ = hz[k - 1] * hz[k] * (hz[k - 1] + hz[k]) / 2;
        const double dc = D[q];
        double F = (1 / tau) * f_1[q] + rp[q];
        F = F + (0.5 * (-u[q]) * (f_1[q + s1] - f_1[q - s1]) / hx2X);
        F = F + (0.5 * (dc) * ((hX * f_1[q - s1] - hx2X * f_1[q] + h_1X * f_1[q + s1]) / hxhxhX));
        double FC = 0, FD = 0;
        for (int item = 1; item <= 2; item++) {   /* both items read f_1 in the first step */
          FC = FC + 0.5 * (-v[q]) * (f_1[q + s2] - f_1[q - s2]) / hx2Y;
          FD = FD + 0.5 * (dc) * ((hY * f_1[q - s2] - hx2Y * f_1[q] + h_1Y * f_1[q + s2]) / hxhxhY);
        }
        F = F + FC + FD;
        FC = 0;
        FD = 0;
        for (int item = 1; item <= 2; item++) {
          FC = FC + 0.5 * (-w[q]) * (f_1[q + 1] - f_1[q - 1]) / hx2Z;
          FD = FD + 0.5 * (dc) * ((hZ * f_1[q - 1] - hx2Z * f_1[q] + h_1Z * f_1[q + 1]) / hxhxhZ);
        }
        F = F + FC + FD;
        f[q] = F;
      }
}

/* The same first-direction right-hand side in the upwind form (schemeType 1,
 * XProblem.cpp:1857-1912): each convective difference is the one-sided
 * difference toward the upstream neighbour over hx[m]. */
static double up_diff(double vel, double fm, double fc, double fp, double h) {
  return vel < 0 ? 0.5 * (-vel) * (fp - fc) / h : 0.5 * (-vel) * (fc - fm) / h;
}
void xfo_adi_first_rhs_upwind(const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                              const double* hz, const double* f_1, const double* u, const double* v,
                              const double* w, double dc, const double* rp, double tau, double* f) {
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
        if (codes[q] != ACT) continue;
        const double hX = hx[i], h_1X = hx[i - 1], hx2X = hx[i - 1] + hx[i];
        const double hxhxhX = hx[i - 1] * hx[i] * (hx[i - 1] + hx[i]) / 2;
        const double hY = hy[j], h_1Y = hy[j - 1], hx2Y = hy[j - 1] + hy[j];
        const double hxhxhY = hy[j - 1] * hy[j] * (hy[j - 1] + hy[j]) / 2;
        const double hZ = hz[k], h_1Z = hz[k - 1], hx2Z = hz[k - 1] + hz[k];
        const double hxhxhZ = hz[k - 1] * hz[k] * (hz[k - 1] + hz[k]) / 2;
        double F = (1 / tau) * f_1[q] + rp[q];
        F = F + up_diff(u[q], f_1[q - s1], f_1[q], f_1[q + s1], hX);
        F = F + (0.5 * (dc) * ((hX * f_1[q - s1] - hx2X * f_1[q] + h_1X * f_1[q + s1]) / hxhxhX));
        double FC = 0, FD = 0;
        for (int item = 1; item <= 2; item++) {   /* both items read f_1 in the first step */
          FC = FC + up_diff(v[q], f_1[q - s2], f_1[q], f_1[q + s2], hY);
          FD = FD + 0.5 * (dc) * ((hY * f_1[q - s2] - hx2Y * f_1[q] + h_1Y * f_1[q + s2]) / hxhxhY);
        }
        F = F + FC + FD;
        FC = 0;
        FD = 0;
        for (int item = 1; item <= 2; item++) {
          FC = FC + up_diff(w[q], f_1[q - 1], f_1[q], f_1[q + 1], hZ);
          FD = FD + 0.5 * (dc) * ((hZ * f_1[q - 1] - hx2Z * f_1[q] + h_1Z * f_1[q + 1]) / hxhxhZ);
        }
        F = F + FC + FD;
        f[q] = F;
      }
}

int xfo_apply_advdiff(const int32_t* codes, const double* normals, const double* hx, const double* hy,
                      const double* hz, const double* u, const double* v, const double* w, double tau, double D,
                      const double* Dfield, int flags, int n1, int n2, int n3, const double* x, double* y) {
  int64_t bad;
  if (xfo_validate(XFO_OP_LAPLACE, codes, normals, n1, n2, n3, &bad) != XFO_OK) return XFO_ERR_MASK;
  xfo_grid g = {n1, n2, n3, (int64_t)n2 * n3, n3, codes, normals, hx, hy, hz, NULL};
  const double conv = (flags & 1) ? 1.0 : 0.0, diff = (flags & 2) ? 1.0 : 0.0, itau = 1 / tau;
  const int64_t s1 = g.s1, s2 = g.s2;
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        int64_t c = ((int64_t)i * n2 + j) * n3 + k;
        if (!active(codes, c)) continue;
        if (codes[c] != ACT) {
          y[c] = lap_row(&g, x, i, j, k);
          continue;
        }
        const double fc = x[c];
        const double Dc = Dfield ? Dfield[c] : D;   /* diffCoefVar[i][j][k], XProblem.cpp:3204 */
        double res = itau * fc;
        if (flags & 4) {   /* the upwind form */
          res = res + ad_dir_upwind(hx, i, u ? u[c] : 0.0, Dc, conv, diff, x[c - s1], fc, x[c + s1]);
          res = res + ad_dir_upwind(hy, j, v ? v[c] : 0.0, Dc, conv, diff, x[c - s2], fc, x[c + s2]);
          res = res + ad_dir_upwind(hz, k, w ? w[c] : 0.0, Dc, conv, diff, x[c - 1], fc, x[c + 1]);
        } else {
          res = res + ad_dir(hx, i, u ? u[c] : 0.0, Dc, conv, diff, x[c - s1], fc, x[c + s1]);
          res = res + ad_dir(hy, j, v ? v[c] : 0.0, Dc, conv, diff, x[c - s2], fc, x[c + s2]);
          res = res + ad_dir(hz, k, w ? w[c] : 0.0, Dc, conv, diff, x[c - 1], fc, x[c + 1]);
        }
        y[c] = res;
      }
  return XFO_OK;
}

/* VTK legacy ASCII volume of one time step, XProblem.cpp:6132-6345, with the
 * reference's format strings and loops (k outer, i inner over node indices
 * 1..N-1 etc.).  Node box (N+1) x (L+1) x (M+1) with codes node_codes;
 * staggered u (N+1)(L+2)(M+2), v (N+2)(L+1)(M+2), w (N+2)(L+2)(M+1);
 * pressure-box fields p, density, conc, vis (N+2)(L+2)(M+2) with the
 * pressure, density and concentration grids' codes (viscosity uses the
 * concentration mask, :6331).  x, y, z: node coordinates.  Returns 0. */
static double xfo_avg8(const int32_t* code, const double* f, int i, int j, int k, int64_t s1, int64_t s2) {
  const int64_t c = i * s1 + j * s2 + k;
  if (code[c] == 0) return 0;
  const int64_t o1 = c + s1, o2 = c + s1 + s2, o3 = c + s1 + 1, o4 = c + s1 + s2 + 1, o5 = c, o6 = c + s2,
                o7 = c + 1, o8 = c + s2 + 1;
  int avr = (int)(code[o1] != 0) + (int)(code[o2] != 0) + (int)(code[o3] != 0) + (int)(code[o4] != 0) +
            (int)(code[o5] != 0) + (int)(code[o6] != 0) + (int)(code[o7] != 0) + (int)(code[o8] != 0);
  double p1 = f[o1], p2 = f[o2], p3 = f[o3], p4 = f[o4], p5 = f[o5], p6 = f[o6], p7 = f[o7], p8 = f[o8];
  return (p1 + p2 + p3 + p4 + p5 + p6 + p7 + p8) / avr;
}

int xfo_vtk_write(const char* path, int N, int L, int M, const int32_t* node_codes, const double* x, const double* y,
                  const double* z, const double* u, const double* v, const double* w, const int32_t* p_codes,
                  const double* p, const int32_t* d_codes, const double* density, const int32_t* c_codes,
                  const double* conc, const double* vis) {
  FILE* f = fopen(path, "w");
  if (!f) return XFO_ERR_ARG;
  const int NML = (N - 1) * (L - 1) * (M - 1);
  const int64_t nb2 = L + 1, nb3 = M + 1;
  const int64_t us1 = (int64_t)(L + 2) * (M + 2), us2 = M + 2;
  const int64_t vs1 = (int64_t)(L + 1) * (M + 2), vs2 = M + 2;
  const int64_t ws1 = (int64_t)(L + 2) * (M + 1), ws2 = M + 1;
  const int64_t ps1 = (int64_t)(L + 2) * (M + 2), ps2 = M + 2;
  fprintf(f, "# vtk DataFile Version 3.0\n");
  fprintf(f, "Flow\nASCII\n\n");
  fprintf(f, "DATASET STRUCTURED_GRID\n");
  fprintf(f, "DIMENSIONS %d %d %d\n", N - 1, L - 1, M - 1);
  fprintf(f, "POINTS %d double\n", NML);
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) fprintf(f, "%f  %f  %f\n", x[i], y[j], z[k]);
  fprintf(f, "POINT_DATA %d\n\nVECTORS Velocity double\n", NML);
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) {
        double uu, vv, ww;
        if (node_codes[(i * nb2 + j) * nb3 + k] == 0) {
          uu = 0; vv = 0; ww = 0;
        } else {
          const int64_t cu = i * us1 + j * us2 + k, cv = i * vs1 + j * vs2 + k, cw = i * ws1 + j * ws2 + k;
          uu = (u[cu] + u[cu + us2] + u[cu + 1] + u[cu + us2 + 1]) / 4;
          vv = (v[cv] + v[cv + vs1] + v[cv + 1] + v[cv + vs1 + 1]) / 4;
          ww = (w[cw] + w[cw + ws1] + w[cw + ws2] + w[cw + ws1 + ws2]) / 4;
        }
        fprintf(f, "%f ", uu);
        fprintf(f, "%f ", vv);
        fprintf(f, "%f\n ", ww);
      }
  fprintf(f, "\nSCALARS Pressure float\nLOOKUP_TABLE default\n");
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) fprintf(f, "%f\n ", xfo_avg8(p_codes, p, i, j, k, ps1, ps2));
  fprintf(f, "\nSCALARS Density float\nLOOKUP_TABLE default\n");
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) fprintf(f, "%f\n", xfo_avg8(d_codes, density, i, j, k, ps1, ps2));
  fprintf(f, "\nSCALARS Concentration float\nLOOKUP_TABLE default\n");
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) fprintf(f, "%f\n", xfo_avg8(c_codes, conc, i, j, k, ps1, ps2));
  fprintf(f, "\nSCALARS Viscosity float\nLOOKUP_TABLE default\n");
  for (int k = 1; k < M; k++)
    for (int j = 1; j < L; j++)
      for (int i = 1; i < N; i++) fprintf(f, "%f\n", xfo_avg8(c_codes, vis, i, j, k, ps1, ps2));
  fclose(f);
  return XFO_OK;
}

/* "%f\n" of each value, concatenated (the C library's formatting); returns
 * the length, writing only when out has room for it. */
int64_t xfo_format_fixed6(const double* values, int64_t n, char* out, int64_t capacity) {
  int64_t len = 0;
  char buf[400];
  for (int64_t q = 0; q < n; q++) {
    int m = snprintf(buf, sizeof(buf), "%f\n", values[q]);
    if (out && len + m <= capacity) memcpy(out + len, buf, (size_t)m);
    len += m;
  }
  return len;
}
