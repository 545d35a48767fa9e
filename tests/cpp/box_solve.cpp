// A C++ caller of the GPU solver with no Python in between: the 32^3
// pressure-type system of a unit cube (Fictive ghost layer: homogeneous
// Neumann walls) with a masked sphere, built and solved through
// xflow_gb300/host/xf_box_system.h over the C ABI, and checked here against
// this file's own restatement of the reference's Laplace rows
// (T3dLaplaceOperator, XOperator.cpp:994-1019: flux form, fluxes toward
// Fictive neighbours zeroed).  Prints one line per solve; exit status 0
// when every check holds.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <random>
#include <vector>

#include "xf_box_system.h"

static const int N = 32, B = N + 2;   // interior cells per axis, box with the ghost layer

static size_t at(int i, int j, int k) { return ((size_t)i * B + j) * B + k; }

// r = b - A x on the Actual cells, as the reference's rows compute A x
static void residual(const std::vector<int32_t>& code, const std::vector<double>& h, const std::vector<double>& x,
                     const std::vector<double>& b, std::vector<double>& r) {
  for (int i = 1; i < B - 1; i++)
    for (int j = 1; j < B - 1; j++)
      for (int k = 1; k < B - 1; k++) {
        const size_t c = at(i, j, k);
        if (code[c] != 1) { r[c] = 0; continue; }
        const size_t nb[6] = {at(i - 1, j, k), at(i + 1, j, k), at(i, j - 1, k), at(i, j + 1, k), at(i, j, k - 1),
                              at(i, j, k + 1)};
        double sum = 0;
        for (int a = 0; a < 3; a++) {
          const double lo = code[nb[2 * a]] == 0 ? 0.0 : (x[c] - x[nb[2 * a]]) / h[0];
          const double hi = code[nb[2 * a + 1]] == 0 ? 0.0 : (x[nb[2 * a + 1]] - x[c]) / h[0];
          sum += (hi - lo) / h[0];
        }
        r[c] = b[c] + sum;   // b - (-laplace x)
      }
}

int main() {
  const size_t n = (size_t)B * B * B;
  std::vector<int32_t> code(n, 0);
  std::vector<double> h(B - 1, 1.0 / N), normals(3 * n, 0.0), b(n, 0.0), x(n, 0.0), r(n, 0.0);
  for (int i = 1; i < B - 1; i++)
    for (int j = 1; j < B - 1; j++)
      for (int k = 1; k < B - 1; k++) {
        const double di = i - 12.5, dj = j - 17.0, dk = k - 20.0;
        code[at(i, j, k)] = di * di + dj * dj + dk * dk < 36.0 ? 0 : 1;   // a Fictive sphere of radius 6 cells
      }
  std::mt19937_64 rng(7);
  std::normal_distribution<double> nd(0.0, 1.0);
  double mean = 0, cnt = 0;
  for (size_t c = 0; c < n; c++)
    if (code[c] == 1) { b[c] = nd(rng); mean += b[c]; cnt += 1; }
  mean /= cnt;
  for (size_t c = 0; c < n; c++)
    if (code[c] == 1) b[c] -= mean;   // compatible with the Neumann walls
  double bnorm = 0;
  for (size_t c = 0; c < n; c++) bnorm += b[c] * b[c];
  bnorm = sqrt(bnorm);

  int failures = 0;
  try {
    xflow::BoxSystem sys(0);
    sys.set_grid(B, B, B, code.data(), h.data(), h.data(), h.data(), normals.data(), XF_OP_LAPLACE);
    // mixed-precision CG to a true relative residual of 1e-8
    xf_solve_opts o;
    xf_solve_opts_default(&o);
    o.precision = XF_PREC_MIXED;
    o.rtol = 1e-8;
    xf_solve_stats st = sys.solve(XF_CG, x.data(), b.data(), &o);
    residual(code, h, x, b, r);
    double rn = 0;
    for (size_t c = 0; c < n; c++) rn += r[c] * r[c];
    const double rel = sqrt(rn) / bnorm;
    printf("mixed CG: %d iterations, reported %.3e, host residual %.3e\n", st.iterations, st.rel_resid, rel);
    if (!(rel <= 1.01e-8)) failures++;
    // the time loop's own solver, BiCGStab with its stopping rule ||r||_inf <= 1e-5, warm-started
    for (size_t c = 0; c < n; c++) x[c] = 0.0;
    st = sys.solve(XF_BICGSTAB, x.data(), b.data());
    residual(code, h, x, b, r);
    double rmax = 0;
    for (size_t c = 0; c < n; c++) rmax = fmax(rmax, fabs(r[c]));
    printf("BiCGStab: %d iterations, host max |r| %.3e\n", st.iterations, rmax);
    if (!(rmax <= 1e-5 * (1 + 1e-9))) failures++;
    // the same grid again: kept, not rebuilt; a bad point code throws the reference's way
    xf_op* op = sys.op();
    sys.set_grid(B, B, B, code.data(), h.data(), h.data(), h.data(), normals.data(), XF_OP_LAPLACE);
    if (sys.op() != op) failures++;
    std::vector<int32_t> bad(code);
    bad[at(5, 5, 5)] = 42;
    bool threw = false;
    try {
      sys.set_grid(B, B, B, bad.data(), h.data(), h.data(), h.data(), normals.data(), XF_OP_LAPLACE);
    } catch (const char* msg) {
      threw = true;
      printf("bad code: threw \"%s\"\n", msg);
    }
    if (!threw) failures++;
  } catch (const char* msg) {
    printf("threw: %s\n", msg);
    return 2;
  }
  printf(failures ? "FAILED %d\n" : "OK\n", failures);
  return failures ? 1 : 0;
}
