// The host side of the drop-in for the reference's pressure-path solver:
// one linear system on the GPU behind the reference's own conventions -
// boxes in the reference's [i][j][k] order (k fastest), point codes and
// per-cell normals as its T3dNormalGrid holds them, and every failure
// reported as a thrown `const char*`, the only error channel the reference
// has (caught in main, XFlow.cpp:78-84).  Header only, C++11, over the C ABI
// of include/xflow.h (link libxflow.so).
//
//   xflow::BoxSystem sys;                       // one CUDA context (device 0)
//   sys.set_grid(n1, n2, n3, codes, hx, hy, hz, normals, XF_OP_VARDIV);
//   sys.set_density(rho);                       // T3dVariableDivergentedOperator::withDensity
//   xf_solve_stats st = sys.solve(XF_BICGSTAB, x, b);   // x: initial guess in, result out
//
// set_grid keeps the device grid and operator while the statement is
// unchanged (the same codes, spacings and normals), so a time loop that
// hands the same grid every step builds them once.  Not thread-safe, like
// the reference's operators (XOperator.h:53, 232, 314).
#pragma once
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "xflow.h"

namespace xflow {

class BoxSystem {
 public:
  explicit BoxSystem(int device = 0) {
    if (xf_create(device, &ctx_) != XF_OK) fail("xflow: no CUDA device for the solver");
  }
  ~BoxSystem() {
    release();
    if (ctx_) xf_destroy(ctx_);
  }
  BoxSystem(const BoxSystem&) = delete;
  BoxSystem& operator=(const BoxSystem&) = delete;

  xf_ctx* context() const { return ctx_; }
  xf_op* op() const { return op_; }

  // The grid (T3dNormalGrid: codes, separations, normals: 3 doubles per cell,
  // 0 where the reference holds no normal) and the operator kind
  // (XF_OP_LAPLACE = T3dLaplaceOperator, XF_OP_VARDIV =
  // T3dVariableDivergentedOperator).
  void set_grid(int n1, int n2, int n3, const int32_t* codes, const double* hx, const double* hy, const double* hz,
                const double* normals, int op_kind) {
    const size_t n = (size_t)n1 * n2 * n3;
    std::vector<double> key;
    key.reserve(n / 2 + n1 + n2 + n3 + 8);
    key.push_back(n1); key.push_back(n2); key.push_back(n3); key.push_back(op_kind);
    key.insert(key.end(), hx, hx + n1 - 1);
    key.insert(key.end(), hy, hy + n2 - 1);
    key.insert(key.end(), hz, hz + n3 - 1);
    uint64_t h = 1469598103934665603ull;   // FNV-1a over the codes and normals
    for (size_t c = 0; c < n; c++) h = (h ^ (uint32_t)codes[c]) * 1099511628211ull;
    if (normals)
      for (size_t c = 0; c < 3 * n; c++) {
        uint64_t bits;
        memcpy(&bits, &normals[c], 8);
        h = (h ^ bits) * 1099511628211ull;
      }
    key.push_back((double)(h >> 11));
    if (op_ && key == key_) return;
    release();
    if (xf_grid_create(ctx_, n1, n2, n3, codes, hx, hy, hz, normals, &grid_) != XF_OK) fail_last();
    if (xf_op_create(grid_, op_kind, &op_) != XF_OK) fail_last();
    key_.swap(key);
    ncell_ = n;
  }

  // withDensity (XOperator.cpp:2243-2255): the density box of a variable-density operator.
  void set_density(const double* rho) {
    need_op();
    if (xf_op_set_density(op_, rho) != XF_OK) fail_last();
  }

  // TSLAE(A, x, b) + SolveBy*() + Result: method XF_CG_REFERENCE,
  // XF_BICGSTAB, XF_MINRES (the reference's algorithms and stopping rules) or
  // XF_BICG (on the packed operator, built on first use); any other method
  // of xf_solve (e.g. XF_CG with XF_PREC_MIXED and a relative tolerance)
  // through `base`.  A status other than XF_OK throws, like the reference's
  // breakdown throws; XF_MAXIT can only come from a cap the caller set.
  xf_solve_stats solve(int method, double* x, const double* b, const xf_solve_opts* base = nullptr) {
    need_op();
    xf_solve_opts o;
    if (base) o = *base;
    else xf_solve_opts_default(&o);
    o.method = method;
    xf_op* a = op_;
    if (method == XF_BICG) {
      if (!pack_ && xf_pack_create(op_, &pack_) != XF_OK) fail_last();
      a = pack_;
    }
    xf_solve_stats st;
    if (xf_solve_host(a, &o, x, b, &st) != XF_OK) fail_last();
    if (st.status != XF_OK) fail(xf_status_string(st.status));
    return st;
  }

 private:
  xf_ctx* ctx_ = nullptr;
  xf_grid* grid_ = nullptr;
  xf_op* op_ = nullptr;
  xf_op* pack_ = nullptr;
  std::vector<double> key_;
  size_t ncell_ = 0;
  std::string err_;

  void release() {
    if (pack_) xf_op_destroy(pack_);
    if (op_) xf_op_destroy(op_);
    if (grid_) xf_grid_destroy(grid_);
    pack_ = nullptr; op_ = nullptr; grid_ = nullptr;
    key_.clear();
  }
  void need_op() {
    if (!op_) fail("xflow: BoxSystem::set_grid has not been called");
  }
  // the reference's error convention: throw a C string (kept alive by the object)
  void fail(const char* msg) { throw msg; }
  void fail_last() {
    err_ = std::string("xflow: ") + xf_last_error(ctx_);
    throw err_.c_str();
  }
};

}  // namespace xflow
