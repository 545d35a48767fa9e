// Operators (T3dLaplaceOperator, T3dVariableDivergentedOperator) and the
// masked matvec y |= A(x) (+/- s) of TRnRelease3dSpace::
// LocalReleaseAssignSpeedLinearCombination(op) (XSpace.cpp:3013-3217).
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

#include "xf_control.cuh"

// y |= A(x) + sign*s (negated when neg), written to y (T) and/or y32 (float);
// fused FP64 dots (w, v) -> slot_w and (v, v) -> slot_self; the last block
// to finish runs the solver control step `ctl`.
template <typename T>
struct MatvecArgs {
  StencilGrid<T> g;
  const T* __restrict__ x;
  T* __restrict__ y;
  float* __restrict__ y32;
  const T* __restrict__ s;
  const T* __restrict__ w;
  int sign, neg, zero_inactive, dot_w, dot_self;
  int slot_w, slot_self, ctl, gate;
  DevScratch* S;
};

// One warp per k-row (i, j): 32 consecutive cells per step, coalesced.
template <typename T, int OP, bool EXACT>
__global__ void __launch_bounds__(256) k_matvec(MatvecArgs<T> a) {
  __shared__ double sh[32];
  __shared__ bool last;
  // Solver kernels turn into no-ops once the solve is done (or, when gated,
  // while no true-residual replacement is pending).
  if (a.ctl != CTL_NONE && (a.S->iscalars[I_DONE] || (a.gate && !a.S->iscalars[I_NEEDREP]))) return;
  const StencilGrid<T>& g = a.g;
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const int nrows = g.n1 * g.n2;
  double dw = 0.0, ds = 0.0;
  for (int r = blockIdx.x * warps + (threadIdx.x >> 5); r < nrows; r += gridDim.x * warps) {
    const int i = r / g.n2, j = r - i * g.n2;
    const int base = r * g.n3;
    for (int k = lane; k < g.n3; k += 32) {
      const int c = base + k;
      const uint8_t kb = g.kind[c];
      if (row_of(kb) == ROW_NONE) {
        if (a.zero_inactive) {
          if (a.y) a.y[c] = T(0);
          if (a.y32) a.y32[c] = 0.f;
        }
        continue;
      }
      T v = apply_row<T, OP, EXACT>(g, a.x, i, j, k, c, kb);
      if (a.sign > 0) v = v + a.s[c];
      else if (a.sign < 0) v = v - a.s[c];
      if (a.neg) v = -v;
      if (a.dot_w) dw += (double)a.w[c] * (double)v;
      if (a.dot_self) ds += (double)v * (double)v;
      if (a.y) a.y[c] = v;
      if (a.y32) a.y32[c] = (float)v;
    }
  }
  if (a.dot_w || a.dot_self || a.ctl != CTL_NONE) {
    double vals[2] = {dw, ds};
    if (publish_partials<2>(a.S, a.slot_w, vals, sh, &last)) {
      double tw = finish_partials(a.S, a.slot_w, sh);
      double ts = finish_partials(a.S, a.slot_w + 1, sh);
      if (threadIdx.x == 0) {
        if (a.dot_w) a.S->scalars[a.slot_w] = tw;
        if (a.dot_self) a.S->scalars[a.slot_self] = ts;
        a.S->tickets[a.slot_w] = 0;
        control_step(a.S, a.ctl);
      }
    }
  }
}

template <typename T>
static void launch_matvec(const xf_op* op, const T* rho, const MvReq<T>& q) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  MatvecArgs<T> a;
  a.g = make_stencil_grid<T>(g, rho);
  a.x = q.x; a.y = q.y; a.y32 = q.y32; a.s = q.s; a.w = q.w;
  a.sign = q.sign; a.neg = q.neg; a.zero_inactive = q.zero_inactive;
  a.dot_w = q.w != nullptr; a.dot_self = q.dot_self;
  // two consecutive partial slots: slot_w and slot_w+1 (self)
  a.slot_w = q.slot; a.slot_self = q.slot + 1; a.ctl = q.ctl; a.gate = q.gate;
  a.S = ctx->scratch;
  const int64_t rows = (int64_t)g->n1 * g->n2;
  int blocks = grid_blocks(ctx, rows * 32, 256, 8);
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  if (op->kind == XF_OP_LAPLACE) {
    if (q.exact) k_matvec<T, XF_OP_LAPLACE, true><<<blocks, 256, 0, ctx->stream>>>(a);
    else k_matvec<T, XF_OP_LAPLACE, false><<<blocks, 256, 0, ctx->stream>>>(a);
  } else {
    if (q.exact) k_matvec<T, XF_OP_VARDIV, true><<<blocks, 256, 0, ctx->stream>>>(a);
    else k_matvec<T, XF_OP_VARDIV, false><<<blocks, 256, 0, ctx->stream>>>(a);
  }
}

void xf_mv64(const xf_op* op, const MvReq<double>& q) { launch_matvec<double>(op, op->rho, q); }
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
  if (!g || !out || (kind != XF_OP_LAPLACE && kind != XF_OP_VARDIV))
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
  xf_op* op = new xf_op();
  op->g = g; op->kind = kind; op->rho = nullptr; op->rho32 = nullptr; op->rho_set = 0;
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

int xf_op_ready(const xf_op* op) {
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
