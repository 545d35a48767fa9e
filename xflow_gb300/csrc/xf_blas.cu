// Masked vector algebra of TRnRelease3dSpace (XSpace.cpp:2424-3487) on the
// GPU: linear combinations, FP64 inner products and norms, abs-max with its
// Rn index.  Reductions are deterministic: per-block partials in a fixed grid,
// summed in fixed order by the last block.
#include <math.h>

#include "xf_stencil.cuh"

template <typename T>
__global__ void k_lincomb(double p1, const T* __restrict__ s1, double p2, const T* __restrict__ s2,
                          const uint8_t* __restrict__ m, int64_t n, T* __restrict__ z) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (!m[c]) continue;
    T a = s1 ? (T)p1 * s1[c] : T(0);
    z[c] = s2 ? a + (T)p2 * s2[c] : a;
  }
}

template <typename T>
__global__ void k_fill(T v, const uint8_t* __restrict__ m, int64_t n, T* __restrict__ z) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    if (m[c]) z[c] = v;
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot(const T* __restrict__ a, const T* __restrict__ b,
                                                     const uint8_t* __restrict__ m, int64_t n, DevScratch* S, int slot) {
  __shared__ double sh[32];
  __shared__ bool last;
  double acc = 0.0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    if (m[c]) acc += (double)a[c] * (double)b[c];
  double v[1] = {acc};
  if (publish_partials<1>(S, slot, v, sh, &last)) {
    double t = finish_partials(S, slot, sh);
    if (threadIdx.x == 0) { S->scalars[slot] = t; S->tickets[slot] = 0; }
  }
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_absmax(const T* __restrict__ a, const uint8_t* __restrict__ m,
                                                        const int32_t* __restrict__ inv, int64_t n, DevScratch* S,
                                                        int slot) {
  __shared__ AbsMax sh[32];
  __shared__ bool last;
  AbsMax best;
  best.v = 0.0; best.c = -1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (!m[c]) continue;
    double v = fabs((double)a[c]);
    if (v > best.v) { best.v = v; best.c = c; }   // NaN never wins, as in the reference
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
  q.v = 0.0; q.c = -1;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    AbsMax u;
    u.v = __ldcg(&S->partials[slot][b]);
    u.c = (long long)__ldcg(&S->partials[slot + 1][b]);
    q = am_combine(q, u);
  }
  q = am_block(q, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = q.c >= 0 ? q.v : 0.0;
    S->scalars[slot + 1] = q.c >= 0 ? (double)inv[q.c] : 1.0;  // Rn index, 1 when nothing beat 0
    S->tickets[slot] = 0;
  }
}

// ---------------------------------------------------------------------------
static int same_grid(const xf_vec* a, const xf_vec* b, const char* what) {
  if (!a || !b) return XF_ERR_ARG;
  if (a->g != b->g) return xf_fail(a->g->ctx, XF_ERR_STATE, "%s: vectors of different grids", what);
  if (a->dtype != b->dtype) return xf_fail(a->g->ctx, XF_ERR_STATE, "%s: mixed dtypes", what);
  return XF_OK;
}

static int read_scalars(xf_ctx* ctx, int slot, int count, double* out) {
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->scalars[slot], count * 8, cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int q = 0; q < count; q++) out[q] = ctx->host_scalars[q];
  return XF_OK;
}

extern "C" int xf_lincomb(double p1, const xf_vec* s1, double p2, const xf_vec* s2, xf_vec* z) {
  int st;
  if (!z || !s1) return XF_ERR_ARG;
  if ((st = same_grid(s1, z, "xf_lincomb"))) return st;
  if (s2 && (st = same_grid(s2, z, "xf_lincomb"))) return st;
  const xf_grid* g = z->g;
  xf_ctx* ctx = g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int bl = grid_blocks(ctx, g->ncell, 256);
  const bool use2 = s2 && p2 != 0.0;   // XSpace.cpp: p = 0 drops the operand
  if (z->dtype == XF_F64)
    k_lincomb<double><<<bl, 256, 0, ctx->stream>>>(p1, p1 != 0.0 ? (const double*)s1->data : nullptr, p2,
                                                    use2 ? (const double*)s2->data : nullptr, g->smask, g->ncell, (double*)z->data);
  else
    k_lincomb<float><<<bl, 256, 0, ctx->stream>>>(p1, p1 != 0.0 ? (const float*)s1->data : nullptr, p2,
                                                   use2 ? (const float*)s2->data : nullptr, g->smask, g->ncell, (float*)z->data);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_vec_fill(xf_vec* z, double v) {
  if (!z) return XF_ERR_ARG;
  const xf_grid* g = z->g;
  xf_ctx* ctx = g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int bl = grid_blocks(ctx, g->ncell, 256);
  if (z->dtype == XF_F64) k_fill<double><<<bl, 256, 0, ctx->stream>>>(v, g->smask, g->ncell, (double*)z->data);
  else k_fill<float><<<bl, 256, 0, ctx->stream>>>((float)v, g->smask, g->ncell, (float*)z->data);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

void xf_dot_async(const xf_grid* g, int dtype, const void* a, const void* b, int slot) {
  xf_ctx* ctx = g->ctx;
  const int bl = red_blocks(ctx, g->ncell);
  if (dtype == XF_F64)
    k_dot<double><<<bl, RED_THREADS, 0, ctx->stream>>>((const double*)a, (const double*)b, g->smask, g->ncell, ctx->scratch, slot);
  else
    k_dot<float><<<bl, RED_THREADS, 0, ctx->stream>>>((const float*)a, (const float*)b, g->smask, g->ncell, ctx->scratch, slot);
}

void xf_absmax_async(const xf_grid* g, int dtype, const void* a, int slot) {
  xf_ctx* ctx = g->ctx;
  const int bl = red_blocks(ctx, g->ncell);
  if (dtype == XF_F64)
    k_absmax<double><<<bl, RED_THREADS, 0, ctx->stream>>>((const double*)a, g->smask, g->inv, g->ncell, ctx->scratch, slot);
  else
    k_absmax<float><<<bl, RED_THREADS, 0, ctx->stream>>>((const float*)a, g->smask, g->inv, g->ncell, ctx->scratch, slot);
}

extern "C" int xf_dot(const xf_vec* a, const xf_vec* b, double* out) {
  int st;
  if (!out) return XF_ERR_ARG;
  if ((st = same_grid(a, b, "xf_dot"))) return st;
  xf_ctx* ctx = a->g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  xf_dot_async(a->g, a->dtype, a->data, b->data, 0);
  return read_scalars(ctx, 0, 1, out);
}

extern "C" int xf_norm(const xf_vec* a, double* out) {
  double s;
  int st = xf_dot(a, a, &s);
  if (st) return st;
  *out = sqrt(s);
  return XF_OK;
}

extern "C" int xf_absmax(const xf_vec* a, double* out, int64_t* rn_index) {
  if (!a || !out) return XF_ERR_ARG;
  xf_ctx* ctx = a->g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  xf_absmax_async(a->g, a->dtype, a->data, 0);
  double r[2];
  int st = read_scalars(ctx, 0, 2, r);
  if (st) return st;
  *out = r[0];
  if (rn_index) *rn_index = (int64_t)r[1];
  return XF_OK;
}

void xf_apply_f64(const xf_op* op, const double* x, double* y, const double* s, int sign, bool exact,
                  bool zero_inactive, const double* w, int slot);
void xf_apply_f32(const xf_op* op, const float* x, float* y, const float* s, int sign, bool zero_inactive,
                  const float* w, int slot);
int xf_op_ready(const xf_op* op);

// (x, A y): the row values are formed in a scratch box and dotted with x in
// the same pass.
extern "C" int xf_dot_op(xf_op* op, const xf_vec* x, const xf_vec* y, double* out) {
  int st;
  if (!op || !out) return XF_ERR_ARG;
  if ((st = same_grid(x, y, "xf_dot_op"))) return st;
  if (x->g != op->g) return xf_fail(op->g->ctx, XF_ERR_STATE, "xf_dot_op: vectors of another grid");
  if ((st = xf_op_ready(op))) return st;
  xf_ctx* ctx = op->g->ctx;
  if (op->kind == XF_OP_PACK && x->dtype != XF_F64)
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_dot_op: packed operators are FP64");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  void* tmp = nullptr;
  const size_t es = x->dtype == XF_F64 ? 8 : 4;
  XF_CUDA(ctx, cudaMallocAsync(&tmp, op->g->ncell * es, ctx->stream));
  if (x->dtype == XF_F64)
    xf_apply_f64(op, (const double*)y->data, (double*)tmp, nullptr, 0, false, true, (const double*)x->data, 0);
  else
    xf_apply_f32(op, (const float*)y->data, (float*)tmp, nullptr, 0, true, (const float*)x->data, 0);
  XF_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  return read_scalars(ctx, 0, 1, out);
}
