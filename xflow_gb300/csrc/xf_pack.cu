// Packed operator: T1dPackOperator (XOperator.cpp:1135-1571) on the GPU.
//
// The reference packs an operator column by column, A(e_j) for every Rn index
// j, reading each column on the rows of j's activity-table entry (the cell,
// then its space neighbours at i-1, i+1, j-1, j+1, k-1, k+1:
// T3dLaplaceOperator::ConstructActivityTables, XOperator.cpp:837-936) and
// keeping the nonzero values; its row storage lists, for row i, the nonzero
// A[i][c] for c over i's activity-table entry in that order.  Its apply is the
// row dot in storage order (:1550-1571), and operator~ switches to the column
// storage (A^T).
//
// Here the columns come from 27 probes instead of N: every row of the
// operators reads at most the 3x3x3 cube around its cell, so cells whose
// (i mod 3, j mod 3, k mod 3) agree never meet in one row, and one exact FP64
// matvec of the indicator of such a colour class yields A(e_c)[r] for every
// row r and every cell c of that class in r's pattern, bit for bit (the row
// sees exactly the inputs A(e_c) would give it).
//
// Storage is ELL with 7 slots, slot-major ([slot][row], coalesced across the
// threads of a warp), entries compacted in the reference's order, columns as
// box cells so that the SpMV works on box vectors; rows in Rn order.  The SpMV
// sums res = res + m * x[col] from res = 0 in that order, as the reference.
#include <vector>

#include "xf_control.cuh"

struct PackData {
  int64_t rows = 0, nnz = 0, nnz_t = 0;
  uint8_t* a_cnt = nullptr;   // [rows]
  int32_t* a_col = nullptr;   // [7][rows] box cells
  double* a_val = nullptr;    // [7][rows]
  uint8_t* t_cnt = nullptr;
  int32_t* t_col = nullptr;
  double* t_val = nullptr;
};

void xf_mv64(const xf_op* op, const MvReq<double>& q);

__device__ __forceinline__ int pk_color(int i, int j, int k) { return (i % 3) * 9 + (j % 3) * 3 + (k % 3); }

// Neighbour of slot s (0 self, 1 i-1, 2 i+1, 3 j-1, 4 j+1, 5 k-1, 6 k+1), or -1
// outside the box.
__device__ __forceinline__ int64_t pk_nb(int s, int i, int j, int k, int n1, int n2, int n3, int64_t c, int64_t s1,
                                         int64_t s2) {
  switch (s) {
    case 0: return c;
    case 1: return i > 0 ? c - s1 : -1;
    case 2: return i < n1 - 1 ? c + s1 : -1;
    case 3: return j > 0 ? c - s2 : -1;
    case 4: return j < n2 - 1 ? c + s2 : -1;
    case 5: return k > 0 ? c - 1 : -1;
    default: return k < n3 - 1 ? c + 1 : -1;
  }
}
__device__ __forceinline__ int pk_opp(int s) { return s == 0 ? 0 : ((s & 1) ? s + 1 : s - 1); }

__global__ void k_pack_probe(const uint8_t* __restrict__ sm, int n1, int n2, int n3, int q, double* __restrict__ e) {
  const int64_t n = (int64_t)n1 * n2 * n3, s1 = (int64_t)n2 * n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / s1), j = (int)((c - i * s1) / n3), k = (int)(c - i * s1 - (int64_t)j * n3);
    e[c] = (sm[c] && pk_color(i, j, k) == q) ? 1.0 : 0.0;
  }
}

// v7[s][r] = A(e_nb)[r] for the pattern slots s of row r whose cell has colour q.
__global__ void k_pack_collect(const uint8_t* __restrict__ sm, const int32_t* __restrict__ inv, int n1, int n2,
                               int n3, int q, const double* __restrict__ y, int64_t R, double* __restrict__ v7) {
  const int64_t n = (int64_t)n1 * n2 * n3, s1 = (int64_t)n2 * n3, s2 = n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (!sm[c]) continue;
    const int i = (int)(c / s1), j = (int)((c - i * s1) / s2), k = (int)(c - i * s1 - j * s2);
    const int64_t r = inv[c] - 1;
    for (int s = 0; s < 7; s++) {
      const int64_t nb = pk_nb(s, i, j, k, n1, n2, n3, c, s1, s2);
      if (nb < 0 || !sm[nb]) continue;
      const int ni = (int)(nb / s1), nj = (int)((nb - ni * s1) / s2), nk = (int)(nb - ni * s1 - nj * s2);
      if (pk_color(ni, nj, nk) == q) v7[s * R + r] = y[c];
    }
  }
}

// Compact the row storage and the column (transposed) storage.
__global__ void k_pack_fill(const uint8_t* __restrict__ sm, const int32_t* __restrict__ inv, int n1, int n2, int n3,
                            int64_t R, const double* __restrict__ v7, uint8_t* a_cnt, int32_t* a_col, double* a_val,
                            uint8_t* t_cnt, int32_t* t_col, double* t_val, unsigned long long* empty) {
  const int64_t n = (int64_t)n1 * n2 * n3, s1 = (int64_t)n2 * n3, s2 = n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (!sm[c]) continue;
    const int i = (int)(c / s1), j = (int)((c - i * s1) / s2), k = (int)(c - i * s1 - j * s2);
    const int64_t r = inv[c] - 1;
    int na = 0, nt = 0;
    for (int s = 0; s < 7; s++) {
      const int64_t nb = pk_nb(s, i, j, k, n1, n2, n3, c, s1, s2);
      if (nb < 0 || !sm[nb]) continue;
      const double va = v7[s * R + r];                       // A[r][nb]
      if (va != 0) {
        a_col[na * R + r] = (int32_t)nb;
        a_val[na * R + r] = va;
        na++;
      }
      const double vt = v7[pk_opp(s) * R + (inv[nb] - 1)];   // A[nb][r]
      if (vt != 0) {
        t_col[nt * R + r] = (int32_t)nb;
        t_val[nt * R + r] = vt;
        nt++;
      }
    }
    a_cnt[r] = (uint8_t)na;
    t_cnt[r] = (uint8_t)nt;
    if (na == 0) atomicMin(&empty[0], (unsigned long long)c);
    if (nt == 0) atomicMin(&empty[1], (unsigned long long)c);
  }
}

struct PackArgs {
  const uint8_t* sm;
  const int32_t* inv;
  const uint8_t* cnt;
  const int32_t* col;
  const double* val;
  int64_t n, R;
  const double* x;
  double* y;
  float* y32;
  const double* s;
  const double* w;
  int sign, neg, zero_inactive, dot_w, dot_self, slot_w, ctl, gate, guard;
  DevScratch* S;
};

// y = A x (+/- s) with the matvec request's epilogue (negation, dots, control).
__global__ void __launch_bounds__(RED_THREADS) k_pack_mv(PackArgs a) {
  __shared__ double sh[32];
  __shared__ bool last;
  if ((a.ctl != CTL_NONE || a.guard) && (a.S->iscalars[I_DONE] || (a.gate && !a.S->iscalars[I_NEEDREP]))) return;
  DotAcc<double> dw, ds;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.n; c += (int64_t)gridDim.x * blockDim.x) {
    if (!a.sm[c]) {
      if (a.zero_inactive) {
        if (a.y) a.y[c] = 0;
        if (a.y32) a.y32[c] = 0.f;
      }
      continue;
    }
    const int64_t r = a.inv[c] - 1;
    const int cnt = a.cnt[r];
    double v = 0;
    for (int q = 0; q < cnt; q++) v = v + a.val[q * a.R + r] * a.x[a.col[q * a.R + r]];
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

// Matvec of a packed operator (FP64; `transpose` flips op's current side).
void xf_pack_mv64(const xf_op* op, const MvReq<double>& q) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  const PackData* P = op->pack;
  const bool t = (op->transposed != 0) != (q.transpose != 0);
  PackArgs a;
  a.sm = g->smask; a.inv = g->inv;
  a.cnt = t ? P->t_cnt : P->a_cnt;
  a.col = t ? P->t_col : P->a_col;
  a.val = t ? P->t_val : P->a_val;
  a.n = g->ncell; a.R = P->rows;
  a.x = q.x; a.y = q.y; a.y32 = q.y32; a.s = q.s; a.w = q.w;
  a.sign = q.sign; a.neg = q.neg; a.zero_inactive = q.zero_inactive;
  a.dot_w = q.w != nullptr; a.dot_self = q.dot_self; a.slot_w = q.slot; a.ctl = q.ctl; a.gate = q.gate;
  a.guard = q.guard;
  a.S = ctx->scratch;
  k_pack_mv<<<red_blocks(ctx, g->ncell), RED_THREADS, 0, ctx->stream>>>(a);
}

void xf_pack_free(PackData* P) {
  if (!P) return;
  void* ps[] = {P->a_cnt, P->a_col, P->a_val, P->t_cnt, P->t_col, P->t_val};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete P;
}

extern "C" int xf_pack_create(xf_op* src, xf_op** out) {
  if (!src || !out) return XF_ERR_ARG;
  *out = nullptr;
  xf_grid* g = src->g;
  xf_ctx* ctx = g->ctx;
  if (src->kind == XF_OP_PACK) return xf_fail(ctx, XF_ERR_ARG, "xf_pack_create: the operator is already packed");
  if ((src->kind == XF_OP_VARDIV && !src->rho_set) || (src->kind == XF_OP_ADVDIFF && !src->adv_set))
    return xf_fail(ctx, XF_ERR_STATE, "xf_pack_create: set the operator's coefficients first");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t R = g->end_index, n = g->ncell;
  if (R <= 0) return xf_fail(ctx, XF_ERR_ARG, "xf_pack_create: the grid has no active cells");
  PackData* P = new PackData();
  P->rows = R;
  double *e = nullptr, *y = nullptr, *v7 = nullptr;
  unsigned long long* empty = nullptr;
  int st = XF_OK;
  auto fail = [&](int s, const char* msg) {
    cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    if (e) cudaFree(e);
    if (y) cudaFree(y);
    if (v7) cudaFree(v7);
    if (empty) cudaFree(empty);
    xf_pack_free(P);
    return xf_fail(ctx, s, "xf_pack_create: %s", msg);
  };
  if (cudaMalloc(&e, n * 8) || cudaMalloc(&y, n * 8) || cudaMalloc(&v7, 7 * R * 8) ||
      cudaMalloc(&empty, 2 * sizeof(unsigned long long)) || cudaMalloc(&P->a_cnt, R) ||
      cudaMalloc(&P->a_col, 7 * R * 4) || cudaMalloc(&P->a_val, 7 * R * 8) || cudaMalloc(&P->t_cnt, R) ||
      cudaMalloc(&P->t_col, 7 * R * 4) || cudaMalloc(&P->t_val, 7 * R * 8))
    return fail(XF_ERR_NOMEM, "device allocation");
  cudaStream_t s = ctx->stream;
  if (cudaMemsetAsync(v7, 0, 7 * R * 8, s) || cudaMemsetAsync(empty, 0xff, 2 * sizeof(unsigned long long), s) ||
      cudaMemsetAsync(P->a_col, 0, 7 * R * 4, s) || cudaMemsetAsync(P->t_col, 0, 7 * R * 4, s) ||
      cudaMemsetAsync(P->a_val, 0, 7 * R * 8, s) || cudaMemsetAsync(P->t_val, 0, 7 * R * 8, s))
    return fail(XF_ERR_CUDA, "memset");
  const int eb = grid_blocks(ctx, n, 256);
  for (int q = 0; q < 27; q++) {
    k_pack_probe<<<eb, 256, 0, s>>>(g->smask, g->n1, g->n2, g->n3, q, e);
    MvReq<double> m;
    m.x = e; m.y = y; m.exact = true;   // the operator's own arithmetic, bit for bit
    xf_mv64(src, m);
    k_pack_collect<<<eb, 256, 0, s>>>(g->smask, g->inv, g->n1, g->n2, g->n3, q, y, R, v7);
  }
  k_pack_fill<<<eb, 256, 0, s>>>(g->smask, g->inv, g->n1, g->n2, g->n3, R, v7, P->a_cnt, P->a_col, P->a_val,
                                 P->t_cnt, P->t_col, P->t_val, empty);
  unsigned long long h_empty[2];
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(h_empty, empty, sizeof(h_empty), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(XF_ERR_CUDA, "probe launches failed");
  if (h_empty[0] != ~0ull || h_empty[1] != ~0ull) {
    // T1dPackOperator's "Zero row was found" throws (XOperator.cpp:1233, 1316)
    const unsigned long long c = h_empty[1] != ~0ull ? h_empty[1] : h_empty[0];
    char msg[160];
    snprintf(msg, sizeof(msg), "zero %s at cell (%d, %d, %d), the reference throws there",
             h_empty[1] != ~0ull ? "column" : "row", (int)(c / g->s1), (int)((c % g->s1) / g->s2), (int)(c % g->s2));
    return fail(XF_ERR_MASK, msg);
  }
  // nnz of both storages (host sum of the counts: set-up only)
  std::vector<uint8_t> ca(R), ct(R);
  if (cudaMemcpy(ca.data(), P->a_cnt, R, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(ct.data(), P->t_cnt, R, cudaMemcpyDeviceToHost))
    return fail(XF_ERR_CUDA, "count download");
  for (int64_t r = 0; r < R; r++) {
    P->nnz += ca[r];
    P->nnz_t += ct[r];
  }
  cudaFree(e);
  cudaFree(y);
  cudaFree(v7);
  cudaFree(empty);
  xf_op* op = new xf_op();
  op->g = g;
  op->kind = XF_OP_PACK;
  op->rho = nullptr;
  op->rho32 = nullptr;
  op->rho_set = 1;
  op->pack = P;
  op->transposed = 0;
  *out = op;
  (void)st;
  return XF_OK;
}

extern "C" int xf_op_transpose(xf_op* op) {
  if (!op) return XF_ERR_ARG;
  if (op->kind != XF_OP_PACK)   // T3dLaplaceOperator::operator~ throws (XOperator.h:302)
    return xf_fail(op->g->ctx, XF_ERR_UNSUPPORTED, "xf_op_transpose: only packed operators have a transpose");
  op->transposed ^= 1;
  return XF_OK;
}

extern "C" int xf_pack_size(const xf_op* op, int64_t* rows, int64_t* nnz, int64_t* nnz_t) {
  if (!op) return XF_ERR_ARG;
  if (op->kind != XF_OP_PACK) return xf_fail(op->g->ctx, XF_ERR_ARG, "xf_pack_size: not a packed operator");
  if (rows) *rows = op->pack->rows;
  if (nnz) *nnz = op->pack->nnz;
  if (nnz_t) *nnz_t = op->pack->nnz_t;
  return XF_OK;
}

extern "C" int xf_pack_download(const xf_op* op, int transpose, int32_t* ptr, int32_t* cols, double* vals) {
  if (!op || !ptr || !cols || !vals) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  if (op->kind != XF_OP_PACK) return xf_fail(ctx, XF_ERR_ARG, "xf_pack_download: not a packed operator");
  const PackData* P = op->pack;
  const int64_t R = P->rows;
  const xf_grid* g = op->g;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<uint8_t> cnt(R);
  std::vector<int32_t> col(7 * R), inv(g->ncell);
  std::vector<double> val(7 * R);
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  XF_CUDA(ctx, cudaMemcpy(cnt.data(), transpose ? P->t_cnt : P->a_cnt, R, cudaMemcpyDeviceToHost));
  XF_CUDA(ctx, cudaMemcpy(col.data(), transpose ? P->t_col : P->a_col, 7 * R * 4, cudaMemcpyDeviceToHost));
  XF_CUDA(ctx, cudaMemcpy(val.data(), transpose ? P->t_val : P->a_val, 7 * R * 8, cudaMemcpyDeviceToHost));
  XF_CUDA(ctx, cudaMemcpy(inv.data(), g->inv, g->ncell * 4, cudaMemcpyDeviceToHost));
  int64_t m = 0;
  ptr[0] = 0;
  for (int64_t r = 0; r < R; r++) {
    for (int q = 0; q < cnt[r]; q++) {
      cols[m] = inv[col[q * R + r]] - 1;
      vals[m] = val[q * R + r];
      m++;
    }
    ptr[r + 1] = (int32_t)m;
  }
  return XF_OK;
}
