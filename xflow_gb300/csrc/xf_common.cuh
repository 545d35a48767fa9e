// Internal definitions shared by the xflow_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/xflow.h"

// ---------------------------------------------------------------------------
// Cell kind byte: bits 0..5 = neighbour in direction (-x,+x,-y,+y,-z,+z) is
// not Fictive (flux open, XOperator.cpp:1003-1008); bits 6..7 = row kind.
enum : uint8_t {
  K_MX = 1, K_PX = 2, K_MY = 4, K_PY = 8, K_MZ = 16, K_PZ = 32,
  K_ROW_SHIFT = 6,
  ROW_NONE = 0, ROW_ACTUAL = 1, ROW_PREDEF = 2, ROW_PRENORM = 3
};
__host__ __device__ inline int row_of(uint8_t k) { return k >> K_ROW_SHIFT; }

// Fixed reduction geometry: deterministic partial sums (one per block, then a
// fixed-order final pass by the last block to finish).
constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 8192;  // partials per slot (stencil grids can be 2-D)
constexpr int NUM_SLOTS = 16;         // independent reductions in flight

// Device-resident scratch of a context.
struct DevScratch {
  double partials[NUM_SLOTS][RED_MAX_BLOCKS];
  unsigned int tickets[NUM_SLOTS];
  double scalars[256];
  long long iscalars[64];
};

struct xf_ctx {
  int device;
  int sm_count;
  cudaStream_t stream;
  DevScratch* scratch;       // device
  double* host_scalars;      // pinned, 256 doubles
  cudaEvent_t ev0, ev1;
  void* work = nullptr;       // device workspace of line solvers (grows, freed by xf_destroy)
  size_t work_bytes = 0;
  char err[512];
};

// Device workspace of at least `bytes` (nullptr when it cannot grow).
void* xf_ctx_work(xf_ctx* ctx, size_t bytes);

struct xf_grid {
  xf_ctx* ctx;
  int n1, n2, n3;
  int64_t ncell, s1, s2;
  int64_t end_index;
  uint8_t* code;             // device, per cell: the reference point code (0..8)
  uint8_t* nflag;            // device, per Normal (code 5) cell: bit 0/1/2 = normal x/y/z nonzero
  uint8_t* kind;             // device, per cell, then 64 zero bytes
  uint8_t* smask;            // device, per cell (0/1)
  int32_t* inv;              // device, Rn index per cell (0 inactive)
  int32_t* brow_of;          // device, per cell: index into brow arrays or -1
  int64_t nbrow;             // PreDefined + PreNormal rows
  double* brow_nrm;          // device, 3 per boundary row
  double *hx, *hy, *hz;      // device separations (n-1 each)
  float *fhx, *fhy, *fhz;
  // fast-path coefficients per index: c?m[i] = 1/(h[i-1]*hh[i]), c?p[i] = 1/(h[i]*hh[i]),
  // hh[i] = (h[i-1]+h[i])/2; rh = 1/h; rhh = 1/hh
  double *cxm, *cxp, *cym, *cyp, *czm, *czp;
  float *fxm, *fxp, *fym, *fyp, *fzm, *fzp;
  double *rhx, *rhy, *rhz, *rhhx, *rhhy, *rhhz;
  float *frhx, *frhy, *frhz, *frhhx, *frhhy, *frhhz;
  double* diag;              // device, per cell: diagonal of the Laplace Actual row (fast FP64)
  int uniform;               // every separation of each axis is equal: coefficients are per-axis constants
  double ucx, ucy, ucz;      // then 1/h^2 per axis (== c?m[i] == c?p[i] for every interior index)
  int lap_status, vardiv_status;
  int64_t lap_bad, vardiv_bad;
};

struct xf_vec {
  xf_grid* g;
  int dtype;
  void* data;
};

struct PackData;   // packed operator storage (xf_pack.cu)
struct xf_op {
  xf_grid* g;
  int kind;
  double* rho;     // device density box (VARDIV)
  float* rho32;
  int rho_set;
  PackData* pack = nullptr;   // XF_OP_PACK
  int transposed = 0;         // XF_OP_PACK: applies A^T (T1dPackOperator::operator~)
  // XF_OP_ADVDIFF: advecting velocity boxes (FP64 and FP32 copies) and coefficients
  double* adv64[3] = {nullptr, nullptr, nullptr};
  float* adv32[3] = {nullptr, nullptr, nullptr};
  double* adD64 = nullptr;   // per-cell diffusion coefficient (null: the constant ad_D)
  float* adD32 = nullptr;
  int adD_set = 0;
  double ad_tau = 1, ad_D = 0;
  int ad_flags = 0, adv_set = 0;
  // the FP64 fast Actual rows' coefficients (7 per cell, SoA), refreshed by
  // xf_op_ready after either setter; invalid until then (the rows then take
  // the exact form)
  mutable double* adc64 = nullptr;
  mutable int adc_valid = 0;
  // and the inverse row diagonals (0 off the active set), for the Jacobi
  // preconditioner of BiCGStab, refreshed with the table
  mutable double* adj64 = nullptr;
  mutable int lap_jac_valid = 0;   // XF_OP_LAPLACE: adj64 holds its inverse diagonals (built on first use)
  // device staging boxes of xf_solve_host, kept between calls
  xf_vec* host_x = nullptr;
  xf_vec* host_b = nullptr;
  // unique per operator ever created (a graph built for one operator is never
  // replayed on another that reuses its address)
  unsigned long long serial = 0;
};

// ---------------------------------------------------------------------------
int xf_fail(xf_ctx* ctx, int status, const char* fmt, ...);
#define XF_CUDA(ctx, call)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return xf_fail((ctx), XF_ERR_CUDA, "%s: %s (%s:%d)", #call,  \
                                          cudaGetErrorString(e_), __FILE__, __LINE__);   \
  } while (0)

inline int grid_blocks(const xf_ctx* ctx, int64_t n, int threads, int per_sm = 8) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)ctx->sm_count * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}
inline int red_blocks(const xf_ctx* ctx, int64_t n) {
  int b = grid_blocks(ctx, n, RED_THREADS, 8);
  return b > RED_MAX_BLOCKS ? RED_MAX_BLOCKS : b;
}
__device__ __forceinline__ int lin_block() { return blockIdx.y * gridDim.x + blockIdx.x; }
__device__ __forceinline__ int num_blocks() { return gridDim.x * gridDim.y; }

// ---------------------------------------------------------------------------
// Per-thread dot accumulators.  FP64 data: plain FP64 FMA.  FP32 data: the
// product a*b is split exactly into hi + lo with one FMA (TwoProduct) and
// summed in float-float (TwoSum), so the per-thread partial carries ~44 bits
// without touching the FP64 pipe (1/58 of the FP32 rate on GB300); partials
// are combined in FP64 across threads and blocks.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float s = hi + p;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (p - bp);
    hi = s;
    lo = lo + (err + e);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Sum of the block's accumulators, valid in thread 0.  FP32 accumulators are
// reduced across each warp in float-float (FP32 pipe) and reach FP64 once per
// warp, so the epilogue issues ~1/32 of the FP64 instructions of a per-thread
// conversion.
__device__ inline double warp_sum(double v);
template <typename T>
__device__ inline double block_sum_acc(const DotAcc<T>& acc, double* sh);
template <>
__device__ inline double block_sum_acc<double>(const DotAcc<double>& acc, double* sh);
template <>
__device__ inline double block_sum_acc<float>(const DotAcc<float>& acc, double* sh) {
  float hi = acc.hi, lo = acc.lo;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float bh = __shfl_xor_sync(0xffffffffu, hi, o), bl = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = hi + bh;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (bh - bp);
    hi = s;
    lo = lo + (bl + err);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = (double)hi + (double)lo;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  return v;
}

// First strict maximum of |a| in flat order: (value, cell) pairs combine by
// larger value, then smaller cell.
struct AbsMax { double v; long long c; };
__device__ __forceinline__ AbsMax am_combine(AbsMax x, AbsMax y) {
  if (y.c < 0) return x;
  if (x.c < 0) return y;
  if (y.v > x.v || (y.v == x.v && y.c < x.c)) return y;
  return x;
}
__device__ __forceinline__ AbsMax am_warp(AbsMax a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    AbsMax b;
    b.v = __shfl_xor_sync(0xffffffffu, a.v, o);
    b.c = __shfl_xor_sync(0xffffffffu, a.c, o);
    a = am_combine(a, b);
  }
  return a;
}
__device__ inline AbsMax am_block(AbsMax a, AbsMax* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  a = am_warp(a);
  __syncthreads();
  if (lane == 0) sh[w] = a;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  AbsMax r;
  r.v = 0; r.c = -1;
  if (threadIdx.x < nw) r = sh[threadIdx.x];
  if (w == 0) r = am_warp(r);
  return r;
}

// Block reduction helpers (FP64).
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; result valid in thread 0.  sh must hold 32 doubles.
__device__ inline double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  return v;
}

template <>
__device__ inline double block_sum_acc<double>(const DotAcc<double>& acc, double* sh) {
  return block_sum(acc.value(), sh);
}

// Publishes one accumulator into partials[slot] under tickets[ticket]; true in
// the last block to arrive.
template <typename T>
__device__ inline bool publish_acc(DevScratch* S, int slot, int ticket, const DotAcc<T>& acc, double* sh, bool* flag) {
  const double s = block_sum_acc<T>(acc, sh);
  if (threadIdx.x == 0) {
    S->partials[slot][lin_block()] = s;
    __threadfence();
    unsigned int t = atomicAdd(&S->tickets[ticket], 1u);
    *flag = (t == (unsigned)num_blocks() - 1);
  }
  __syncthreads();
  return *flag;
}

// Publishes this block's partial of `nval` sums into slot partials and returns
// true in the last block to arrive (all partials visible).  `flag` is shared.
template <int NV>
__device__ inline bool publish_partials(DevScratch* S, int slot0, const double (&v)[NV], double* sh, bool* flag) {
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double s = block_sum(v[q], sh);
    if (threadIdx.x == 0) S->partials[slot0 + q][lin_block()] = s;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int t = atomicAdd(&S->tickets[slot0], 1u);
    *flag = (t == (unsigned)num_blocks() - 1);
  }
  __syncthreads();
  return *flag;
}

// In the last block: fixed-order sum of the published partials of slot.
__device__ inline double finish_partials(DevScratch* S, int slot, double* sh) {
  __threadfence();
  double v = 0.0;
  const int nb = num_blocks();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v += __ldcg(&S->partials[slot][b]);
  return block_sum(v, sh);
}

// ---------------------------------------------------------------------------
// BF16 activations of the learned preconditioner are stored in channel planes
// of 8: plane q holds channels 8q .. 8q+7 of every cell, 16 bytes per cell,
// so element (cell c, channel ch) sits at (ch / 8) * plane_stride + c * 8 +
// ch % 8.  A block of consecutive cells of one plane is then the canonical
// K-major operand layout of the tensor cores (core matrices of 8 rows x 16
// bytes), copied by one bulk copy whatever its first cell.
//
// Convolution weights for the tensor cores, tiled per (16-channel input
// chunk c, slab s = 3 (di+1) + (dj+1), 8-channel half q, stacked output row
// n = dk_index * Co + o, 8 channels): the 9 slabs of one chunk are contiguous,
// and each (c, s) block is the canonical K-major B operand of one MMA.
__host__ __device__ inline int64_t conv_tiled_index(int t, int o, int i, int co, int ci) {
  const int s = t / 3, n = (t % 3) * co + o, c = i >> 4, q = (i >> 3) & 1, e = i & 7;
  return ((((int64_t)c * 9 + s) * 2 + q) * (3 * co) + n) * 8 + e;
}
