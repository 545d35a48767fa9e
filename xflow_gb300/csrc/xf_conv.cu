// Tensor-core (tcgen05) kernels of the learned preconditioner.
//
// xf_tc_gemm_bf16: one 128 x N x K tile, D = A B^T with BF16 A (128 x K) and
// B (N x K), K contiguous, FP32 accumulation in tensor memory.  It is the
// building block the implicit-GEMM convolutions below use, exposed so that
// its operand layout and descriptors are checked on their own.
#include <cuda.h>
#include <cuda_bf16.h>

#include <stdlib.h>

#include "xf_common.cuh"
#include "xf_tc.cuh"

constexpr int TC_M = 128;

// Copies a rows x K BF16 matrix (K contiguous, `ld` elements per row) into
// the canonical no-swizzle K-major layout: core matrix (row group g, K group
// q) at g * (K / 8) * 128 + q * 128 bytes.
__device__ __forceinline__ void stage_kmajor(uint8_t* dst, const uint16_t* src, int rows, int K, int ld) {
  const int kg = K / 8;
  for (int u = threadIdx.x; u < rows * kg; u += blockDim.x) {
    const int r = u / kg, q = u - r * kg;
    const uint4 v = *reinterpret_cast<const uint4*>(src + (int64_t)r * ld + q * 8);
    *reinterpret_cast<uint4*>(dst + (r >> 3) * kg * 128 + q * 128 + (r & 7) * 16) = v;
  }
}

__host__ __device__ inline uint32_t tmem_cols(int n) {
  uint32_t c = 32;
  while ((int)c < n) c <<= 1;
  return c;
}

// variant 0: LBO = distance between K-adjacent core matrices, SBO = between
// row-adjacent ones; variant 1: the two swapped (both stay inside the tiles).
__global__ void __launch_bounds__(128) k_tc_gemm(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                 float* __restrict__ D, int N, int K, int variant,
                                                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  uint8_t* sA = smem;
  uint8_t* sB = smem + TC_M * K * 2;
  stage_kmajor(sA, A, TC_M, K, K);
  stage_kmajor(sB, B, N, K, K);
  tc::fence_async_smem();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = tmem_cols(N);
  if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base;
  const uint32_t kstride = 128, rstride = (uint32_t)(K / 8) * 128;
  const uint32_t lbo = variant ? rstride : kstride, sbo = variant ? kstride : rstride;
  if (threadIdx.x == 0) {
    const uint32_t idesc = tc::idesc_bf16_f32(TC_M, N);
    for (int s = 0; s < K / 16; s++) {
      const uint64_t ad = tc::smem_desc(tc::smem_addr(sA + s * 256), lbo, sbo);
      const uint64_t bd = tc::smem_desc(tc::smem_addr(sB + s * 256), lbo, sbo);
      tc::mma_bf16(tbase, ad, bd, idesc, s > 0);
    }
    tc::mma_commit(&mbar);
  }
  bool ok = __syncthreads_and(tc::mbar_wait(&mbar, 0));
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    ok = __syncthreads_and(tc::mbar_wait(&mbar, 0));   // let the MMAs drain before the columns are freed
  }
  tc::fence_after_sync();
  if (ok) {
    const int row = warp * 32 + lane;
    for (int c = 0; c < N; c += 8) {
      float v[8];
      tc::tmem_ld8(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int q = 0; q < 8; q++) D[(int64_t)row * N + c + q] = v[q];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

extern "C" int xf_tc_gemm_bf16(xf_ctx* ctx, int N, int K, const uint16_t* host_a, const uint16_t* host_b,
                               float* host_d, int variant) {
  if (!ctx || !host_a || !host_b || !host_d) return XF_ERR_ARG;
  if (N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16 || (variant != 0 && variant != 1))
    return xf_fail(ctx, XF_ERR_ARG, "xf_tc_gemm_bf16: N in 16..256 and K in 16..256, multiples of 16");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  uint16_t *a = nullptr, *b = nullptr;
  float* d = nullptr;
  int* err = nullptr;
  auto cleanup = [&]() {
    cudaFree(a); cudaFree(b); cudaFree(d); cudaFree(err);
  };
  if (cudaMalloc(&a, TC_M * K * 2) || cudaMalloc(&b, N * K * 2) || cudaMalloc(&d, TC_M * N * 4) ||
      cudaMalloc(&err, 4)) {
    cleanup();
    cudaGetLastError();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_tc_gemm_bf16: allocation");
  }
  cudaStream_t s = ctx->stream;
  cudaMemcpyAsync(a, host_a, TC_M * K * 2, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b, host_b, N * K * 2, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(d, 0, TC_M * N * 4, s);
  cudaMemsetAsync(err, 0, 4, s);
  const size_t smem = (size_t)(TC_M + N) * K * 2;
  if (cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cleanup();
    return xf_fail(ctx, XF_ERR_CUDA, "xf_tc_gemm_bf16: shared memory attribute");
  }
  k_tc_gemm<<<1, 128, smem, s>>>(a, b, d, N, K, variant, err);
  int herr = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host_d, d, TC_M * N * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return xf_fail(ctx, XF_ERR_CUDA, "xf_tc_gemm_bf16: %s", cudaGetErrorString(e));
  if (herr) return xf_fail(ctx, XF_ERR_CUDA, "xf_tc_gemm_bf16: the MMA completion wait ran out");
  return XF_OK;
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution as an implicit GEMM on the tensor cores.
//
// Activations are channels-last BF16 boxes of the level's grid (the box with
// its ghost layer, cell c = (i n2 + j) n3 + k, Ci channels per cell, row pitch
// `ld` channels), allocated with a zero margin of XF_CONV_MARGIN(n2, n3) rows
// before cell 0 and after the last cell, so every tap of every tile reads
// inside the allocation.  Ghost and inactive cells hold 0 in every activation
// (the epilogue multiplies by the level's mask), which makes the ghost layer
// the zero padding of the convolution, also across the flattened row ends.
//
// A tile is 128 consecutive cells.  For tap t at offset o_t the A operand is
// the contiguous block of rows c0 + o_t .. c0 + o_t + 127 (128 x Ci), the B
// operand W[t] (Co x Ci); the 27 taps x Ci/16 MMAs accumulate in tensor
// memory (128 lanes x Co FP32 columns).  Operand stages rotate through
// XF_CONV_STAGES shared-memory buffers; a stage is refilled only after the
// tensor core has signalled (mbarrier) that the MMAs reading it are done.
// Epilogue: + bias, ReLU (optional), x mask, BF16 or FP32 store of the first
// `out_ch` channels at row pitch out_ld.
constexpr int CONV_STAGES = 3;

struct ConvArgs {
  const uint16_t* in;   // cell 0, channel 0 of the input slice
  int in_ld, Ci;
  const uint16_t* W;    // [27][Co][Ci]
  const float* bias;    // [Co] or null
  int Co;
  const uint8_t* mask;  // [ncell]
  int n2, n3;
  int64_t ncell;
  uint16_t* out16;      // cell 0, first output channel (BF16), or null
  float* out32;         // or FP32
  int out_ld, out_ch, relu;
  const uint16_t* gate;   // optional: zero the outputs where gate[c * gate_ld + ch] <= 0 (ReLU backward)
  int gate_ld;
  int* err;
};

__global__ void __launch_bounds__(128) k_conv3_tc(ConvArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar[CONV_STAGES];
  __shared__ uint32_t tmem_base;
  const int Ci = a.Ci, Co = a.Co;
  const int stage_a = TC_M * Ci * 2, stage_b = Co * Ci * 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = tmem_cols(Co);
  if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
  if (threadIdx.x == 0)
    for (int s = 0; s < CONV_STAGES; s++) tc::mbar_init(&mbar[s], 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base;
  const uint32_t idesc = tc::idesc_bf16_f32(TC_M, Co);
  const uint32_t lbo = 128, sbo = (uint32_t)(Ci / 8) * 128;
  const int64_t P = (int64_t)a.n2 * a.n3;
  uint32_t issued[CONV_STAGES] = {0, 0, 0}, waited[CONV_STAGES] = {0, 0, 0};
  bool ok = true;
  auto drain = [&](int s) {   // wait for the stage's outstanding commit (at most one)
    if (waited[s] < issued[s]) {
      const bool w = tc::mbar_wait(&mbar[s], (issued[s] - 1) & 1);
      if (!w) ok = false;
      waited[s] = issued[s];
    }
  };
  const int64_t ntiles = (a.ncell + TC_M - 1) / TC_M;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t c0 = tile * TC_M;
    for (int t = 0; t < 27; t++) {
      const int s = t % CONV_STAGES;
      drain(s);
      const int di = t / 9 - 1, dj = (t / 3) % 3 - 1, dk = t % 3 - 1;
      const int64_t off = di * P + dj * (int64_t)a.n3 + dk;
      uint8_t* sA = smem + s * (stage_a + stage_b);
      uint8_t* sB = sA + stage_a;
      stage_kmajor(sA, a.in + (c0 + off) * a.in_ld, TC_M, Ci, a.in_ld);
      stage_kmajor(sB, a.W + (int64_t)t * Co * Ci, Co, Ci, Ci);
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc::fence_after_sync();
        for (int k = 0; k < Ci / 16; k++) {
          const uint64_t ad = tc::smem_desc(tc::smem_addr(sA + k * 256), lbo, sbo);
          const uint64_t bd = tc::smem_desc(tc::smem_addr(sB + k * 256), lbo, sbo);
          tc::mma_bf16(tbase, ad, bd, idesc, t > 0 || k > 0);
        }
        tc::mma_commit(&mbar[s]);
      }
      issued[s]++;
    }
    for (int s = 0; s < CONV_STAGES; s++) drain(s);
    ok = __syncthreads_and(ok);
    if (!ok) break;
    tc::fence_after_sync();
    // epilogue: warp w owns rows 32w .. 32w+31 (TMEM lanes)
    const int64_t c = c0 + warp * 32 + lane;
    const bool live = c < a.ncell;
    const float m = live ? (float)a.mask[c] : 0.f;
    for (int co = 0; co < Co; co += 8) {
      float v[8];
      tc::tmem_ld8(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)co, v);
      if (!live || co >= a.out_ch) continue;
      uint16_t gt[8];
      if (a.gate) *reinterpret_cast<uint4*>(gt) = *reinterpret_cast<const uint4*>(a.gate + c * a.gate_ld + co);
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float x = v[q] + (a.bias ? a.bias[co + q] : 0.f);
        if (a.relu) x = fmaxf(x, 0.f);
        if (a.gate && ((gt[q] & 0x8000u) || !(gt[q] & 0x7FFFu))) x = 0.f;   // gate value <= 0
        v[q] = x * m;
      }
      if (a.out16) {
        uint32_t pk[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
          pk[q] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(a.out16 + c * a.out_ld + co) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      } else {
        const int nq = min(8, a.out_ch - co);
        for (int q = 0; q < nq; q++) a.out32[c * a.out_ld + co + q] = v[q];
      }
    }
    tc::fence_before_sync();
    __syncthreads();   // TMEM is read before the next tile's first MMA overwrites it
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(a.err, 1);
    for (int s = 0; s < CONV_STAGES; s++)
      if (waited[s] < issued[s]) tc::mbar_wait(&mbar[s], (issued[s] - 1) & 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

// ---------------------------------------------------------------------------
// The same convolution with the three k-taps of each (di, dj) stacked along N,
// fed by the tensor memory accelerator.
//
// A tcgen05.mma of M = 128, K = 16 costs about the same time for any N up to
// 32 (about 39 cycles on GB300; 44 at N = 64, 60 at 128), so one MMA of
// N = 3 Co replaces three of N = Co.  For slab (di, dj) the A operand is the
// 128 rows X[c0 - 1 + di P + dj n3 + r], the B operand the taps (di, dj, -1),
// (di, dj, 0), (di, dj, +1) stacked, [3 Co][Ci] (consecutive in the weight
// layout [27][Co][Ci]); TMEM accumulates D_dk over the nine slabs, and the
// epilogue applies the k shift on the output side:
//     y[c0 + r - 1] = D_-1[r - 1] + D_0[r] + D_+1[r + 1],   r = 1 .. 126,
// neighbouring TMEM rows coming from the neighbouring lanes (warp shuffles; a
// shared-memory exchange across warps).  A tile therefore yields 126 cells;
// the last tile starts at ncell - 126 (its overlap rewrites identical values).
//
// A pipeline step is one (slab, 16-channel chunk): a 128 x 16 block of X and
// a 3 Co x 16 block of W, each one 2-D tensor copy (cp.async.bulk.tensor)
// with the 32-byte swizzle, which writes exactly the K-major SWIZZLE_32B
// operand layout the MMA descriptors name (rows of 32 bytes, the two 16-byte
// halves of rows 4..7 of every 8-row group exchanged).  Rows outside the box
// [0, ncell) read as zeros (the copy's out-of-bounds fill), like the zero
// margins.  The CTA is persistent and warp-specialised:
//   warp 4, one thread: issues the copies of each step into a ring of
//       stages (full barrier: the copies' transaction bytes; empty barrier:
//       the MMA that read the stage has completed);
//   warp 5, one thread: one MMA per step into one of two TMEM accumulators
//       (so the epilogue of a tile overlaps the next tile's MMAs), a commit
//       per stage and one per finished tile;
//   warps 0-3: the epilogue, TMEM lanes 32 w .. 32 w + 31.
// Every wait is bounded by the SM clock; a wait that runs out sets the
// kernel's error flag and an abort flag in shared memory that ends every
// role's loop, after which the copies and MMAs in flight are waited for
// (bounded) before TMEM is freed.  Requires 3 Co <= 256 (Co <= 80), Ci and Co
// multiples of 16.
constexpr int TM_THREADS = 192;
constexpr int TM_MAX_STAGES = 12;
constexpr long long TM_WAIT_CYCLES = 1ll << 31;   // about a second at the SM clock

// K-major operand descriptor for the 32-byte swizzle: rows of 32 bytes, 8-row
// groups 256 bytes apart (SBO); the leading offset is unused for a K extent
// within the swizzle span.
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;              // LBO (unused): 16 bytes
  d |= (uint64_t)(256 >> 4) << 32;     // SBO: 8 rows x 32 bytes
  d |= (uint64_t)1 << 46;              // descriptor version of this architecture
  d |= (uint64_t)6 << 61;              // layout: SWIZZLE_32B
  return d;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(mbar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(mbar)) : "memory");
}
// 2-D tensor copy global -> shared, completing on `mbar` (transaction bytes).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          tc::smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(tc::smem_addr(mbar))
      : "memory");
}
// Waits for phase `parity` of `mbar`; false when the abort flag is raised or
// the wait runs past TM_WAIT_CYCLES (which raises it).
__device__ __forceinline__ bool tm_wait(uint64_t* mbar, uint32_t parity, volatile int* abort_flag,
                                        bool honour_abort = true) {
  const uint32_t a = tc::smem_addr(mbar);
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (honour_abort && *abort_flag) return false;
    if (clock64() - t0 > TM_WAIT_CYCLES) {
      *abort_flag = 1;
      return false;
    }
  }
}
// Barrier 1 over the four epilogue warps with an AND of `pred`.
__device__ __forceinline__ bool epi_sync_and(bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.cta.red.and.pred q, 1, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)pred)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void epi_sync() { asm volatile("barrier.cta.sync 1, 128;" ::: "memory"); }

// Shared-memory plan of one CTA (host and device).
struct TmPlan {
  int stage_bytes, stages, acc_off, tmem_cols, smem_bytes;
};
__host__ __device__ inline TmPlan tm_plan(int Co, int per_sm_budget) {
  TmPlan p;
  const int n3 = 3 * Co;
  p.stage_bytes = ((128 * 32 + n3 * 32) + 1023) / 1024 * 1024;
  p.acc_off = (n3 + 31) / 32 * 32;
  p.tmem_cols = (int)tmem_cols(p.acc_off + n3);
  int st = (per_sm_budget - 1024) / p.stage_bytes;
  p.stages = st > TM_MAX_STAGES ? TM_MAX_STAGES : st < 3 ? 3 : st;
  p.smem_bytes = p.stages * p.stage_bytes + 1024;   // + alignment slack
  return p;
}

__global__ void __launch_bounds__(TM_THREADS) k_conv3_tma(ConvArgs a, const __grid_constant__ CUtensorMap tmX,
                                                          const __grid_constant__ CUtensorMap tmW, TmPlan plan) {
  extern __shared__ uint8_t dsm[];
  __shared__ uint64_t full[TM_MAX_STAGES], empty[TM_MAX_STAGES], tfull[2], tempty[2], mdone;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ float xch[4][2][80];   // per warp: lane 31's D_-1 row, lane 0's D_+1 row
  const int Ci = a.Ci, Co = a.Co, N3 = 3 * Co, nk = Ci / 16;
  const int steps = 9 * nk;   // pipeline steps per tile
  const int S = plan.stages;
  const uint32_t ab = 128 * 32, bb = (uint32_t)N3 * 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // 1024-byte aligned stages (the swizzle pattern repeats every 256 bytes)
  const uint32_t raw = tc::smem_addr(dsm);
  uint8_t* smem = dsm + ((1024u - (raw & 1023u)) & 1023u);
  if (warp == 0) tc::tmem_alloc(&tmem_base, (uint32_t)plan.tmem_cols);
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int q = 0; q < 2; q++) {
      tc::mbar_init(&tfull[q], 1);
      tc::mbar_init(&tempty[q], 128);
    }
    tc::mbar_init(&mdone, 1);
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base;
  volatile int* abort_p = &abort_flag;
  const int64_t P = (int64_t)a.n2 * a.n3;
  const int64_t ntiles = (a.ncell + 125) / 126;
  const int my_tiles = ntiles > blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_start = [&](int k) {   // first output cell of this CTA's k-th tile
    const int64_t st = ((int64_t)blockIdx.x + (int64_t)k * gridDim.x) * 126;
    return st + 126 > a.ncell ? (a.ncell > 126 ? a.ncell - 126 : (int64_t)0) : st;
  };

  if (warp == 4) {
    if (lane == 0) {   // ---- producer
      int g = 0;
      int last[TM_MAX_STAGES];
      for (int s = 0; s < TM_MAX_STAGES; s++) last[s] = -1;
      bool ok = true;
      for (int k = 0; k < my_tiles && ok; k++) {
        const int64_t row_base = tile_start(k) - 1;
        for (int sl = 0; sl < 9 && ok; sl++) {
          const int di = sl / 3 - 1, dj = sl % 3 - 1;
          const int row0 = (int)(row_base + di * P + dj * (int64_t)a.n3);
          for (int c = 0; c < nk; c++, g++) {
            const int st = g % S;
            if (g >= S && !tm_wait(&empty[st], (uint32_t)(((g / S) - 1) & 1), abort_p)) {
              ok = false;
              break;
            }
            uint8_t* sa = smem + st * plan.stage_bytes;
            mbar_expect_tx(&full[st], ab + bb);
            tma_load_2d(sa, &tmX, c * 16, row0, &full[st]);
            tma_load_2d(sa + ab, &tmW, c * 16, sl * N3, &full[st]);
            last[st] = g;
          }
        }
      }
      // every copy issued has landed before the CTA may leave
      for (int s = 0; s < S; s++)
        if (last[s] >= 0) tm_wait(&full[s], (uint32_t)((last[s] / S) & 1), abort_p, false);
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {   // ---- MMA issuer
      const uint32_t idesc = tc::idesc_bf16_f32(128, N3);
      int g = 0;
      bool ok = true;
      for (int k = 0; k < my_tiles && ok; k++) {
        const int acc = k & 1;
        if (k >= 2 && !tm_wait(&tempty[acc], (uint32_t)(((k / 2) - 1) & 1), abort_p)) break;
        tc::fence_after_sync();
        const uint32_t dacc = tbase + (uint32_t)(acc * plan.acc_off);
        for (int u = 0; u < steps; u++, g++) {
          const int st = g % S;
          if (!tm_wait(&full[st], (uint32_t)((g / S) & 1), abort_p)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint8_t* sa = smem + st * plan.stage_bytes;
          tc::mma_bf16(dacc, smem_desc_sw32(tc::smem_addr(sa)), smem_desc_sw32(tc::smem_addr(sa + ab)), idesc,
                       u > 0);
          tc::mma_commit(&empty[st]);
        }
        if (ok) tc::mma_commit(&tfull[acc]);
      }
      // every MMA issued has completed before TMEM is freed
      tc::mma_commit(&mdone);
      tm_wait(&mdone, 0, abort_p, false);
    }
    __syncwarp();
  } else {   // ---- epilogue, warps 0-3
    for (int k = 0; k < my_tiles; k++) {
      const int acc = k & 1;
      const bool got = tm_wait(&tfull[acc], (uint32_t)((k / 2) & 1), abort_p);
      if (!epi_sync_and(got)) break;
      tc::fence_after_sync();
      const int64_t c0 = tile_start(k);
      const uint32_t trow = tbase + (uint32_t)(acc * plan.acc_off) + ((uint32_t)(warp * 32) << 16);
      // pass 1: rows at the warp edges for the neighbouring warps
      for (int co = 0; co < Co; co += 8) {
        uint32_t dm[8], dp[8];
        tc::tmem_ld8_nowait(trow + (uint32_t)co, dm);
        tc::tmem_ld8_nowait(trow + (uint32_t)(2 * Co + co), dp);
        tc::tmem_wait_ld(dm, dp);
        if (lane == 31)
          for (int q = 0; q < 8; q++) xch[warp][0][co + q] = __uint_as_float(dm[q]);
        if (lane == 0)
          for (int q = 0; q < 8; q++) xch[warp][1][co + q] = __uint_as_float(dp[q]);
      }
      epi_sync();
      const int r = warp * 32 + lane;
      const int64_t c = c0 + r - 1;
      const bool live = r >= 1 && r <= 126 && c < a.ncell;
      const float m = live ? (float)a.mask[c] : 0.f;
      for (int co = 0; co < Co; co += 8) {
        uint32_t dm[8], d0[8], dp[8];
        tc::tmem_ld8_nowait(trow + (uint32_t)co, dm);
        tc::tmem_ld8_nowait(trow + (uint32_t)(Co + co), d0);
        tc::tmem_ld8_nowait(trow + (uint32_t)(2 * Co + co), dp);
        tc::tmem_wait_ld(dm, d0, dp);
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          float prev = __shfl_up_sync(0xffffffffu, __uint_as_float(dm[q]), 1);
          float next = __shfl_down_sync(0xffffffffu, __uint_as_float(dp[q]), 1);
          if (lane == 0) prev = warp > 0 ? xch[warp - 1][0][co + q] : 0.f;
          if (lane == 31) next = warp < 3 ? xch[warp + 1][1][co + q] : 0.f;
          v[q] = prev + __uint_as_float(d0[q]) + next;
        }
        if (!live || co >= a.out_ch) continue;
        uint16_t gt[8];
        if (a.gate) *reinterpret_cast<uint4*>(gt) = *reinterpret_cast<const uint4*>(a.gate + c * a.gate_ld + co);
#pragma unroll
        for (int q = 0; q < 8; q++) {
          float x = v[q] + (a.bias ? a.bias[co + q] : 0.f);
          if (a.relu) x = fmaxf(x, 0.f);
          if (a.gate && ((gt[q] & 0x8000u) || !(gt[q] & 0x7FFFu))) x = 0.f;   // gate value <= 0
          v[q] = x * m;
        }
        if (a.out16) {
          uint32_t pk[4];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
            pk[q] = *reinterpret_cast<const uint32_t*>(&h);
          }
          *reinterpret_cast<uint4*>(a.out16 + c * a.out_ld + co) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        } else {
          const int nq = min(8, a.out_ch - co);
          for (int q = 0; q < nq; q++) a.out32[c * a.out_ld + co + q] = v[q];
        }
      }
      // the accumulator is read: the MMA issuer may overwrite it two tiles on
      tc::fence_before_sync();
      mbar_arrive(&tempty[acc]);
      epi_sync();   // the exchange rows are read before the next tile rewrites them
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) atomicExch(a.err, 1);
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, (uint32_t)plan.tmem_cols);
}

// cuTensorMapEncodeTiled, from the driver at run time (the library links the
// runtime only).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}
// A BF16 matrix of `rows` x `cols` (row pitch `ld` elements) read in boxes of
// box_rows x 16 columns with the 32-byte swizzle; rows outside [0, rows) read
// as zeros.
static bool encode_sw32(CUtensorMap* m, const void* base, int64_t rows, int cols, int ld, int box_rows) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {16, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Error flag of the convolutions: a slot of the context scratch, cleared by
// xf_conv_status.
constexpr int I_CONV_ERR = 60;
static int* conv_err_flag(xf_ctx* ctx) { return reinterpret_cast<int*>(&ctx->scratch->iscalars[I_CONV_ERR]); }

// Launch on the context stream (arguments checked by the caller).
// The dynamic shared-memory attribute of a convolution kernel, raised once
// per kernel and device to the largest size asked for (so that the launches
// of a captured solve set no attribute).
static cudaError_t set_max_smem(const void* kern, int which, int device, size_t smem) {
  static size_t done[4][64] = {};
  size_t& d = done[which][device & 63];
  if (smem <= d) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) d = smem;
  return e;
}

int xf_conv_launch(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int in_ld, int ci, const void* weights,
                   const float* bias, int co, const uint8_t* mask, void* out, int out_ld, int out_ch, int out_fp32,
                   int relu, const void* gate, int gate_ld) {
  int* err = conv_err_flag(ctx);
  ConvArgs a;
  a.gate = (const uint16_t*)gate; a.gate_ld = gate_ld;
  a.in = (const uint16_t*)in; a.in_ld = in_ld; a.Ci = ci;
  a.W = (const uint16_t*)weights; a.bias = bias; a.Co = co;
  a.mask = mask; a.n2 = n2; a.n3 = n3; a.ncell = (int64_t)n1 * n2 * n3;
  a.out16 = out_fp32 ? nullptr : (uint16_t*)out;
  a.out32 = out_fp32 ? (float*)out : nullptr;
  a.out_ld = out_ld; a.out_ch = out_ch; a.relu = relu; a.err = err;
  const int64_t ntiles = (a.ncell + TC_M - 1) / TC_M;
  if (3 * co <= 256) {
    // k-taps stacked along N, operands by tensor copies (the per-tap kernel
    // below takes wider outputs).  CTAs per SM: tensor-memory columns (512 per
    // SM) first, then the shared memory (227 KB per SM, with ~4 KB static and
    // reserved per CTA) is split between them.
    const int tcols = (int)tmem_cols((3 * co + 31) / 32 * 32 + 3 * co);
    int per_sm = 512 / tcols;
    if (per_sm > 4) per_sm = 4;
    const TmPlan plan = tm_plan(co, (227 * 1024) / per_sm - 4 * 1024);
    if (a.ncell + (int64_t)n2 * n3 + n3 + 2 > 2147483647LL)   // the copies' row coordinates are 32-bit
      return xf_fail(ctx, XF_ERR_ARG, "convolution: box too large for 32-bit copy coordinates");
    CUtensorMap tmX, tmW;
    if (!encode_sw32(&tmX, in, a.ncell, ci, in_ld, 128) || !encode_sw32(&tmW, weights, 27LL * co, ci, ci, 3 * co))
      return xf_fail(ctx, XF_ERR_CUDA, "convolution: tensor map encoding failed");
    XF_CUDA(ctx, set_max_smem((const void*)k_conv3_tma, 0, ctx->device, (size_t)plan.smem_bytes));
    const int64_t tiles = (a.ncell + 125) / 126;
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    if (blocks > tiles) blocks = tiles;
    k_conv3_tma<<<(int)blocks, TM_THREADS, plan.smem_bytes, ctx->stream>>>(a, tmX, tmW, plan);
    XF_CUDA(ctx, cudaGetLastError());
    return XF_OK;
  }
  const size_t smem = (size_t)CONV_STAGES * (TC_M * ci * 2 + co * ci * 2);
  XF_CUDA(ctx, set_max_smem((const void*)k_conv3_tc, 3, ctx->device, smem));
  // Residency from the kernel's real limits: shared memory (227 KB per SM, with
  // ~1 KB static and reserved per CTA), tensor-memory columns (512 per SM) and
  // threads (2048 per SM).
  int per_sm = (int)((227 * 1024) / (smem + 2048));
  per_sm = min(per_sm, (int)(512 / tmem_cols(co)));
  per_sm = min(per_sm, 16);
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (int64_t)ctx->sm_count * per_sm;
  if (blocks > ntiles) blocks = ntiles;
  k_conv3_tc<<<(int)blocks, 128, smem, ctx->stream>>>(a);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_conv3d_bf16(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int in_ld, int ci,
                              const void* weights, const float* bias, int co, const uint8_t* mask, void* out,
                              int out_ld, int out_ch, int out_fp32, int relu) {
  if (!ctx || !in || !weights || !mask || !out) return XF_ERR_ARG;
  if (ci < 16 || ci > 128 || ci % 16 || co < 16 || co > 128 || co % 16 || out_ch < 1 || out_ch > co ||
      in_ld < ci || in_ld % 8 || out_ld < out_ch || (!out_fp32 && (out_ld % 8 || out_ch % 8)) || n1 < 3 || n2 < 3 ||
      n3 < 3)
    return xf_fail(ctx, XF_ERR_ARG, "xf_conv3d_bf16: channel counts / pitches out of range");
  if (((uintptr_t)in | (uintptr_t)weights | (uintptr_t)out) & 15)
    return xf_fail(ctx, XF_ERR_ARG, "xf_conv3d_bf16: pointers must be 16-byte aligned");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  return xf_conv_launch(ctx, n1, n2, n3, in, in_ld, ci, weights, bias, co, mask, out, out_ld, out_ch, out_fp32, relu,
                        nullptr, 0);
}

// Reads and clears the error flag of the convolutions since the last call
// (synchronises the stream).
extern "C" int xf_conv_status(xf_ctx* ctx) {
  if (!ctx) return XF_ERR_ARG;
  int* err = conv_err_flag(ctx);
  int h = 0;
  XF_CUDA(ctx, cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  XF_CUDA(ctx, cudaMemsetAsync(err, 0, 4, ctx->stream));
  if (h) return xf_fail(ctx, XF_ERR_CUDA, "convolution: a tensor-core completion wait ran out");
  return XF_OK;
}
