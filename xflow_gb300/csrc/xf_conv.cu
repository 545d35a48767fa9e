// Tensor-core (tcgen05) kernels of the learned preconditioner.
//
// xf_tc_gemm_bf16: one 128 x N x K tile, D = A B^T with BF16 A (128 x K) and
// B (N x K), K contiguous, FP32 accumulation in tensor memory.  It is the
// building block the implicit-GEMM convolutions below use, exposed so that
// its operand layout and descriptors are checked on their own.
#include <cuda_bf16.h>

#include <stdlib.h>

#include <algorithm>

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
// Activations are BF16 boxes of the level's grid (the box with its ghost
// layer, cell c = (i n2 + j) n3 + k) in channel planes of 8 (xf_common.cuh),
// every plane allocated with a zero margin of XF_CONV_MARGIN(n2, n3) rows
// before cell 0 and after the last cell, so every tap of every tile reads
// inside the allocation.  Ghost and inactive cells hold 0 in every activation
// (the epilogue multiplies by the level's mask), which makes the ghost layer
// the zero padding of the convolution, also across the flattened row ends.
// Epilogue: + bias, ReLU (optional), x mask, then the first `out_ch`
// channels stored as BF16 planes or as FP32 cell rows (pitch out_ld).
struct ConvArgs {
  const uint16_t* in;   // plane 0, cell 0 of the input slice
  int64_t in_ps;        // plane stride (elements)
  int Ci;
  const uint16_t* W;    // [27][Co][Ci]
  const uint16_t* Wt;   // the same tiled (conv_tiled_index)
  const float* bias;    // [Co] or null
  int Co;
  const uint8_t* mask;  // [ncell]
  int n2, n3;
  int64_t ncell;
  uint16_t* out16;      // plane 0, cell 0 of the output slice (BF16 planes), or null
  int64_t out_ps;
  float* out32;         // or FP32 rows of pitch out_ld
  int out_ld, out_ch, relu;
  const uint16_t* gate;   // optional BF16 planes: zero the outputs where the gate value <= 0 (ReLU backward)
  int64_t gate_ps;
  int* err;
};

// Epilogue of one cell and 8 output channels (co .. co+7).
__device__ __forceinline__ void conv_store8(const ConvArgs& a, int64_t c, int co, float m, float (&v)[8]) {
  uint16_t gt[8];
  if (a.gate) *reinterpret_cast<uint4*>(gt) = *reinterpret_cast<const uint4*>(a.gate + (co >> 3) * a.gate_ps + c * 8);
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
    *reinterpret_cast<uint4*>(a.out16 + (co >> 3) * a.out_ps + c * 8) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  } else {
    const int nq = min(8, a.out_ch - co);
    for (int q = 0; q < nq; q++) a.out32[c * a.out_ld + co + q] = v[q];
  }
}

// ---------------------------------------------------------------------------
// Per-tap form, for wide outputs (3 Co > 256).  A tile is 128 consecutive
// cells.  For tap t at offset o_t the A operand is the block of rows
// c0 + o_t .. c0 + o_t + 127 (128 x Ci), the B operand W[t] (Co x Ci); the
// 27 taps x Ci/16 MMAs accumulate in tensor memory (128 lanes x Co FP32
// columns).  Operands are staged by the threads in the canonical no-swizzle
// K-major layout; stages rotate through CONV_STAGES buffers, a stage being
// refilled only after the tensor core has signalled (mbarrier) that the MMAs
// reading it are done.
constexpr int CONV_STAGES = 3;

__global__ void __launch_bounds__(128) k_conv3_tc(ConvArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar[CONV_STAGES];
  __shared__ uint32_t tmem_base;
  const int Ci = a.Ci, Co = a.Co, kg = Ci / 8;
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
  const uint32_t lbo = 128, sbo = (uint32_t)kg * 128;
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
      for (int u = threadIdx.x; u < TC_M * kg; u += blockDim.x) {   // A from the channel planes
        const int r = u / kg, q = u - r * kg;
        const uint4 v = *reinterpret_cast<const uint4*>(a.in + q * a.in_ps + (c0 + off + r) * 8);
        *reinterpret_cast<uint4*>(sA + (r >> 3) * kg * 128 + q * 128 + (r & 7) * 16) = v;
      }
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
      conv_store8(a, c, co, m, v);
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
// The convolution with the three k-taps of each (di, dj) stacked along N, fed
// by bulk copies.
//
// A tcgen05.mma of M = 128, K = 16 costs about the same time for any N up to
// 32 (about 39 cycles on GB300; 44 at N = 64, 60 at 128), so one MMA of
// N = 3 Co replaces three of N = Co.  For slab (di, dj) the A operand is the
// 128 rows X[c0 - 1 + di P + dj n3 + r], the B operand the taps (di, dj, -1),
// (di, dj, 0), (di, dj, +1) stacked, 3 Co x 16 per input chunk; TMEM
// accumulates D_dk over the nine slabs and the input chunks, and the epilogue
// applies the k shift on the output side:
//     y[c0 + r - 1] = D_-1[r - 1] + D_0[r] + D_+1[r + 1],   r = 1 .. 126,
// neighbouring TMEM rows coming from the neighbouring lanes (warp shuffles;
// across warps, the edge rows through shared memory as 16-byte stores by
// lanes 31 and 0 and 16-byte loads by every lane: scalar single-lane
// exchanges cost about three times as long).  A tile therefore yields 126 cells;
// the last tile starts at ncell - 126 (its overlap rewrites identical values).
//
// A pipeline stage is one (tile, 16-channel input chunk): for each of the
// nine slabs the two 8-channel planes' 128 rows, 2 KB each, one bulk copy
// (cp.async.bulk) apiece, which is already the canonical K-major operand
// layout; nine MMAs read it.  The tiled weights stay resident in shared
// memory when they fit beside two stages, else each stage also carries its
// chunk's nine B blocks.  Each control step therefore covers nine MMAs.
// The CTA is persistent and warp-specialised:
//   warp 4: issues each stage's copies into a ring, one copy per lane (one
//       thread issuing all of them was the pipeline's bottleneck), lane 0
//       keeping the barriers (full: the copies' transaction bytes; empty: the MMAs that
//       read the stage have completed);
//   warp 5, one thread: the MMAs into one of two TMEM accumulators (the
//       epilogue of a tile overlaps the next tile's MMAs), a commit per
//       stage and one per finished tile;
//   warps 0-3: the epilogue, TMEM lanes 32 w .. 32 w + 31.
// Every wait is bounded by the SM clock; a wait that runs out sets the
// kernel's error flag and an abort flag in shared memory that ends every
// role's loop, after which the copies and MMAs in flight are waited for
// (bounded) before TMEM is freed.  Requires 3 Co <= 256 (Co <= 80), Ci and Co
// multiples of 16.
constexpr int BK_THREADS = 192;
constexpr int BK_MAX_STAGES = 6;
constexpr uint32_t BK_SLAB = 128 * 32;            // one slab's A block (two planes x 2 KB)
constexpr uint32_t BK_A = 9 * BK_SLAB;            // the nine slabs of one chunk
constexpr long long BK_WAIT_CYCLES = 1ll << 31;   // about a second at the SM clock

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(mbar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(mbar)) : "memory");
}
// Bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completing on `mbar` (transaction bytes).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_addr(mbar))
               : "memory");
}
// Waits for phase `parity` of `mbar`; false when the abort flag is raised or
// the wait runs past BK_WAIT_CYCLES (which raises it).
__device__ __forceinline__ bool bk_wait(uint64_t* mbar, uint32_t parity, volatile int* abort_flag,
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
    if (clock64() - t0 > BK_WAIT_CYCLES) {
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

// Shared-memory plan of one CTA.
struct BkPlan {
  int stages, per_sm, resident, acc_off, tmem_cols, smem_bytes;
  uint32_t w_bytes, b_bytes, stage_bytes, w_region;
};
static BkPlan bk_plan(int ci, int co, int static_smem) {
  BkPlan p = {};
  const int n3 = 3 * co;
  p.acc_off = (n3 + 31) / 32 * 32;
  p.tmem_cols = (int)tmem_cols(p.acc_off + n3);
  const int per_sm_t = std::min(2, 512 / p.tmem_cols);
  p.w_bytes = (uint32_t)(27 * co * ci * 2);
  p.b_bytes = (uint32_t)(9 * n3 * 32);
  const uint32_t w_region = (p.w_bytes + 1023) / 1024 * 1024;
  const uint32_t st_res = BK_A, st_str = (BK_A + p.b_bytes + 1023) / 1024 * 1024;
  // (CTAs per SM, weights resident): two CTAs first, resident weights first
  for (int k = 0; k < 4; k++) {
    const int per_sm = k < 2 ? per_sm_t : 1;
    const bool res = (k % 2) == 0;
    if (k < 2 && per_sm_t < 2) continue;
    // dynamic shared memory of one CTA: 228 KB per SM less 1 KB reserved per
    // CTA, at most 227 KB per CTA, less the static part and the alignment slack
    const int dyn = std::min(227 * 1024, (228 * 1024) / per_sm - 1024) - static_smem - 1024;
    const int avail = dyn - (res ? (int)w_region : 0);
    const int st = avail > 0 ? avail / (int)(res ? st_res : st_str) : 0;
    if (st >= 2) {
      p.per_sm = per_sm;
      p.resident = res;
      p.stages = std::min(st, BK_MAX_STAGES);
      p.stage_bytes = res ? st_res : st_str;
      p.w_region = res ? w_region : 0;
      p.smem_bytes = (int)(p.w_region + p.stages * p.stage_bytes + 1024);
      return p;
    }
  }
  return p;   // stages = 0: no plan (never for Co <= 80)
}

__global__ void __launch_bounds__(BK_THREADS) k_conv3_bulk(ConvArgs a, BkPlan plan) {
  extern __shared__ uint8_t dsm[];
  __shared__ uint64_t full[BK_MAX_STAGES], empty[BK_MAX_STAGES], tfull[2], tempty[2], wfull, mdone;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ __align__(16) float xch[2][4][2][80];   // per tile parity and warp: lane 31's D_-1 row, lane 0's D_+1 row
  const int Ci = a.Ci, Co = a.Co, N3 = 3 * Co, nk = Ci / 16;
  const int S = plan.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t raw = tc::smem_addr(dsm);
  uint8_t* smem = dsm + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* wsm = smem;                    // resident tiled weights
  uint8_t* stg = smem + plan.w_region;    // the stages
  if (warp == 0) tc::tmem_alloc(&tmem_base, (uint32_t)plan.tmem_cols);
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int q = 0; q < 2; q++) {
      tc::mbar_init(&tfull[q], 1);
      tc::mbar_init(&tempty[q], 4);
    }
    tc::mbar_init(&wfull, 1);
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

  if (warp == 4) {   // ---- producer: lane 0 takes the barriers, lanes 0..17 one A copy each
    if (plan.resident && my_tiles > 0 && lane == 0) {
      mbar_expect_tx(&wfull, plan.w_bytes);
      bulk_load(wsm, a.Wt, plan.w_bytes, &wfull);
    }
    // this lane's copy: slab sl = lane / 2, plane q = lane % 2 (lane 18: the
    // streamed weights)
    const int sl = lane >> 1, q = lane & 1;
    const int64_t slab_off = (sl / 3 - 1) * P + (sl % 3 - 1) * (int64_t)a.n3;
    int st = 0, pass = 0, issued = 0;
    bool ok = true;
    for (int k = 0; k < my_tiles && ok; k++) {
      const int64_t row_base = tile_start(k) - 1;
      for (int c = 0; c < nk; c++) {
        if (pass > 0) {
          bool w = true;
          if (lane == 0) w = bk_wait(&empty[st], (uint32_t)((pass - 1) & 1), abort_p);
          if (!__shfl_sync(0xffffffffu, w, 0)) {
            ok = false;
            break;
          }
        }
        uint8_t* sa = stg + st * plan.stage_bytes;
        if (lane == 0) mbar_expect_tx(&full[st], BK_A + (plan.resident ? 0u : plan.b_bytes));
        if (lane < 18)
          bulk_load(sa + sl * BK_SLAB + q * 2048, a.in + (2 * c + q) * a.in_ps + (row_base + slab_off) * 8, 2048,
                    &full[st]);
        else if (lane == 18 && !plan.resident)
          bulk_load(sa + BK_A, a.Wt + (int64_t)c * 9 * N3 * 16, plan.b_bytes, &full[st]);
        issued++;
        if (++st == S) {
          st = 0;
          pass++;
        }
      }
    }
    // every copy issued has landed before the CTA may leave: the last phase
    // of each stage used, and the weights
    if (lane == 0) {
      for (int s = 0; s < S; s++) {
        const int n = issued / S + (s < issued % S ? 1 : 0);   // uses of stage s
        if (n > 0) bk_wait(&full[s], (uint32_t)((n - 1) & 1), abort_p, false);
      }
      if (plan.resident && my_tiles > 0) bk_wait(&wfull, 0, abort_p, false);
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {   // ---- MMA issuer
      const uint32_t idesc = tc::idesc_bf16_f32(128, N3);
      const uint32_t b_lbo = (uint32_t)N3 * 16;
      bool ok = !plan.resident || my_tiles == 0 || bk_wait(&wfull, 0, abort_p);
      int st = 0, pass = 0;
      for (int k = 0; k < my_tiles && ok; k++) {
        const int acc = k & 1;
        if (k >= 2 && !bk_wait(&tempty[acc], (uint32_t)(((k >> 1) - 1) & 1), abort_p)) break;
        tc::fence_after_sync();
        const uint32_t dacc = tbase + (uint32_t)(acc * plan.acc_off);
        for (int c = 0; c < nk; c++) {
          if (!bk_wait(&full[st], (uint32_t)(pass & 1), abort_p)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint8_t* sa = stg + st * plan.stage_bytes;
          const uint8_t* sb = plan.resident ? wsm + (size_t)c * 9 * N3 * 32 : sa + BK_A;
#pragma unroll 1
          for (int sl = 0; sl < 9; sl++) {
            const uint64_t ad = tc::smem_desc(tc::smem_addr(sa + sl * BK_SLAB), 2048, 128);
            const uint64_t bd = tc::smem_desc(tc::smem_addr(sb + sl * N3 * 32), b_lbo, 128);
            tc::mma_bf16(dacc, ad, bd, idesc, c > 0 || sl > 0);
          }
          tc::mma_commit(&empty[st]);
          if (++st == S) {
            st = 0;
            pass++;
          }
        }
        if (ok) tc::mma_commit(&tfull[acc]);
      }
      // every MMA issued has completed before TMEM is freed
      tc::mma_commit(&mdone);
      bk_wait(&mdone, 0, abort_p, false);
    }
    __syncwarp();
  } else {   // ---- epilogue, warps 0-3
    for (int k = 0; k < my_tiles; k++) {
      const int acc = k & 1;
      const bool got = bk_wait(&tfull[acc], (uint32_t)((k >> 1) & 1), abort_p);
      if (!epi_sync_and(got)) break;
      tc::fence_after_sync();
      const int64_t c0 = tile_start(k);
      const uint32_t trow = tbase + (uint32_t)(acc * plan.acc_off) + ((uint32_t)(warp * 32) << 16);
      float(*xc)[2][80] = xch[acc];
      const int r = warp * 32 + lane;
      const int64_t c = c0 + r - 1;
      const bool live = r >= 1 && r <= 126 && c < a.ncell;
      const float m = live ? (float)a.mask[c] : 0.f;
      // the neighbour row a lane needs from another warp: lane 0 warp-1's
      // D_-1 edge, lane 31 warp+1's D_+1 edge (others read one and discard it)
      const float* nbr = lane == 0 ? xc[warp > 0 ? warp - 1 : 0][0] : xc[warp < 3 ? warp + 1 : 3][1];
      const bool has_nbr = lane == 0 ? warp > 0 : warp < 3;
      // 16 output channels at a time: D_-1, D_0 and D_+1 columns in three
      // loads under one wait
      for (int co = 0; co < Co; co += 16) {
        uint32_t dm[16], d0[16], dp[16];
        tc::tmem_ld16_nowait(trow + (uint32_t)co, dm);
        tc::tmem_ld16_nowait(trow + (uint32_t)(Co + co), d0);
        tc::tmem_ld16_nowait(trow + (uint32_t)(2 * Co + co), dp);
        tc::tmem_wait_ld(dm, d0, dp);
        if (lane == 31 || lane == 0) {
          const uint32_t* e = lane == 31 ? dm : dp;
          float4* dst = reinterpret_cast<float4*>(&xc[warp][lane == 31 ? 0 : 1][co]);
#pragma unroll
          for (int j = 0; j < 4; j++)
            dst[j] = make_float4(__uint_as_float(e[4 * j]), __uint_as_float(e[4 * j + 1]),
                                 __uint_as_float(e[4 * j + 2]), __uint_as_float(e[4 * j + 3]));
        }
        epi_sync();
        float nb[16];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float4 w4 = reinterpret_cast<const float4*>(nbr + co)[j];
          nb[4 * j] = w4.x; nb[4 * j + 1] = w4.y; nb[4 * j + 2] = w4.z; nb[4 * j + 3] = w4.w;
        }
        float v[2][8];
#pragma unroll
        for (int q = 0; q < 16; q++) {
          float prev = __shfl_up_sync(0xffffffffu, __uint_as_float(dm[q]), 1);
          float next = __shfl_down_sync(0xffffffffu, __uint_as_float(dp[q]), 1);
          const float e = has_nbr ? nb[q] : 0.f;
          if (lane == 0) prev = e;
          if (lane == 31) next = e;
          v[q >> 3][q & 7] = prev + __uint_as_float(d0[q]) + next;
        }
        if (live && co < a.out_ch) conv_store8(a, c, co, m, v[0]);
        if (live && co + 8 < a.out_ch) conv_store8(a, c, co + 8, m, v[1]);
      }
      // the accumulator is read: the MMA issuer may overwrite it two tiles on
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) atomicExch(a.err, 1);
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, (uint32_t)plan.tmem_cols);
}

// Error flag of the convolutions: a slot of the context scratch, cleared by
// xf_conv_status.
constexpr int I_CONV_ERR = 60;
static int* conv_err_flag(xf_ctx* ctx) { return reinterpret_cast<int*>(&ctx->scratch->iscalars[I_CONV_ERR]); }

// The dynamic shared-memory attribute of a convolution kernel, raised once
// per kernel and device to the largest size asked for (so that the launches
// of a captured solve set no attribute).
static cudaError_t set_max_smem(const void* kern, int which, int device, size_t smem) {
  static size_t done[3][64] = {};
  size_t& d = done[which][device & 63];
  if (smem <= d) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) d = smem;
  return e;
}

// ---------------------------------------------------------------------------
// Weight gradient of the convolution on the tensor cores:
//     dW[t][co][ci] = sum over cells c of g[c][co] x[c + off_t][ci].
// With the activations in channel planes, 8 consecutive cells of one plane
// are also the canonical MN-major core matrix (8 channels along M or N, one
// cell per 16-byte row along K), so the sum over cells is the K dimension of
// an MMA: M = 128 rows of stacked (tap, input channel) pairs (128 / ci taps per
// row tile), N = co, A = the shifted x blocks, B = g.  A stage is 128 cells:
// per (tap, plane) of the row tile and per plane of g one 2 KB bulk copy (one
// per lane of the producer warp), eight MMAs of K = 16 cells.  Each CTA takes
// one row tile and one range of cells (a multiple of 128: the cells past the
// box read the zero margins), accumulates in TMEM, and writes its FP32
// partial; k_wgrad_tc_sum adds the ranges in a fixed order (deterministic).
// Descriptors: no swizzle, MN-major (instruction descriptor bits 15 and 16),
// LBO = the K-direction core-matrix stride (128 bytes), SBO = the MN-direction
// stride (2 KB).
constexpr int WG_KC = 128;                         // cells per stage
constexpr int WG_STAGES = 3;
constexpr uint32_t WG_BLOCK = WG_KC * 16;          // one (tap, plane) block of a stage
constexpr uint32_t WG_A = 16 * WG_BLOCK;           // the row tile's A region (16 blocks)

struct WgArgs {
  const uint16_t* g;   // plane 0, cell 0
  int64_t gps;
  int co;
  const uint16_t* x;
  int64_t xps;
  int ci;
  int n2, n3;
  int taps, mtiles, splits, stages;   // taps per row tile, row tiles, cell ranges, stages per range
  int64_t chunks;                      // 128-cell stages in all
  uint32_t stage_bytes;
  float* partial;   // [mtile][split][128][co]
  int* err;
};

__global__ void __launch_bounds__(BK_THREADS) k_wgrad_tc(WgArgs a) {
  extern __shared__ uint8_t dsm[];
  __shared__ uint64_t full[WG_STAGES], empty[WG_STAGES], mdone;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % a.mtiles, sp = blockIdx.x / a.mtiles;
  const int cp = a.ci / 8, t0 = mt * a.taps, tn = min(27, t0 + a.taps) - t0;
  const int ga = tn * cp, gb = a.co / 8;   // blocks of A and of B per stage
  const uint32_t raw = tc::smem_addr(dsm);
  uint8_t* smem = dsm + ((1024u - (raw & 1023u)) & 1023u);
  const uint32_t ncols = tmem_cols(a.co);
  if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
  if (threadIdx.x == 0) {
    for (int st = 0; st < WG_STAGES; st++) {
      tc::mbar_init(&full[st], 1);
      tc::mbar_init(&empty[st], 1);
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
  const int64_t cell0 = (int64_t)sp * a.stages * WG_KC;
  // this range's stages: the last range stops at the box's last 128-cell chunk
  const int my_stages = (int)min((int64_t)a.stages, a.chunks - (int64_t)sp * a.stages);
  if (warp == 4) {   // ---- producer: one copy per lane
    const bool is_a = lane < ga, is_b = lane >= ga && lane < ga + gb;
    const uint16_t* src = nullptr;
    uint32_t dst_off = 0;
    if (is_a) {
      const int t = t0 + lane / cp, q = lane % cp;
      const int64_t off = (t / 9 - 1) * P + ((t / 3) % 3 - 1) * (int64_t)a.n3 + (t % 3 - 1);
      src = a.x + q * a.xps + off * 8;
      dst_off = (uint32_t)lane * WG_BLOCK;
    } else if (is_b) {
      const int q = lane - ga;
      src = a.g + q * a.gps;
      dst_off = WG_A + (uint32_t)q * WG_BLOCK;
    }
    int st = 0, pass = 0, issued = 0;
    for (int k = 0; k < my_stages; k++) {
      if (pass > 0) {
        bool w = true;
        if (lane == 0) w = bk_wait(&empty[st], (uint32_t)((pass - 1) & 1), abort_p);
        if (!__shfl_sync(0xffffffffu, w, 0)) break;
      }
      uint8_t* sa = smem + st * a.stage_bytes;
      if (lane == 0) mbar_expect_tx(&full[st], (uint32_t)(ga + gb) * WG_BLOCK);
      if (is_a || is_b) bulk_load(sa + dst_off, src + (cell0 + (int64_t)k * WG_KC) * 8, WG_BLOCK, &full[st]);
      issued++;
      if (++st == WG_STAGES) {
        st = 0;
        pass++;
      }
    }
    if (lane == 0)   // every copy issued has landed before the CTA may leave
      for (int s2 = 0; s2 < WG_STAGES; s2++) {
        const int n = issued / WG_STAGES + (s2 < issued % WG_STAGES ? 1 : 0);
        if (n > 0) bk_wait(&full[s2], (uint32_t)((n - 1) & 1), abort_p, false);
      }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {   // ---- MMA issuer
      const uint32_t idesc = tc::idesc_bf16_f32(128, a.co) | (1u << 15) | (1u << 16);   // A and B MN-major
      int st = 0, pass = 0;
      for (int k = 0; k < my_stages; k++) {
        if (!bk_wait(&full[st], (uint32_t)(pass & 1), abort_p)) break;
        tc::fence_after_sync();
        const uint8_t* sa = smem + st * a.stage_bytes;
#pragma unroll 1
        for (int kk = 0; kk < WG_KC / 16; kk++) {
          const uint64_t ad = tc::smem_desc(tc::smem_addr(sa + kk * 256), 128, WG_BLOCK);
          const uint64_t bd = tc::smem_desc(tc::smem_addr(sa + WG_A + kk * 256), 128, WG_BLOCK);
          tc::mma_bf16(tbase, ad, bd, idesc, k > 0 || kk > 0);
        }
        tc::mma_commit(&empty[st]);
        if (++st == WG_STAGES) {
          st = 0;
          pass++;
        }
      }
      tc::mma_commit(&mdone);   // every MMA issued
    }
    __syncwarp();
  } else {   // ---- epilogue, warps 0-3: the partial of this tile and range
    const bool got = bk_wait(&mdone, 0, abort_p, false);
    if (__all_sync(0xffffffffu, got) && !*abort_p) {
      tc::fence_after_sync();
      const int row = warp * 32 + lane;
      float* dst = a.partial + (((int64_t)mt * a.splits + sp) * 128 + row) * a.co;
      for (int co = 0; co < a.co; co += 8) {
        float v[8];
        tc::tmem_ld8(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)co, v);
        *reinterpret_cast<float4*>(dst + co) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4*>(dst + co + 4) = make_float4(v[4], v[5], v[6], v[7]);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) atomicExch(a.err, 1);
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

// gw[t][co][ci] += the ranges' partials in range order.
__global__ void k_wgrad_tc_sum(const float* __restrict__ partial, int mtiles, int splits, int taps, int ci, int co,
                               float* __restrict__ gw) {
  const int64_t n = (int64_t)27 * co * ci;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(u / ((int64_t)co * ci));
    const int o = (int)((u / ci) % co), i = (int)(u % ci);
    const int mt = t / taps, row = (t - mt * taps) * ci + i;
    float s = 0.f;
    for (int sp = 0; sp < splits; sp++) s += partial[(((int64_t)mt * splits + sp) * 128 + row) * co + o];
    gw[u] += s;
  }
}

// The row tiles and cell ranges of a layer's weight gradient, and the FP32
// partial buffer it needs (floats).
void xf_wgrad_tc_plan(const xf_ctx* ctx, int64_t ncell, int ci, int co, int* mtiles, int* splits, int* stages,
                      int64_t* partial_floats) {
  const int taps = 128 / ci;
  *mtiles = (27 + taps - 1) / taps;
  const int64_t chunks = (ncell + WG_KC - 1) / WG_KC;
  int64_t sp = ((int64_t)ctx->sm_count * 2 + *mtiles - 1) / *mtiles;
  if (sp > chunks) sp = chunks;
  if (sp < 1) sp = 1;
  *stages = (int)((chunks + sp - 1) / sp);
  *splits = (int)((chunks + *stages - 1) / *stages);
  *partial_floats = (int64_t)*mtiles * *splits * 128 * co;
}

// gw ([27][co][ci] FP32) += the weight gradient of g (co channels) against x
// (ci channels), both BF16 planes with their zero margins; partial holds
// xf_wgrad_tc_plan's floats.  ci and co multiples of 16, ci <= 128, co <= 64.
int xf_wgrad_tc(xf_ctx* ctx, int n1, int n2, int n3, const void* g, int64_t gps, int co, const void* x, int64_t xps,
                int ci, float* partial, float* gw) {
  if (ci % 16 || co % 16 || ci < 16 || ci > 128 || co < 16 || co > 64)
    return xf_fail(ctx, XF_ERR_ARG, "weight gradient: channel counts out of range");
  WgArgs a;
  a.g = (const uint16_t*)g; a.gps = gps; a.co = co;
  a.x = (const uint16_t*)x; a.xps = xps; a.ci = ci;
  a.n2 = n2; a.n3 = n3;
  int64_t pf = 0;
  xf_wgrad_tc_plan(ctx, (int64_t)n1 * n2 * n3, ci, co, &a.mtiles, &a.splits, &a.stages, &pf);
  a.taps = 128 / ci;
  a.chunks = ((int64_t)n1 * n2 * n3 + WG_KC - 1) / WG_KC;
  a.stage_bytes = (WG_A + (uint32_t)co / 8 * WG_BLOCK + 1023) / 1024 * 1024;
  a.partial = partial;
  a.err = conv_err_flag(ctx);
  const size_t smem = (size_t)WG_STAGES * a.stage_bytes + 1024;
  XF_CUDA(ctx, set_max_smem((const void*)k_wgrad_tc, 2, ctx->device, smem));
  k_wgrad_tc<<<a.mtiles * a.splits, BK_THREADS, smem, ctx->stream>>>(a);
  const int64_t nw = (int64_t)27 * co * ci;
  k_wgrad_tc_sum<<<(unsigned)((nw + 255) / 256), 256, 0, ctx->stream>>>(partial, a.mtiles, a.splits, a.taps, ci, co,
                                                                        gw);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// Launch on the context stream (arguments checked by the caller).  `weights`
// is [27][co][ci]; `tiled` the same in the tiled order (needed when 3 co <= 256).
int xf_conv_launch(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int64_t in_ps, int ci, const void* weights,
                   const void* tiled, const float* bias, int co, const uint8_t* mask, void* out, int64_t out_pitch,
                   int out_ch, int out_fp32, int relu, const void* gate, int64_t gate_ps) {
  int* err = conv_err_flag(ctx);
  ConvArgs a;
  a.gate = (const uint16_t*)gate; a.gate_ps = gate_ps;
  a.in = (const uint16_t*)in; a.in_ps = in_ps; a.Ci = ci;
  a.W = (const uint16_t*)weights; a.Wt = (const uint16_t*)tiled; a.bias = bias; a.Co = co;
  a.mask = mask; a.n2 = n2; a.n3 = n3; a.ncell = (int64_t)n1 * n2 * n3;
  a.out16 = out_fp32 ? nullptr : (uint16_t*)out;
  a.out32 = out_fp32 ? (float*)out : nullptr;
  a.out_ps = out_fp32 ? 0 : out_pitch;
  a.out_ld = out_fp32 ? (int)out_pitch : 0;
  a.out_ch = out_ch; a.relu = relu; a.err = err;
  if (3 * co <= 256) {
    // k-taps stacked along N, operands by bulk copies (the per-tap kernel
    // below takes wider outputs)
    static int static_smem = -1;
    if (static_smem < 0) {
      cudaFuncAttributes fa;
      XF_CUDA(ctx, cudaFuncGetAttributes(&fa, k_conv3_bulk));
      static_smem = (int)fa.sharedSizeBytes;
    }
    const BkPlan plan = bk_plan(ci, co, static_smem);
    if (plan.stages < 2 || !tiled) return xf_fail(ctx, XF_ERR_ARG, "convolution: no stacked-tap plan");
    XF_CUDA(ctx, set_max_smem((const void*)k_conv3_bulk, 0, ctx->device, (size_t)plan.smem_bytes));
    const int64_t tiles = (a.ncell + 125) / 126;
    int64_t blocks = (int64_t)ctx->sm_count * plan.per_sm;
    if (blocks > tiles) blocks = tiles;
    k_conv3_bulk<<<(int)blocks, BK_THREADS, plan.smem_bytes, ctx->stream>>>(a, plan);
    XF_CUDA(ctx, cudaGetLastError());
    return XF_OK;
  }
  const size_t smem = (size_t)CONV_STAGES * (TC_M * ci * 2 + co * ci * 2);
  XF_CUDA(ctx, set_max_smem((const void*)k_conv3_tc, 1, ctx->device, smem));
  // Residency from the kernel's real limits: shared memory (227 KB per SM, with
  // ~1 KB static and reserved per CTA), tensor-memory columns (512 per SM) and
  // threads (2048 per SM).
  int per_sm = (int)((227 * 1024) / (smem + 2048));
  per_sm = min(per_sm, (int)(512 / tmem_cols(co)));
  per_sm = min(per_sm, 16);
  if (per_sm < 1) per_sm = 1;
  const int64_t ntiles = (a.ncell + TC_M - 1) / TC_M;
  int64_t blocks = (int64_t)ctx->sm_count * per_sm;
  if (blocks > ntiles) blocks = ntiles;
  k_conv3_tc<<<(int)blocks, 128, smem, ctx->stream>>>(a);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// Weights [27][co][ci] into the tiled order (conv_tiled_index).
__global__ void k_tile_weights(const uint16_t* __restrict__ w, int co, int ci, uint16_t* __restrict__ wt) {
  const int64_t n = (int64_t)27 * co * ci;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(u / ((int64_t)co * ci));
    const int o = (int)((u / ci) % co), i = (int)(u % ci);
    wt[conv_tiled_index(t, o, i, co, ci)] = w[u];
  }
}

extern "C" int xf_conv3d_bf16(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int64_t in_ps, int ci,
                              const void* weights, const float* bias, int co, const uint8_t* mask, void* out,
                              int64_t out_pitch, int out_ch, int out_fp32, int relu) {
  if (!ctx || !in || !weights || !mask || !out) return XF_ERR_ARG;
  const int64_t ncell = (int64_t)n1 * n2 * n3;
  const int64_t rows_min = ncell + XF_CONV_MARGIN(n2, n3);   // a plane's rows from cell 0 on
  if (ci < 16 || ci > 128 || ci % 16 || co < 16 || co > 128 || co % 16 || out_ch < 1 || out_ch > co ||
      n1 < 3 || n2 < 3 || n3 < 3 || in_ps < (rows_min + XF_CONV_MARGIN(n2, n3)) * 8 || in_ps % 8 ||
      (out_fp32 ? out_pitch < out_ch : (out_pitch < ncell * 8 || out_pitch % 8 || out_ch % 8)))
    return xf_fail(ctx, XF_ERR_ARG, "xf_conv3d_bf16: channel counts / plane strides out of range");
  if (((uintptr_t)in | (uintptr_t)weights | (uintptr_t)out) & 15)
    return xf_fail(ctx, XF_ERR_ARG, "xf_conv3d_bf16: pointers must be 16-byte aligned");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  void* tiled = nullptr;
  const int64_t nw = (int64_t)27 * co * ci;
  if (3 * co <= 256) {
    XF_CUDA(ctx, cudaMallocAsync(&tiled, nw * 2, ctx->stream));
    k_tile_weights<<<(unsigned)((nw + 255) / 256), 256, 0, ctx->stream>>>((const uint16_t*)weights, co, ci,
                                                                          (uint16_t*)tiled);
  }
  const int st = xf_conv_launch(ctx, n1, n2, n3, in, in_ps, ci, weights, tiled, bias, co, mask, out, out_pitch,
                                out_ch, out_fp32, relu, nullptr, 0);
  if (tiled) cudaFreeAsync(tiled, ctx->stream);
  return st;
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
