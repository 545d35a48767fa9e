// Tensor-core (tcgen05) kernels of the learned preconditioner.
//
// xf_tc_gemm_bf16: one 128 x N x K tile, D = A B^T with BF16 A (128 x K) and
// B (N x K), K contiguous, FP32 accumulation in tensor memory.  It is the
// building block the implicit-GEMM convolutions below use, exposed so that
// its operand layout and descriptors are checked on their own.
#include <cuda_bf16.h>

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
