// Measurement probes behind design decisions (no counterpart in the
// reference): the tcgen05.mma issue rate versus N, which made the U-Net
// convolution stack its three k-taps along N, and the FP64 / FP32 FMA rates,
// which made the solvers' hot paths FP32 with FP64 only where correctness
// needs it.  Each returns numbers; bench.py --probes prints them.
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "xf_common.cuh"
#include "xf_tc.cuh"

namespace {

constexpr int PR_A_BYTES = 16384;   // A operand: 128 rows x 64 BF16 (four K = 16 slices)
constexpr int PR_B_BYTES = 32768;   // B operand: up to 256 rows x 64 BF16

// Thread 0 issues `iters` x 4 back-to-back MMAs (M = 128, K = 16, BF16 in,
// FP32 accumulate in TMEM) on operands resident in shared memory, commits,
// waits on an mbarrier (bounded) and records its clock64 cycles and SM.
// layout 0: interleaved no-swizzle K-major (LBO 128 B, SBO 1 KB); layout 1:
// column of chunks (LBO rows x 16 B, SBO 128 B).
__global__ void __launch_bounds__(128) k_probe_mma(int N, int iters, int layout, unsigned long long* out) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tbase;
  uint16_t* s16 = reinterpret_cast<uint16_t*>(smem);
  for (int i = threadIdx.x; i < (PR_A_BYTES + PR_B_BYTES) / 2; i += blockDim.x) s16[i] = 0x3c00;   // BF16 1.0
  const uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&tbase, ncols);
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x == 0) {
    const uint32_t A = tc::smem_addr(smem), B = tc::smem_addr(smem + PR_A_BYTES);
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    const uint32_t lboA = layout ? 128 * 16 : 128, sboA = layout ? 128 : 1024;
    const uint32_t lboB = layout ? (uint32_t)N * 16 : 128, sboB = layout ? 128 : 1024;
    const unsigned long long t0 = clock64();
    for (int it = 0; it < iters; it++)
      for (int kk = 0; kk < 4; kk++) {
        const uint64_t ad = tc::smem_desc(A + kk * 2 * lboA, lboA, sboA);
        const uint64_t bd = tc::smem_desc(B + kk * 2 * lboB, lboB, sboB);
        tc::mma_bf16(tbase, ad, bd, idesc, it > 0 || kk > 0);
      }
    tc::mma_commit(&mbar);
    bool ok = tc::mbar_wait(&mbar, 0);
    const unsigned long long dt = clock64() - t0;
    if (!ok) ok = tc::mbar_wait(&mbar, 0);   // let the MMAs finish before TMEM is released (bounded)
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    out[2 * blockIdx.x] = ok ? dt : 0;
    out[2 * blockIdx.x + 1] = smid;
  }
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tbase, ncols);
}

// Eight independent FMA chains per thread, `iters` steps each.
template <typename T>
__global__ void k_probe_fma(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int fma_rate(xf_ctx* ctx, double* tflops) {
  const int blocks = ctx->sm_count * 8, threads = 256, iters = 4096, reps = 5;
  T* out = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&out, sizeof(T) * blocks * threads, ctx->stream));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_probe_fma<T><<<blocks, threads, 0, ctx->stream>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e0, ctx->stream);
  for (int r = 0; r < reps; r++) k_probe_fma<T><<<blocks, threads, 0, ctx->stream>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1, ctx->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, ctx->stream);
  if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess)
    return xf_fail(ctx, XF_ERR_CUDA, "xf_probe_fma_rate: %s", cudaGetErrorString(e));
  *tflops = (double)reps * blocks * threads * iters * 8 * 2 / (ms * 1e-3) / 1e12;
  return XF_OK;
}

}  // namespace

extern "C" int xf_probe_mma_rate(xf_ctx* ctx, int n, int ctas_per_sm, int layout, double* cycles_per_mma) {
  if (!ctx || !cycles_per_mma || (n != 16 && n != 32 && n != 64 && n != 128 && n != 256) || ctas_per_sm < 1 ||
      (layout != 0 && layout != 1))
    return XF_ERR_ARG;
  const int ncols = n <= 32 ? 32 : n;
  if (ncols * ctas_per_sm > 512 || ctas_per_sm > 4)   // TMEM columns and shared memory of one SM
    return xf_fail(ctx, XF_ERR_ARG, "xf_probe_mma_rate: %d CTAs of %d TMEM columns do not fit one SM", ctas_per_sm, ncols);
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int smem = PR_A_BYTES + PR_B_BYTES;
  XF_CUDA(ctx, cudaFuncSetAttribute(k_probe_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int grid = ctx->sm_count * ctas_per_sm, iters = n <= 32 ? 1024 : 512;
  unsigned long long* d = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&d, 2 * sizeof(unsigned long long) * grid, ctx->stream));
  k_probe_mma<<<grid, 128, smem, ctx->stream>>>(n, iters, layout, d);
  std::vector<unsigned long long> h(2 * (size_t)grid);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFreeAsync(d, ctx->stream);
  if (e != cudaSuccess) return xf_fail(ctx, XF_ERR_CUDA, "xf_probe_mma_rate: %s", cudaGetErrorString(e));
  // per SM: the MMAs issued there over its longest CTA's cycles, averaged over SMs
  std::vector<unsigned long long> mx(4096, 0), cnt(4096, 0);
  for (int b = 0; b < grid; b++) {
    if (!h[2 * b]) return xf_fail(ctx, XF_ERR_CUDA, "xf_probe_mma_rate: an MMA wait ran out");
    const size_t sm = h[2 * b + 1] < 4096 ? h[2 * b + 1] : 4095;
    mx[sm] = std::max(mx[sm], h[2 * b]);
    cnt[sm]++;
  }
  double rate = 0;
  int nsm = 0;
  for (int s = 0; s < 4096; s++)
    if (cnt[s]) {
      rate += (double)cnt[s] * iters * 4 / (double)mx[s];
      nsm++;
    }
  *cycles_per_mma = nsm ? nsm / rate : 0.0;
  return XF_OK;
}

extern "C" int xf_probe_fma_rate(xf_ctx* ctx, int fp64, double* tflops) {
  if (!ctx || !tflops) return XF_ERR_ARG;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  return fp64 ? fma_rate<double>(ctx, tflops) : fma_rate<float>(ctx, tflops);
}
