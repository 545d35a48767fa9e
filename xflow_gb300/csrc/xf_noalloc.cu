// xf_dot_noalloc: the masked FP64 inner product of xf_dot for callers that
// cannot allocate device memory: a host application that carves all of its
// device memory out of its own pool at start-up (a time loop run under a
// fixed memory budget, or a GPU shared with another library that holds the
// rest, where a new allocation fails part-way through a step), and loops
// that must not call cudaFree, which waits for the whole device to go idle.
// It takes caller-owned device
// arrays and a caller-owned device result, and keeps its scratch (the
// per-block partial sums and the last-block ticket) in a file-scope
// __device__ array, so it calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// Limits and sharing:
//  * n <= XF_NOALLOC_MAX_ELEMS (XF_NOALLOC_MAX_BLOCKS blocks of 256 threads x
//    16 elements); larger n is rejected with XF_ERR_ARG.
//  * The scratch (8192 doubles + a counter, 64 KiB) lives on every device that
//    loads the library until the process exits.
//  * Every call shares it: calls whose kernels overlap on the GPU (different
//    streams, or different host threads on one device) race and give wrong
//    sums.  Calls ordered on one stream are safe; the ticket is returned to
//    zero by each call's last block.
//  * The first call on a device resolves the scratch's device address with
//    cudaGetSymbolAddress (with that device current) and keeps it; make that
//    first call before any stream capture.  The address belongs to the
//    device's primary context: after cudaDeviceReset the process must be
//    restarted before it calls this entry point again.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xflow.h"

#define XF_NOALLOC_MAX_BLOCKS 8192
#define XF_NOALLOC_THREADS 256
#define XF_NOALLOC_PER_THREAD 16

struct NoallocScratch {
  double partials[XF_NOALLOC_MAX_BLOCKS];
  unsigned int ticket;
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

__device__ static double nb_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ static double nb_block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = nb_warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = nb_warp_sum(v);
  return v;
}

// Each block sums a contiguous run of XF_NOALLOC_THREADS * XF_NOALLOC_PER_THREAD
// elements; the last block to finish adds the partials in block order.
__global__ void __launch_bounds__(XF_NOALLOC_THREADS) k_dot_noalloc(const double* __restrict__ a,
                                                                  const double* __restrict__ b,
                                                                  const uint8_t* __restrict__ m, int64_t n,
                                                                  double* __restrict__ out, NoallocScratch* scr) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int64_t base = (int64_t)blockIdx.x * XF_NOALLOC_THREADS * XF_NOALLOC_PER_THREAD;
  double acc = 0.0;
#pragma unroll
  for (int q = 0; q < XF_NOALLOC_PER_THREAD; q++) {
    const int64_t c = base + (int64_t)q * XF_NOALLOC_THREADS + threadIdx.x;
    if (c < n && (m == nullptr || m[c])) acc += a[c] * b[c];
  }
  const double s = nb_block_sum(acc, sh);
  if (threadIdx.x == 0) {
    scr->partials[blockIdx.x] = s;
    __threadfence();
    const unsigned int t = atomicAdd(&scr->ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) v += __ldcg(&scr->partials[k]);
  v = nb_block_sum(v, sh);
  if (threadIdx.x == 0) {
    *out = v;
    scr->ticket = 0;   // the next call starts from zero
  }
}

// Device address of the scratch, resolved once per device.
#define XF_NOALLOC_MAX_DEVICES 64
static NoallocScratch* g_scratch_ptr[XF_NOALLOC_MAX_DEVICES];

extern "C" int xf_dot_noalloc(const double* d_a, const double* d_b, const uint8_t* d_mask, int64_t n, double* d_out,
                              void* stream) {
  if (!d_a || !d_b || !d_out || n < 0) return XF_ERR_ARG;
  const int64_t max_elems = (int64_t)XF_NOALLOC_MAX_BLOCKS * XF_NOALLOC_THREADS * XF_NOALLOC_PER_THREAD;
  if (n > max_elems) return XF_ERR_ARG;   // beyond the static scratch: XF_NOALLOC_MAX_ELEMS
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return XF_ERR_CUDA;
  if (dev < 0 || dev >= XF_NOALLOC_MAX_DEVICES) return XF_ERR_UNSUPPORTED;
  if (!g_scratch_ptr[dev]) {
    NoallocScratch* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_noalloc_scratch) != cudaSuccess || !p) return XF_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  const int64_t per_block = (int64_t)XF_NOALLOC_THREADS * XF_NOALLOC_PER_THREAD;
  int blocks = (int)((n + per_block - 1) / per_block);
  if (blocks < 1) blocks = 1;
  // launched through cudaLaunchKernel so that its own status is returned (an
  // earlier, unrelated error is neither reported nor cleared here)
  NoallocScratch* scr = g_scratch_ptr[dev];
  void* args[] = {(void*)&d_a, (void*)&d_b, (void*)&d_mask, (void*)&n, (void*)&d_out, (void*)&scr};
  return cudaLaunchKernel((const void*)k_dot_noalloc, dim3(blocks), dim3(XF_NOALLOC_THREADS), args, 0,
                          (cudaStream_t)stream) == cudaSuccess
             ? XF_OK
             : XF_ERR_CUDA;
}
