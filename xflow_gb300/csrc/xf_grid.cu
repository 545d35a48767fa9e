// Context, grid (T3dNormalGrid + TRnRelease3dSpaceModel) and vector
// (TRnRelease3dSpace) management, and the GPU Rn numbering.
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>

#include <vector>

#include "xf_common.cuh"

int xf_fail(xf_ctx* ctx, int status, const char* fmt, ...) {
  if (ctx) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
    va_end(ap);
  }
  return status;
}

extern "C" const char* xf_status_string(int s) {
  switch (s) {
    case XF_OK: return "ok";
    case XF_ERR_ARG: return "bad argument";
    case XF_ERR_CUDA: return "CUDA error";
    case XF_ERR_MASK: return "grid row the operator is not defined for";
    case XF_ERR_NOMEM: return "out of device memory";
    case XF_ERR_STATE: return "object mismatch";
    case XF_ERR_UNSUPPORTED: return "unsupported combination";
    case XF_ERR_CHECK: return "border-condition check failed";
    case XF_STALL: return "solver stalled";
    case XF_DIVERGED: return "solver diverged";
    case XF_NAN: return "NaN in solver";
    case XF_MAXIT: return "iteration cap reached";
    case XF_BREAKDOWN: return "solver breakdown";
    default: return "unknown status";
  }
}

extern "C" const char* xf_last_error(const xf_ctx* ctx) { return ctx ? ctx->err : "no context"; }

extern "C" int xf_create(int device, xf_ctx** out) {
  if (!out) return XF_ERR_ARG;
  *out = nullptr;
  xf_ctx* ctx = new xf_ctx();
  memset(ctx->err, 0, sizeof(ctx->err));
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete ctx; return XF_ERR_CUDA; }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { delete ctx; return XF_ERR_CUDA; }
  ctx->sm_count = prop.multiProcessorCount;
  // Solver work vectors come from the device's default pool (cudaMallocAsync):
  // keep what one solve frees for the next instead of unmapping it at every
  // synchronisation (an attribute of this process's pool).
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return XF_ERR_CUDA; }
  if (cudaMalloc(&ctx->scratch, sizeof(DevScratch)) != cudaSuccess) { delete ctx; return XF_ERR_NOMEM; }
  cudaMemsetAsync(ctx->scratch, 0, sizeof(DevScratch), ctx->stream);
  if (cudaMallocHost(&ctx->host_scalars, 256 * sizeof(double)) != cudaSuccess) { delete ctx; return XF_ERR_NOMEM; }
  cudaEventCreate(&ctx->ev0);
  cudaEventCreate(&ctx->ev1);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { delete ctx; return XF_ERR_CUDA; }
  *out = ctx;
  return XF_OK;
}

void* xf_ctx_work(xf_ctx* ctx, size_t bytes) {
  if (ctx->work_bytes >= bytes) return ctx->work;
  if (ctx->work) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->work);
  }
  ctx->work = nullptr;
  ctx->work_bytes = 0;
  if (cudaMalloc(&ctx->work, bytes) != cudaSuccess) {
    cudaGetLastError();
    ctx->work = nullptr;
    return nullptr;
  }
  ctx->work_bytes = bytes;
  return ctx->work;
}

extern "C" int xf_destroy(xf_ctx* ctx) {
  if (!ctx) return XF_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->scratch);
  if (ctx->work) cudaFree(ctx->work);
  cudaFreeHost(ctx->host_scalars);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return XF_OK;
}

extern "C" int xf_synchronize(xf_ctx* ctx) {
  if (!ctx) return XF_ERR_ARG;
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" void* xf_stream(xf_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// ---------------------------------------------------------------------------
// Classification: one pass over the codes computes the kind byte, the space
// mask, the boundary-row flag, and the first cell each operator rejects.
// The checks restate XOperator.cpp:971-1123 / 1933-2227 and
// XSpaceModel.cpp:283-319, plus index-range checks for reads the reference
// would make outside its arrays.
__global__ void k_classify(const int32_t* __restrict__ codes, const double* __restrict__ nrm, int n1, int n2,
                           int n3, uint8_t* __restrict__ kind, uint8_t* __restrict__ smask,
                           uint8_t* __restrict__ isb, unsigned long long* bad /* [2] */) {
  const int64_t n = (int64_t)n1 * n2 * n3, s1 = (int64_t)n2 * n3, s2 = n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / s1), j = (int)((c / s2) % n2), k = (int)(c % n3);
    const int m = codes[c];
    const bool known = (m == 0 || m == 1 || m == 3 || m == 4 || m == 5 || m == 6 || m == 7 || m == 8);
    const bool act = (m == 1 || m == 4 || m == 5 || m == 6 || m == 8);
    const bool interior = i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 2;
    bool ok_l = true, ok_v = true;
    uint8_t kb = 0;
    int row = ROW_NONE;
    if (!known || m == 5 || m == 8) {
      ok_l = ok_v = false;
    } else if (m == 1) {
      ok_l = ok_v = interior;
      row = ROW_ACTUAL;
      if (interior) {
        kb |= codes[c - s1] != 0 ? K_MX : 0;
        kb |= codes[c + s1] != 0 ? K_PX : 0;
        kb |= codes[c - s2] != 0 ? K_MY : 0;
        kb |= codes[c + s2] != 0 ? K_PY : 0;
        kb |= codes[c - 1] != 0 ? K_MZ : 0;
        kb |= codes[c + 1] != 0 ? K_PZ : 0;
      }
    } else if (m == 4 || m == 6) {
      const double nx = nrm ? nrm[3 * c] : 0.0, ny = nrm ? nrm[3 * c + 1] : 0.0, nz = nrm ? nrm[3 * c + 2] : 0.0;
      bool ok = !(nx == 0 && ny == 0 && nz == 0);
      if (ok && m == 4) {
        if (nx != 0) ok = (ny == 0 && nz == 0 && fabs(nx) == 1);
        else if (ny != 0) ok = (nx == 0 && nz == 0 && fabs(ny) == 1);
        else ok = (nx == 0 && ny == 0 && fabs(nz) == 1);
        if (ok) {
          const int di = nx > 0 ? -1 : nx < 0 ? 1 : 0, dj = ny > 0 ? -1 : ny < 0 ? 1 : 0, dk = nz > 0 ? -1 : nz < 0 ? 1 : 0;
          ok = i + di >= 0 && i + di < n1 && j + dj >= 0 && j + dj < n2 && k + dk >= 0 && k + dk < n3;
        }
        ok_l = ok_v = ok;
        row = ROW_PREDEF;
      } else if (ok) {
        const int lo_i = nx > 0 ? -1 : 0, hi_i = nx < 0 ? 1 : 0;
        const int lo_j = ny > 0 ? -1 : 0, hi_j = ny < 0 ? 1 : 0;
        const int lo_k = nz > 0 ? -1 : 0, hi_k = nz < 0 ? 1 : 0;
        ok = i + lo_i >= 0 && i + hi_i < n1 && j + lo_j >= 0 && j + hi_j < n2 && k + lo_k >= 0 && k + hi_k < n3;
        ok_l = ok;
        ok_v = ok && interior;
        row = ROW_PRENORM;
      } else {
        ok_l = ok_v = false;
        row = m == 4 ? ROW_PREDEF : ROW_PRENORM;
      }
    }
    if (!ok_l) atomicMin(&bad[0], (unsigned long long)c);
    if (!ok_v) atomicMin(&bad[1], (unsigned long long)c);
    kind[c] = kb | (uint8_t)(row << K_ROW_SHIFT);
    smask[c] = act ? 1 : 0;
    isb[c] = (row == ROW_PREDEF || row == ROW_PRENORM) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of 0/1 flags in flat (i->j->k) order, three passes.
constexpr int SCAN_TILE = 4096;
constexpr int SCAN_THREADS = 512;  // 8 flags per thread

__global__ void k_scan_count(const uint8_t* __restrict__ f, int64_t n, int32_t* __restrict__ tile_cnt) {
  __shared__ int sh[32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int cnt = 0;
  for (int t = threadIdx.x; t < SCAN_TILE; t += blockDim.x) {
    int64_t c = base + t;
    if (c < n) cnt += f[c] ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    tile_cnt[blockIdx.x] = s;
  }
}

// Single block: exclusive scan of tile counts (int64 offsets), total at [ntile].
__global__ void k_scan_tiles(const int32_t* __restrict__ cnt, int64_t ntile, int64_t* __restrict__ off) {
  __shared__ int64_t carry;
  __shared__ int64_t sh[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < ntile; b0 += blockDim.x) {
    int64_t t = b0 + threadIdx.x;
    int64_t v = t < ntile ? cnt[t] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      int64_t a = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += a;
      __syncthreads();
    }
    if (t < ntile) off[t] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += sh[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) off[ntile] = carry;
}

// Per tile: rank = tile offset + exclusive scan within the tile.  Writes
// out[c] = rank + base_value for flagged cells and `off_value` otherwise.
__global__ void k_scan_apply(const uint8_t* __restrict__ f, int64_t n, const int64_t* __restrict__ off,
                             int32_t* __restrict__ out, int32_t base_value, int32_t off_value) {
  __shared__ int wsum[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  constexpr int PER = SCAN_TILE / SCAN_THREADS;
  const int64_t c0 = base + (int64_t)threadIdx.x * PER;
  int flags[PER];
  int local = 0;
#pragma unroll
  for (int q = 0; q < PER; q++) {
    int64_t c = c0 + q;
    flags[q] = (c < n && f[c]) ? 1 : 0;
    local += flags[q];
  }
  // inclusive warp scan of per-thread counts
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = local;
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    int v = lane < SCAN_THREADS / 32 ? wsum[lane] : 0;
    int incw = v;
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, incw, o);
      if (lane >= o) incw += u;
    }
    if (lane < SCAN_THREADS / 32) wsum[lane] = incw - v;
  }
  __syncthreads();
  int64_t r = off[blockIdx.x] + wsum[w] + (inc - local);
#pragma unroll
  for (int q = 0; q < PER; q++) {
    int64_t c = c0 + q;
    if (c < n) {
      out[c] = flags[q] ? (int32_t)(r + base_value) : off_value;
      r += flags[q];
    }
  }
}

// Exclusive-scan numbering: out[c] = (rank among flagged) + base_value for
// flagged cells, off_value elsewhere; returns the count.
static int scan_number(xf_ctx* ctx, const uint8_t* d_flags, int64_t n, int32_t* d_out, int32_t base_value,
                       int32_t off_value, int64_t* count) {
  const int64_t ntile = (n + SCAN_TILE - 1) / SCAN_TILE;
  int32_t* d_cnt = nullptr;
  int64_t* d_off = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&d_cnt, ntile * sizeof(int32_t), ctx->stream));
  XF_CUDA(ctx, cudaMallocAsync(&d_off, (ntile + 1) * sizeof(int64_t), ctx->stream));
  k_scan_count<<<(unsigned)ntile, SCAN_THREADS, 0, ctx->stream>>>(d_flags, n, d_cnt);
  k_scan_tiles<<<1, 1024, 0, ctx->stream>>>(d_cnt, ntile, d_off);
  k_scan_apply<<<(unsigned)ntile, SCAN_THREADS, 0, ctx->stream>>>(d_flags, n, d_off, d_out, base_value, off_value);
  int64_t total = 0;
  XF_CUDA(ctx, cudaMemcpyAsync(&total, d_off + ntile, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaFreeAsync(d_cnt, ctx->stream));
  XF_CUDA(ctx, cudaFreeAsync(d_off, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  XF_CUDA(ctx, cudaGetLastError());
  *count = total;
  return XF_OK;
}

__global__ void k_gather_normals(const double* __restrict__ nrm, const int32_t* __restrict__ brow_of, int64_t n,
                                 double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    int32_t b = brow_of[c];
    if (b >= 0) {
      out[3 * b] = nrm ? nrm[3 * c] : 0.0;
      out[3 * b + 1] = nrm ? nrm[3 * c + 1] : 0.0;
      out[3 * b + 2] = nrm ? nrm[3 * c + 2] : 0.0;
    }
  }
}

__global__ void k_rn_fwd(const int32_t* __restrict__ inv, int64_t n, int n2, int n3, int32_t* __restrict__ fwd) {
  const int64_t s1 = (int64_t)n2 * n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = inv[c];
    if (r > 0) {
      fwd[3 * (int64_t)(r - 1)] = (int32_t)(c / s1);
      fwd[3 * (int64_t)(r - 1) + 1] = (int32_t)((c / n3) % n2);
      fwd[3 * (int64_t)(r - 1) + 2] = (int32_t)(c % n3);
    }
  }
}

template <typename T>
static int upload_array(xf_ctx* ctx, T** dst, const std::vector<T>& src) {
  XF_CUDA(ctx, cudaMalloc(dst, src.size() * sizeof(T)));
  XF_CUDA(ctx, cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return XF_OK;
}

// Per-index coefficients of the fast stencil, from the reference's spacing
// expressions (XOperator.cpp:973-992): hh = (h[i-1]+h[i])/2.
static int build_coeffs(xf_grid* g, const double* h, int n, double** cm, double** cp, float** fm, float** fp,
                        double** rh, double** rhh, float** frh, float** frhh) {
  std::vector<double> vm(n, 0.0), vp(n, 0.0), vrh(n, 0.0), vrhh(n, 0.0);
  std::vector<float> wm(n, 0.f), wp(n, 0.f), wrh(n, 0.f), wrhh(n, 0.f);
  for (int i = 0; i < n - 1; i++) vrh[i] = 1.0 / h[i];
  for (int i = 1; i < n - 1; i++) {
    double hh = (h[i - 1] + h[i]) / 2;
    vm[i] = 1.0 / (h[i - 1] * hh);
    vp[i] = 1.0 / (h[i] * hh);
    vrhh[i] = 1.0 / hh;
  }
  for (int i = 0; i < n; i++) {
    wm[i] = (float)vm[i]; wp[i] = (float)vp[i]; wrh[i] = (float)vrh[i]; wrhh[i] = (float)vrhh[i];
  }
  int st;
  if ((st = upload_array(g->ctx, cm, vm)) || (st = upload_array(g->ctx, cp, vp)) || (st = upload_array(g->ctx, fm, wm)) ||
      (st = upload_array(g->ctx, fp, wp)) || (st = upload_array(g->ctx, rh, vrh)) || (st = upload_array(g->ctx, rhh, vrhh)) ||
      (st = upload_array(g->ctx, frh, wrh)) || (st = upload_array(g->ctx, frhh, wrhh)))
    return st;
  return XF_OK;
}

// Diagonal of each Laplace Actual row in coefficient form: the sum of the
// open faces' coefficients (0 for every other row).
__global__ void k_diag(const uint8_t* __restrict__ kind, const double* __restrict__ cxm, const double* __restrict__ cxp,
                       const double* __restrict__ cym, const double* __restrict__ cyp, const double* __restrict__ czm,
                       const double* __restrict__ czp, int n1, int n2, int n3, double* __restrict__ diag) {
  const int64_t n = (int64_t)n1 * n2 * n3, s1 = (int64_t)n2 * n3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t kb = kind[c];
    double d = 0.0;
    if (row_of(kb) == ROW_ACTUAL) {
      const int i = (int)(c / s1), j = (int)((c / n3) % n2), k = (int)(c % n3);
      d = (((kb & K_PX) ? cxp[i] : 0.0) + ((kb & K_MX) ? cxm[i] : 0.0)) +
          (((kb & K_PY) ? cyp[j] : 0.0) + ((kb & K_MY) ? cym[j] : 0.0)) +
          (((kb & K_PZ) ? czp[k] : 0.0) + ((kb & K_MZ) ? czm[k] : 0.0));
    }
    diag[c] = d;
  }
}

extern "C" int xf_grid_destroy(xf_grid* g) {
  if (!g) return XF_ERR_ARG;
  cudaSetDevice(g->ctx->device);
  cudaStreamSynchronize(g->ctx->stream);
  void* ptrs[] = {g->diag, g->code, g->nflag, g->kind, g->smask, g->inv, g->brow_of, g->brow_nrm, g->hx, g->hy, g->hz, g->fhx, g->fhy, g->fhz,
                  g->cxm, g->cxp, g->cym, g->cyp, g->czm, g->czp, g->fxm, g->fxp, g->fym, g->fyp, g->fzm, g->fzp,
                  g->rhx, g->rhy, g->rhz, g->rhhx, g->rhhy, g->rhhz, g->frhx, g->frhy, g->frhz, g->frhhx, g->frhhy, g->frhhz};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete g;
  return XF_OK;
}

// Point codes as bytes (codes outside 0..255 become 255: an unknown code), and
// the nonzero components of Normal cells' normals.
__global__ void k_code_bytes(const int32_t* __restrict__ codes, const double* __restrict__ nrm, int64_t n,
                             uint8_t* __restrict__ out, uint8_t* __restrict__ nflag) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t m = codes[c];
    out[c] = (m >= 0 && m < 255) ? (uint8_t)m : (uint8_t)255;
    uint8_t f = 0;
    if (m == 5 && nrm) f = (nrm[3 * c] != 0 ? 1 : 0) | (nrm[3 * c + 1] != 0 ? 2 : 0) | (nrm[3 * c + 2] != 0 ? 4 : 0);
    nflag[c] = f;
  }
}

extern "C" int xf_grid_create(xf_ctx* ctx, int n1, int n2, int n3, const int32_t* codes, const double* hx,
                              const double* hy, const double* hz, const double* normals, xf_grid** out) {
  if (!ctx || !out || !codes || !hx || !hy || !hz || n1 < 2 || n2 < 2 || n3 < 2)
    return xf_fail(ctx, XF_ERR_ARG, "xf_grid_create: bad arguments");
  *out = nullptr;
  const int64_t n = (int64_t)n1 * n2 * n3;
  if (n >= (int64_t)INT32_MAX) return xf_fail(ctx, XF_ERR_ARG, "xf_grid_create: box too large for int32 Rn indices");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  xf_grid* g = new xf_grid();
  memset(g, 0, sizeof(*g));
  g->ctx = ctx;
  g->n1 = n1; g->n2 = n2; g->n3 = n3;
  g->ncell = n; g->s1 = (int64_t)n2 * n3; g->s2 = n3;
  int st = XF_OK;
  int32_t* d_codes = nullptr;
  double* d_nrm = nullptr;
  uint8_t* d_isb = nullptr;
  unsigned long long* d_bad = nullptr;
  unsigned long long h_bad[2] = {~0ull, ~0ull};
  auto cleanup = [&]() {
    if (d_codes) cudaFree(d_codes);
    if (d_nrm) cudaFree(d_nrm);
    if (d_isb) cudaFree(d_isb);
    if (d_bad) cudaFree(d_bad);
  };
#define G_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { st = xf_fail(ctx, XF_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); goto fail; } } while (0)
  G_TRY(cudaMalloc(&d_codes, n * sizeof(int32_t)));
  G_TRY(cudaMemcpyAsync(d_codes, codes, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  if (normals) {
    G_TRY(cudaMalloc(&d_nrm, 3 * n * sizeof(double)));
    G_TRY(cudaMemcpyAsync(d_nrm, normals, 3 * n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  // 64 zero bytes past the box: bulk copies of kind rows round their ends up
  // to 16 bytes
  G_TRY(cudaMalloc(&g->kind, n + 64));
  G_TRY(cudaMemsetAsync(g->kind + n, 0, 64, ctx->stream));
  G_TRY(cudaMalloc(&g->smask, n));
  G_TRY(cudaMalloc(&d_isb, n));
  G_TRY(cudaMalloc(&g->inv, n * sizeof(int32_t)));
  G_TRY(cudaMalloc(&g->brow_of, n * sizeof(int32_t)));
  G_TRY(cudaMalloc(&d_bad, 2 * sizeof(unsigned long long)));
  G_TRY(cudaMemcpyAsync(d_bad, h_bad, sizeof(h_bad), cudaMemcpyHostToDevice, ctx->stream));
  k_classify<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(d_codes, d_nrm, n1, n2, n3, g->kind, g->smask, d_isb, d_bad);
  G_TRY(cudaGetLastError());
  G_TRY(cudaMalloc(&g->code, n));
  G_TRY(cudaMalloc(&g->nflag, n));
  k_code_bytes<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(d_codes, d_nrm, n, g->code, g->nflag);
  G_TRY(cudaGetLastError());
  G_TRY(cudaMemcpyAsync(h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost, ctx->stream));
  if ((st = scan_number(ctx, g->smask, n, g->inv, 1, 0, &g->end_index)) != XF_OK) goto fail;
  if ((st = scan_number(ctx, d_isb, n, g->brow_of, 0, -1, &g->nbrow)) != XF_OK) goto fail;
  G_TRY(cudaMalloc(&g->brow_nrm, (g->nbrow > 0 ? g->nbrow : 1) * 3 * sizeof(double)));
  if (g->nbrow > 0)
    k_gather_normals<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(d_nrm, g->brow_of, n, g->brow_nrm);
  G_TRY(cudaGetLastError());
  g->lap_status = h_bad[0] == ~0ull ? XF_OK : XF_ERR_MASK;
  g->vardiv_status = h_bad[1] == ~0ull ? XF_OK : XF_ERR_MASK;
  g->lap_bad = h_bad[0] == ~0ull ? -1 : (int64_t)h_bad[0];
  g->vardiv_bad = h_bad[1] == ~0ull ? -1 : (int64_t)h_bad[1];
  {
    std::vector<double> vx(hx, hx + n1 - 1), vy(hy, hy + n2 - 1), vz(hz, hz + n3 - 1);
    if ((st = upload_array(ctx, &g->hx, vx)) || (st = upload_array(ctx, &g->hy, vy)) || (st = upload_array(ctx, &g->hz, vz)))
      goto fail;
    std::vector<float> fx(vx.begin(), vx.end()), fy(vy.begin(), vy.end()), fz(vz.begin(), vz.end());
    if ((st = upload_array(ctx, &g->fhx, fx)) || (st = upload_array(ctx, &g->fhy, fy)) || (st = upload_array(ctx, &g->fhz, fz)))
      goto fail;
    if ((st = build_coeffs(g, hx, n1, &g->cxm, &g->cxp, &g->fxm, &g->fxp, &g->rhx, &g->rhhx, &g->frhx, &g->frhhx)) ||
        (st = build_coeffs(g, hy, n2, &g->cym, &g->cyp, &g->fym, &g->fyp, &g->rhy, &g->rhhy, &g->frhy, &g->frhhy)) ||
        (st = build_coeffs(g, hz, n3, &g->czm, &g->czp, &g->fzm, &g->fzp, &g->rhz, &g->rhhz, &g->frhz, &g->frhhz)))
      goto fail;
  }
  {
    // Uniform axes: c?m[i] = c?p[i] = 1/(h*h) for every interior index, bit for
    // bit the table value (1/(h*((h+h)/2)) == 1/(h*h) exactly).
    auto uni = [](const double* h, int n, double* c) {
      for (int i = 1; i < n - 1; i++)
        if (h[i] != h[0]) return false;
      *c = 1.0 / (h[0] * ((h[0] + h[0]) / 2));
      return true;
    };
    g->uniform = uni(hx, n1, &g->ucx) && uni(hy, n2, &g->ucy) && uni(hz, n3, &g->ucz);
  }
  G_TRY(cudaMalloc(&g->diag, n * sizeof(double)));
  k_diag<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(g->kind, g->cxm, g->cxp, g->cym, g->cyp, g->czm, g->czp,
                                                             n1, n2, n3, g->diag);
  G_TRY(cudaGetLastError());
  G_TRY(cudaStreamSynchronize(ctx->stream));
#undef G_TRY
  cleanup();
  *out = g;
  return XF_OK;
fail:
  cudaStreamSynchronize(ctx->stream);
  cleanup();
  xf_grid_destroy(g);
  return st;
}

extern "C" int xf_grid_end_index(const xf_grid* g, int64_t* e) {
  if (!g || !e) return XF_ERR_ARG;
  *e = g->end_index;
  return XF_OK;
}

extern "C" int xf_grid_check(const xf_grid* g, int op, int64_t* bad) {
  if (!g) return XF_ERR_ARG;
  int st = op == XF_OP_VARDIV ? g->vardiv_status : g->lap_status;
  if (bad) *bad = op == XF_OP_VARDIV ? g->vardiv_bad : g->lap_bad;
  return st;
}

extern "C" int xf_grid_rn_map(const xf_grid* g, int32_t* inv_box, int32_t* fwd_ijk) {
  if (!g) return XF_ERR_ARG;
  xf_ctx* ctx = g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  if (inv_box)
    XF_CUDA(ctx, cudaMemcpyAsync(inv_box, g->inv, g->ncell * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  if (fwd_ijk && g->end_index > 0) {
    int32_t* d_fwd = nullptr;
    XF_CUDA(ctx, cudaMallocAsync(&d_fwd, 3 * g->end_index * sizeof(int32_t), ctx->stream));
    k_rn_fwd<<<grid_blocks(ctx, g->ncell, 256), 256, 0, ctx->stream>>>(g->inv, g->ncell, g->n2, g->n3, d_fwd);
    XF_CUDA(ctx, cudaGetLastError());
    XF_CUDA(ctx, cudaMemcpyAsync(fwd_ijk, d_fwd, 3 * g->end_index * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    XF_CUDA(ctx, cudaFreeAsync(d_fwd, ctx->stream));
  }
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" int xf_grid_space_mask(const xf_grid* g, uint8_t* smask_box) {
  if (!g || !smask_box) return XF_ERR_ARG;
  xf_ctx* ctx = g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaMemcpyAsync(smask_box, g->smask, g->ncell, cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

// ---------------------------------------------------------------------------
extern "C" int xf_vec_create(xf_grid* g, int dtype, xf_vec** out) {
  if (!g || !out || (dtype != XF_F64 && dtype != XF_F32)) return xf_fail(g ? g->ctx : nullptr, XF_ERR_ARG, "xf_vec_create: bad arguments");
  xf_ctx* ctx = g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  size_t bytes = g->ncell * (dtype == XF_F64 ? 8 : 4);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_vec_create: cannot allocate %zu bytes", bytes);
  }
  XF_CUDA(ctx, cudaMemsetAsync(p, 0, bytes, ctx->stream));
  xf_vec* v = new xf_vec();
  v->g = g; v->dtype = dtype; v->data = p;
  *out = v;
  return XF_OK;
}

extern "C" int xf_vec_destroy(xf_vec* v) {
  if (!v) return XF_ERR_ARG;
  cudaSetDevice(v->g->ctx->device);
  cudaStreamSynchronize(v->g->ctx->stream);
  cudaFree(v->data);
  delete v;
  return XF_OK;
}

extern "C" void* xf_vec_data(xf_vec* v) { return v ? v->data : nullptr; }

__global__ void k_cast_d2f(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) b[c] = (float)a[c];
}
__global__ void k_cast_f2d(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) b[c] = (double)a[c];
}

extern "C" int xf_vec_upload(xf_vec* v, const double* host) {
  if (!v || !host) return XF_ERR_ARG;
  xf_ctx* ctx = v->g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t n = v->g->ncell;
  if (v->dtype == XF_F64) {
    XF_CUDA(ctx, cudaMemcpyAsync(v->data, host, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    double* tmp = nullptr;
    XF_CUDA(ctx, cudaMallocAsync(&tmp, n * 8, ctx->stream));
    XF_CUDA(ctx, cudaMemcpyAsync(tmp, host, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    k_cast_d2f<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(tmp, (float*)v->data, n);
    XF_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  }
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" int xf_vec_download(const xf_vec* v, double* host) {
  if (!v || !host) return XF_ERR_ARG;
  xf_ctx* ctx = v->g->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t n = v->g->ncell;
  if (v->dtype == XF_F64) {
    XF_CUDA(ctx, cudaMemcpyAsync(host, v->data, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    double* tmp = nullptr;
    XF_CUDA(ctx, cudaMallocAsync(&tmp, n * 8, ctx->stream));
    k_cast_f2d<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>((const float*)v->data, tmp, n);
    XF_CUDA(ctx, cudaMemcpyAsync(host, tmp, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    XF_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  }
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" int xf_vec_assign(xf_vec* dst, const xf_vec* src) {
  if (!dst || !src) return XF_ERR_ARG;
  if (dst->g != src->g) return xf_fail(dst->g->ctx, XF_ERR_STATE, "xf_vec_assign: vectors of different grids");
  xf_ctx* ctx = dst->g->ctx;
  const int64_t n = dst->g->ncell;
  if (dst->dtype == src->dtype) {
    XF_CUDA(ctx, cudaMemcpyAsync(dst->data, src->data, n * (dst->dtype == XF_F64 ? 8 : 4), cudaMemcpyDeviceToDevice, ctx->stream));
  } else if (dst->dtype == XF_F32) {
    k_cast_d2f<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>((const double*)src->data, (float*)dst->data, n);
  } else {
    k_cast_f2d<<<grid_blocks(ctx, n, 256), 256, 0, ctx->stream>>>((const float*)src->data, (double*)dst->data, n);
  }
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}
