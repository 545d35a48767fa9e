// Learned preconditioner: a 3-level 3-D U-Net (16/32/64 channels, 3x3x3
// convolutions, ReLU, BF16 weights and activations, FP32 accumulation) run
// by the tensor-core convolution of xf_conv.cu, trained on (residual, error)
// pairs by this file's own backward pass, and applied inside a flexible CG.
// No counterpart in the reference (it has no learned component).
//
// Levels: the grid's box (ghost layer included) is level 0; level l+1 halves
// the interior ((n-2)/2 + 2 per axis, interior divisible by 4), its cell
// (I,J,K) covering the fine interior cells 2I-1..2I (per axis).  Masks: level
// 0 = the grid's space mask, level l+1 = any child active.
//
// Network (channels):
//   enc0a 1->16, enc0b 16->16 (skip S0) | pool | enc1a 16->32, enc1b 32->32
//   (skip S1) | pool | mid_a 32->64, mid_b 64->64 | up -> [64 | S1] ->
//   dec1a 96->32, dec1b 32->32 | up -> [32 | S0] -> dec0a 48->16,
//   dec0b 16->16, out 16->1 (no ReLU).
// The skips are written by their encoder convolutions straight into the
// channel slices of the decoder inputs (no concatenation copies).  The input
// channel is padded to 16 and the output to 16 (the padding weights stay 0).
// Input r is divided by its RMS over the active cells; the output is the
// preconditioned direction (its scale is irrelevant to the flexible CG).
#include <math.h>

#include <vector>

#include "xf_control.cuh"

int xf_conv_launch(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int64_t in_ps, int ci, const void* weights,
                   const void* tiled, const float* bias, int co, const uint8_t* mask, void* out, int64_t out_pitch,
                   int out_ch, int out_fp32, int relu, const void* gate, int64_t gate_ps);
void xf_mv64(const xf_op* op, const MvReq<double>& q);
void xf_wgrad_tc_plan(const xf_ctx* ctx, int64_t ncell, int ci, int co, int* mtiles, int* splits, int* stages,
                      int64_t* partial_floats);
int xf_wgrad_tc(xf_ctx* ctx, int n1, int n2, int n3, const void* g, int64_t gps, int co, const void* x, int64_t xps,
                int ci, float* partial, float* gw);
void xf_cg_q32_dot(const xf_op* op, const float* p, float* q, int slot);
bool xf_tl_prolong_ay_supported(const xf_grid* g);
void xf_tl_prolong_ay(const xf_op* op, const float* zc, int c2, int c3, float* y, float* ay, int slot);
void xf_cg_res64(const xf_op* op, const double* x, const double* b, float* r32, int slot, int ctl);
void xf_dot_async(const xf_grid* g, int dtype, const void* a, const void* b, int slot);
int xf_op_ready(const xf_op* op);
bool xf_cg_poly_supported(const xf_grid* g);
bool xf_cheb_factors(double lmax, double ratio, int deg, float (*f)[3]);
void xf_cheb2_coeffs(double lmax, double ratio, float out[3]);
void xf_cg_poly_tl_launch(const xf_op* op, bool first, bool last, const float* in, const float* q, float* out,
                          const float coeffs[3], int s_yay, int s_yr, const float* y, float tsc, float* z2,
                          const float* r, const float* qw, int s_zr, int s_zq);
void xf_cg_poly_first_launch(const xf_op* op, const float* r, float* w, const float coeffs[3], const float* q,
                             const float* pa, const float* pb, float* e, float* r_out);

namespace {

struct Level {
  int n1, n2, n3;
  int64_t n, margin;
  uint8_t* mask = nullptr;
  int64_t active = 0;
};

// BF16 activation box in channel planes of 8 (xf_common.cuh), every plane
// with its zero margins
struct Act {
  uint16_t* base = nullptr;
  int C = 0, level = 0;
  int64_t rows = 0;   // cells per plane, margins included
  int64_t ps() const { return rows * 8; }
  uint16_t* p0(const Level* L) const { return base + L[level].margin * 8; }                 // plane 0, cell 0
  uint16_t* ch(const Level* L, int c0) const { return p0(L) + (int64_t)(c0 / 8) * ps(); }   // channel c0's plane
};

enum { ENC0A, ENC0B, ENC1A, ENC1B, MIDA, MIDB, DEC1A, DEC1B, DEC0A, DEC0B, OUTL, NLAYER };
const int LCI[NLAYER] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16, 16};
const int LCO[NLAYER] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16, 16};
const int LLEV[NLAYER] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0, 0};
const int LRELU[NLAYER] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0};

struct Layer {
  int ci, co;
  int64_t nw;                 // 27 * co * ci
  float* w = nullptr;         // FP32 master [27][co][ci]
  float* b = nullptr;         // [co]
  uint16_t* w16 = nullptr;    // BF16 [27][co][ci]
  uint16_t* wt16 = nullptr;   // BF16 flipped transpose [27][ci][co]: w16[26-t][co][ci]
  uint16_t *w16t = nullptr, *wt16t = nullptr;   // the same two in the tensor cores' tiled order
  float *gw = nullptr, *gb = nullptr;                  // gradients
  float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;   // Adam moments
};

}  // namespace

struct TlGraph;   // the graph-driven mixed two-level solve, kept with the network (below)
void xf_tl_graph_free(TlGraph* t);

struct xf_unet {
  TlGraph* tlg = nullptr;
  xf_ctx* ctx;
  const xf_grid* g;
  Level L[3];
  Layer ly[NLAYER];
  // forward activations
  Act X0, A0, CAT0, D0a, D0b;       // level 0 (CAT0 = [up 32 | S0 16])
  Act P1, A1, CAT1, D1a, D1b;       // level 1 (CAT1 = [up 64 | S1 32])
  Act P2, M2a, M2b;                 // level 2
  float* zout = nullptr;            // level-0 box, FP32, 1 channel
  // backward buffers (gradients w.r.t. pre-activations, BF16)
  Act G0_16a, G0_16b, G0_48, G1_32a, G1_32b, G1_96, G2_64a, G2_64b, G1_16, G2_32;
  float* gsum = nullptr;            // FP32 [level-0 cells x 16]: S0 gradient accumulator
  float* gsum1 = nullptr;           // FP32 [level-1 cells x 32]: S1 gradient accumulator
  double* red = nullptr;            // device reductions: [0] sum r^2, [1] sum e^2, [2] loss
  double* rpart = nullptr;          // per-block partials of the sums of squares, 2 x RP_MAX
  unsigned* rtick = nullptr;        // their last-block tickets
  float* wpart = nullptr;           // tensor-core weight-gradient partials [row tile][cell range][128][co]
  float* bpart = nullptr;           // per-chunk bias-gradient partials [chunk][co]
  double* zd = nullptr;             // level-0 box, FP64: the output (A-norm loss)
  double* az = nullptr;             // A zd
  int step = 0;
};

// ---------------------------------------------------------------------------
// Coarse mask: any active child.
__global__ void k_mask_pool(const uint8_t* __restrict__ fine, int f2, int f3, uint8_t* __restrict__ coarse, int c1,
                            int c2, int c3) {
  const int64_t n = (int64_t)c1 * c2 * c3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int I = (int)(c / ((int64_t)c2 * c3)), J = (int)((c / c3) % c2), K = (int)(c % c3);
    uint8_t m = 0;
    if (I >= 1 && I <= c1 - 2 && J >= 1 && J <= c2 - 2 && K >= 1 && K <= c3 - 2)
      for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
          for (int d = 0; d < 2; d++)
            m |= fine[((int64_t)(2 * I - 1 + a) * f2 + (2 * J - 1 + b)) * f3 + (2 * K - 1 + d)];
    coarse[c] = m ? 1 : 0;
  }
}

__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }
__device__ __forceinline__ uint16_t f2bf(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);   // inf / nan
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

// Average of the 8 children (inactive children hold 0), times the coarse mask.
// src: fine slice (plane 0 at cell 0, plane stride sps), dst: coarse (dps),
// C channels; one thread per cell and plane (16 bytes).
__device__ __forceinline__ void bf8_acc(float (&s)[8], uint4 v) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    s[2 * q] += bf2f((uint16_t)(w[q] & 0xFFFFu));
    s[2 * q + 1] += bf2f((uint16_t)(w[q] >> 16));
  }
}
__device__ __forceinline__ uint4 bf8_pack(const float (&s)[8], float scale) {
  uint32_t w[4];
#pragma unroll
  for (int q = 0; q < 4; q++) w[q] = (uint32_t)f2bf(s[2 * q] * scale) | ((uint32_t)f2bf(s[2 * q + 1] * scale) << 16);
  return make_uint4(w[0], w[1], w[2], w[3]);
}
__global__ void k_pool(const uint16_t* __restrict__ src, int64_t sps, int f2, int f3, uint16_t* __restrict__ dst,
                       int64_t dps, const uint8_t* __restrict__ cmask, int c1, int c2, int c3, int C) {
  const int C8 = C / 8;
  const int64_t n = (int64_t)c1 * c2 * c3 * C8;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = u / C8;
    const int g = (int)(u - c * C8);
    const int I = (int)(c / ((int64_t)c2 * c3)), J = (int)((c / c3) % c2), K = (int)(c % c3);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (cmask[c])
      for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
          for (int d = 0; d < 2; d++)
            bf8_acc(s, *reinterpret_cast<const uint4*>(
                           src + g * sps + (((int64_t)(2 * I - 1 + a) * f2 + (2 * J - 1 + b)) * f3 + (2 * K - 1 + d)) * 8));
    *reinterpret_cast<uint4*>(dst + g * dps + c * 8) = bf8_pack(s, 0.125f);
  }
}

// Pooling backward: every active fine child receives 1/8 of its parent's
// gradient, added to an FP32 accumulator (pitch ald).
__global__ void k_pool_bwd(const uint16_t* __restrict__ gcoarse, int64_t gps, int c2, int c3,
                           const uint8_t* __restrict__ fmask, int f1, int f2, int f3, float* __restrict__ acc,
                           int ald, int C) {
  const int64_t n = (int64_t)f1 * f2 * f3 * C;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = u / C;
    const int ch = (int)(u - c * C);
    if (!fmask[c]) continue;
    const int i = (int)(c / ((int64_t)f2 * f3)), j = (int)((c / f3) % f2), k = (int)(c % f3);
    const int64_t pc = ((int64_t)(1 + (i - 1) / 2) * c2 + (1 + (j - 1) / 2)) * c3 + (1 + (k - 1) / 2);
    acc[c * ald + ch] += 0.125f * bf2f(gcoarse[(ch >> 3) * gps + pc * 8 + (ch & 7)]);
  }
}

// Nearest upsampling of a coarse slice into a fine slice, times the fine mask;
// one plane (8 channels, 16 bytes) per thread.
__global__ void k_upsample(const uint16_t* __restrict__ src, int64_t sps, int c2, int c3, uint16_t* __restrict__ dst,
                           int64_t dps, const uint8_t* __restrict__ fmask, int f1, int f2, int f3, int C) {
  const int C8 = C / 8;
  const int64_t n = (int64_t)f1 * f2 * f3 * C8;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = u / C8;
    const int g = (int)(u - c * C8);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (fmask[c]) {
      const int i = (int)(c / ((int64_t)f2 * f3)), j = (int)((c / f3) % f2), k = (int)(c % f3);
      const int64_t pc = ((int64_t)(1 + (i - 1) / 2) * c2 + (1 + (j - 1) / 2)) * c3 + (1 + (k - 1) / 2);
      v = *reinterpret_cast<const uint4*>(src + g * sps + pc * 8);
    }
    *reinterpret_cast<uint4*>(dst + g * dps + c * 8) = v;
  }
}

// Upsampling backward: a coarse cell's gradient is the sum over its 8
// children; then x coarse mask and the coarse activation's ReLU gate.
__global__ void k_upsample_bwd(const uint16_t* __restrict__ gfine, int64_t gps, int f2, int f3,
                               const uint16_t* __restrict__ gate, int64_t gtps, const uint8_t* __restrict__ cmask,
                               int c1, int c2, int c3, uint16_t* __restrict__ dst, int64_t dps, int C) {
  const int64_t n = (int64_t)c1 * c2 * c3 * C;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = u / C;
    const int ch = (int)(u - c * C);
    float s = 0.f;
    const int64_t pl = (int64_t)(ch >> 3), e = ch & 7;
    if (cmask[c] && bf2f(gate[pl * gtps + c * 8 + e]) > 0.f) {
      const int I = (int)(c / ((int64_t)c2 * c3)), J = (int)((c / c3) % c2), K = (int)(c % c3);
      for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
          for (int d = 0; d < 2; d++)
            s += bf2f(gfine[pl * gps + (((int64_t)(2 * I - 1 + a) * f2 + (2 * J - 1 + b)) * f3 + (2 * K - 1 + d)) * 8 + e]);
    }
    dst[pl * dps + c * 8 + e] = f2bf(s);
  }
}

// Skip gradient: dPre = (skip part of the decoder's input gradient + pooled
// path's accumulator) x mask x ReLU gate; the accumulator is cleared.
__global__ void k_skip_grad(const uint16_t* __restrict__ gskip, int64_t gps, float* __restrict__ acc, int ald,
                            const uint16_t* __restrict__ gate, int64_t gtps, const uint8_t* __restrict__ mask,
                            int64_t ncell, uint16_t* __restrict__ dst, int64_t dps, int C) {
  const int64_t n = ncell * C;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = u / C;
    const int ch = (int)(u - c * C);
    const int64_t o = c * 8 + (ch & 7), pl = ch >> 3;
    float v = bf2f(gskip[pl * gps + o]) + acc[c * ald + ch];
    acc[c * ald + ch] = 0.f;
    if (!mask[c] || !(bf2f(gate[pl * gtps + o]) > 0.f)) v = 0.f;
    dst[pl * dps + o] = f2bf(v);
  }
}

// Sum of squares over the active cells into red[slot].  Per-block partials,
// summed in a fixed order by the last block to finish, so the result does
// not depend on scheduling (256 threads, at most RP_MAX blocks).
constexpr int RP_MAX = 4096;
__global__ void __launch_bounds__(256) k_sumsq(const double* __restrict__ x, const uint8_t* __restrict__ m, int64_t n,
                                               double* red, int slot, double* part, unsigned* tick) {
  __shared__ double sw[8];
  __shared__ bool last;
  double s = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    if (m[c]) s += x[c] * x[c];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0;
    for (int w = 0; w < 8; w++) b += sw[w];
    part[slot * RP_MAX + blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(&tick[slot], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // the last block sums the partials: thread t takes t, t + 256, ... in
  // order, then a fixed tree over the threads (the same order every run)
  __threadfence();
  double t = 0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += 256) t += __ldcg(&part[slot * RP_MAX + k]);
  __shared__ double st[256];
  st[threadIdx.x] = t;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) st[threadIdx.x] += st[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    red[slot] = st[0];
    tick[slot] = 0;
  }
}

// Level-0 input: channel 0 = r / rms(r) on active cells, channels 1..15 = 0.
__global__ void k_unet_input(const double* __restrict__ r, const uint8_t* __restrict__ m, int64_t n,
                             const double* __restrict__ red, double count, uint16_t* __restrict__ x0, int64_t ps) {
  const double ss = red[0];
  const float inv = ss > 0 ? (float)(1.0 / sqrt(ss / count)) : 0.f;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    uint16_t v[16] = {0};
    if (m[c]) v[0] = f2bf((float)r[c] * inv);
    *reinterpret_cast<uint4*>(x0 + c * 8) = *reinterpret_cast<uint4*>(&v[0]);
    *reinterpret_cast<uint4*>(x0 + ps + c * 8) = *reinterpret_cast<uint4*>(&v[8]);
  }
}

// Loss (mean over active cells of (z - t)^2, t = e / rms(e)) and its
// gradient as the output layer's 16-channel dPre (channel 0).
__global__ void k_unet_loss(const float* __restrict__ z, const double* __restrict__ e, const uint8_t* __restrict__ m,
                            int64_t n, double count, double* red, uint16_t* __restrict__ g16, int64_t ps) {
  const double ss = red[1];
  const double inv = ss > 0 ? 1.0 / sqrt(ss / count) : 0.0;
  double l = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    uint16_t v[16] = {0};
    if (m[c]) {
      const double d = (double)z[c] - e[c] * inv;
      l += d * d;
      v[0] = f2bf((float)(2.0 * d / count));
    }
    *reinterpret_cast<uint4*>(g16 + c * 8) = *reinterpret_cast<uint4*>(&v[0]);
    *reinterpret_cast<uint4*>(g16 + ps + c * 8) = *reinterpret_cast<uint4*>(&v[8]);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&red[2], l / count);
}

// Bias gradient gb[co] += sum over cells of g[c][co] (the weight gradients run
// on the tensor cores, xf_wgrad_tc).  Block = (8-channel plane, chunk of
// cells); each thread sums 8 channels over its cells, the block in a fixed
// tree, and k_bgrad_sum adds the chunks in order (deterministic).
// Cells per block: 4096, or more so that a level has at most WG_MAX_CHUNKS
// chunks (the partial buffer's size).
constexpr int WG_MAX_CHUNKS = 128;
static int64_t wg_chunk(int64_t n) {
  int64_t c = (n + WG_MAX_CHUNKS - 1) / WG_MAX_CHUNKS;
  c = (c + 255) / 256 * 256;
  return c < 4096 ? 4096 : c;
}
__global__ void __launch_bounds__(256) k_bgrad(const uint16_t* __restrict__ g, int64_t gps, int64_t ncell, int chunk,
                                               int co, float* __restrict__ bpart) {
  __shared__ float red[8][256];
  const int q = blockIdx.y;
  const int64_t c_beg = (int64_t)blockIdx.x * chunk, c_end = min(ncell, c_beg + chunk);
  float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int64_t c = c_beg + threadIdx.x; c < c_end; c += 256) bf8_acc(s, *reinterpret_cast<const uint4*>(g + q * gps + c * 8));
  for (int e = 0; e < 8; e++) red[e][threadIdx.x] = s[e];
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
      for (int e = 0; e < 8; e++) red[e][threadIdx.x] += red[e][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 8) bpart[(int64_t)blockIdx.x * co + q * 8 + threadIdx.x] = red[threadIdx.x][0];
}
__global__ void k_bgrad_sum(const float* __restrict__ bpart, int nchunk, int co, float* __restrict__ gb) {
  const int u = threadIdx.x;
  if (u >= co) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; c++) s += bpart[(int64_t)c * co + u];
  gb[u] += s;
}

// Adam step on one layer (bias-corrected, step counts from 1), then the BF16
// copies: w16[t][co][ci] and the flipped transpose wt16[26-t][ci][co], each
// also in the tiled order.
__global__ void k_adam(float* w, float* gwt, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, int clear) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const float gr = gwt[u];
    const float mm = b1 * m[u] + (1 - b1) * gr;
    const float vv = b2 * v[u] + (1 - b2) * gr * gr;
    m[u] = mm;
    v[u] = vv;
    w[u] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    if (clear) gwt[u] = 0.f;
  }
}

__global__ void k_weights_bf16(const float* __restrict__ w, int co, int ci, uint16_t* __restrict__ w16,
                               uint16_t* __restrict__ wt16, uint16_t* __restrict__ w16t, uint16_t* __restrict__ wt16t) {
  const int64_t n = (int64_t)27 * co * ci;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(u / ((int64_t)co * ci));
    const int o = (int)((u / ci) % co), i = (int)(u % ci);
    const uint16_t h = f2bf(w[u]);
    w16[u] = h;
    wt16[((int64_t)(26 - t) * ci + i) * co + o] = h;
    w16t[conv_tiled_index(t, o, i, co, ci)] = h;
    wt16t[conv_tiled_index(26 - t, i, o, ci, co)] = h;
  }
}

// A-norm loss 1 - (z,r) / sqrt((z,Az)(e,r)) (one minus the A-norm cosine of
// the output and the error; dots in scalars[10..12]) and its gradient
// -(r - (z,r)/(z,Az) A z) / sqrt((z,Az)(e,r)) as the output layer's
// 16-channel dPre (channel 0).
__global__ void k_anorm_grad(const double* __restrict__ r, const double* __restrict__ az,
                             const uint8_t* __restrict__ m, int64_t n, const DevScratch* __restrict__ S, double* red,
                             uint16_t* __restrict__ g16, int64_t ps) {
  const double zr = S->scalars[10], zaz = S->scalars[11], er = S->scalars[12];
  const bool ok = zaz > 0 && er > 0;
  const double c1 = ok ? -1 / sqrt(zaz * er) : 0.0, c2 = ok ? zr / zaz : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) red[2] = ok ? 1 - zr / sqrt(zaz * er) : 1.0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    uint16_t v[16] = {0};
    if (m[c]) v[0] = f2bf((float)(c1 * (r[c] - c2 * az[c])));
    *reinterpret_cast<uint4*>(g16 + c * 8) = *reinterpret_cast<uint4*>(&v[0]);
    *reinterpret_cast<uint4*>(g16 + ps + c * 8) = *reinterpret_cast<uint4*>(&v[8]);
  }
}

__global__ void k_f2d_mask(const float* __restrict__ z, const uint8_t* __restrict__ m, int64_t n,
                           double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    out[c] = m[c] ? (double)z[c] : 0.0;
}

// ---------------------------------------------------------------------------
// Host side
static int ublocks(xf_ctx* ctx, int64_t n) { return grid_blocks(ctx, n, 256); }
// k_sumsq's grid: its partial buffer holds RP_MAX blocks (the loop is grid-stride)
static int sumsq_blocks(xf_ctx* ctx, int64_t n) { return std::min(ublocks(ctx, n), RP_MAX); }

static int act_alloc(xf_unet* u, Act& a, int level, int C) {
  a.level = level;
  a.C = C;
  a.rows = u->L[level].n + 2 * u->L[level].margin;
  if (cudaMalloc(&a.base, a.rows * C * 2) != cudaSuccess) {
    cudaGetLastError();
    a.base = nullptr;
    return XF_ERR_NOMEM;
  }
  return cudaMemsetAsync(a.base, 0, a.rows * C * 2, u->ctx->stream) == cudaSuccess ? XF_OK : XF_ERR_CUDA;
}

static void unet_free(xf_unet* u) {
  Act* a[] = {&u->X0, &u->A0, &u->CAT0, &u->D0a, &u->D0b, &u->P1, &u->A1, &u->CAT1, &u->D1a, &u->D1b,
              &u->P2, &u->M2a, &u->M2b, &u->G0_16a, &u->G0_16b, &u->G0_48, &u->G1_32a, &u->G1_32b,
              &u->G1_96, &u->G2_64a, &u->G2_64b, &u->G1_16, &u->G2_32};
  for (Act* x : a)
    if (x->base) cudaFree(x->base);
  for (int l = 1; l < 3; l++)
    if (u->L[l].mask) cudaFree(u->L[l].mask);
  for (Layer& y : u->ly) {
    void* ps[] = {y.w, y.b, y.w16, y.wt16, y.w16t, y.wt16t, y.gw, y.gb, y.mw, y.vw, y.mb, y.vb};
    for (void* p : ps)
      if (p) cudaFree(p);
  }
  if (u->zout) cudaFree(u->zout);
  if (u->gsum) cudaFree(u->gsum);
  if (u->gsum1) cudaFree(u->gsum1);
  if (u->red) cudaFree(u->red);
  if (u->rpart) cudaFree(u->rpart);
  if (u->rtick) cudaFree(u->rtick);
  if (u->wpart) cudaFree(u->wpart);
  if (u->bpart) cudaFree(u->bpart);
  if (u->zd) cudaFree(u->zd);
  if (u->az) cudaFree(u->az);
  if (u->tlg) xf_tl_graph_free(u->tlg);
  delete u;
}

extern "C" int xf_unet_destroy(xf_unet* u) {
  if (!u) return XF_OK;
  cudaSetDevice(u->ctx->device);
  cudaStreamSynchronize(u->ctx->stream);
  unet_free(u);
  return XF_OK;
}

static int64_t count_active(xf_ctx* ctx, const uint8_t* mask, int64_t n) {
  std::vector<uint8_t> h(n);
  if (cudaMemcpy(h.data(), mask, n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  int64_t s = 0;
  for (int64_t c = 0; c < n; c++) s += h[c] != 0;
  return s;
}

extern "C" int xf_unet_create(const xf_grid* g, xf_unet** out) {
  if (!g || !out) return XF_ERR_ARG;
  *out = nullptr;
  xf_ctx* ctx = g->ctx;
  if ((g->n1 - 2) % 4 || (g->n2 - 2) % 4 || (g->n3 - 2) % 4 || g->n1 < 10 || g->n2 < 10 || g->n3 < 10)
    return xf_fail(ctx, XF_ERR_ARG, "xf_unet_create: interior dimensions must be multiples of 4 (>= 8)");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  xf_unet* u = new xf_unet();
  u->ctx = ctx;
  u->g = g;
  int dims[3] = {g->n1, g->n2, g->n3};
  for (int l = 0; l < 3; l++) {
    Level& L = u->L[l];
    L.n1 = dims[0]; L.n2 = dims[1]; L.n3 = dims[2];
    L.n = (int64_t)L.n1 * L.n2 * L.n3;
    L.margin = XF_CONV_MARGIN(L.n2, L.n3);
    for (int a = 0; a < 3; a++) dims[a] = (dims[a] - 2) / 2 + 2;
  }
  u->L[0].mask = g->smask;
  int st = XF_OK;
  for (int l = 1; l < 3 && !st; l++) {
    if (cudaMalloc(&u->L[l].mask, u->L[l].n) != cudaSuccess) st = XF_ERR_NOMEM;
    else
      k_mask_pool<<<ublocks(ctx, u->L[l].n), 256, 0, ctx->stream>>>(u->L[l - 1].mask, u->L[l - 1].n2, u->L[l - 1].n3,
                                                                   u->L[l].mask, u->L[l].n1, u->L[l].n2, u->L[l].n3);
  }
  struct { Act* a; int level, C; } acts[] = {
      {&u->X0, 0, 16}, {&u->A0, 0, 16}, {&u->CAT0, 0, 48}, {&u->D0a, 0, 16}, {&u->D0b, 0, 16},
      {&u->P1, 1, 16}, {&u->A1, 1, 32}, {&u->CAT1, 1, 96}, {&u->D1a, 1, 32}, {&u->D1b, 1, 32},
      {&u->P2, 2, 32}, {&u->M2a, 2, 64}, {&u->M2b, 2, 64},
      {&u->G0_16a, 0, 16}, {&u->G0_16b, 0, 16}, {&u->G0_48, 0, 48}, {&u->G1_32a, 1, 32}, {&u->G1_32b, 1, 32},
      {&u->G1_96, 1, 96}, {&u->G2_64a, 2, 64}, {&u->G2_64b, 2, 64}, {&u->G1_16, 1, 16}, {&u->G2_32, 2, 32}};
  for (auto& e : acts)
    if (!st) st = act_alloc(u, *e.a, e.level, e.C);
  for (int k = 0; k < NLAYER && !st; k++) {
    Layer& y = u->ly[k];
    y.ci = LCI[k]; y.co = LCO[k];
    y.nw = (int64_t)27 * y.co * y.ci;
    float** f32[] = {&y.w, &y.gw, &y.mw, &y.vw};
    for (float** p : f32)
      if (!st && cudaMalloc(p, y.nw * 4) != cudaSuccess) st = XF_ERR_NOMEM;
    float** fb[] = {&y.b, &y.gb, &y.mb, &y.vb};
    for (float** p : fb)
      if (!st && cudaMalloc(p, y.co * 4) != cudaSuccess) st = XF_ERR_NOMEM;
    if (!st && (cudaMalloc(&y.w16, y.nw * 2) != cudaSuccess || cudaMalloc(&y.wt16, y.nw * 2) != cudaSuccess ||
                cudaMalloc(&y.w16t, y.nw * 2) != cudaSuccess || cudaMalloc(&y.wt16t, y.nw * 2) != cudaSuccess))
      st = XF_ERR_NOMEM;
    if (!st) {
      cudaMemsetAsync(y.w, 0, y.nw * 4, ctx->stream); cudaMemsetAsync(y.gw, 0, y.nw * 4, ctx->stream);
      cudaMemsetAsync(y.mw, 0, y.nw * 4, ctx->stream); cudaMemsetAsync(y.vw, 0, y.nw * 4, ctx->stream);
      cudaMemsetAsync(y.b, 0, y.co * 4, ctx->stream); cudaMemsetAsync(y.gb, 0, y.co * 4, ctx->stream);
      cudaMemsetAsync(y.mb, 0, y.co * 4, ctx->stream); cudaMemsetAsync(y.vb, 0, y.co * 4, ctx->stream);
      cudaMemsetAsync(y.w16, 0, y.nw * 2, ctx->stream); cudaMemsetAsync(y.wt16, 0, y.nw * 2, ctx->stream);
      cudaMemsetAsync(y.w16t, 0, y.nw * 2, ctx->stream); cudaMemsetAsync(y.wt16t, 0, y.nw * 2, ctx->stream);
    }
  }
  if (!st && (cudaMalloc(&u->zout, u->L[0].n * 4) != cudaSuccess ||
              cudaMalloc(&u->gsum, u->L[0].n * 16 * 4) != cudaSuccess ||
              cudaMalloc(&u->gsum1, u->L[1].n * 32 * 4) != cudaSuccess || cudaMalloc(&u->red, 8 * 8) != cudaSuccess ||
              cudaMalloc(&u->zd, u->L[0].n * 8) != cudaSuccess || cudaMalloc(&u->az, u->L[0].n * 8) != cudaSuccess))
    st = XF_ERR_NOMEM;
  if (!st) {   // partial buffers of the deterministic reductions
    int64_t wneed = 1;
    for (int k = 0; k < NLAYER; k++) {
      int mt, sp, stg;
      int64_t need;
      xf_wgrad_tc_plan(ctx, u->L[LLEV[k]].n, u->ly[k].ci, u->ly[k].co, &mt, &sp, &stg, &need);
      if (need > wneed) wneed = need;
    }
    if (cudaMalloc(&u->rpart, 2 * RP_MAX * 8) != cudaSuccess || cudaMalloc(&u->rtick, 4 * 4) != cudaSuccess ||
        cudaMalloc(&u->wpart, wneed * 4) != cudaSuccess || cudaMalloc(&u->bpart, WG_MAX_CHUNKS * 64 * 4) != cudaSuccess)
      st = XF_ERR_NOMEM;
    else
      cudaMemsetAsync(u->rtick, 0, 4 * 4, ctx->stream);
  }
  if (!st) {
    cudaMemsetAsync(u->zout, 0, u->L[0].n * 4, ctx->stream);
    cudaMemsetAsync(u->gsum, 0, u->L[0].n * 16 * 4, ctx->stream);
    cudaMemsetAsync(u->gsum1, 0, u->L[1].n * 32 * 4, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) st = XF_ERR_CUDA;
  }
  for (int l = 0; l < 3 && !st; l++) {
    u->L[l].active = count_active(ctx, u->L[l].mask, u->L[l].n);
    if (u->L[l].active < 0) st = XF_ERR_CUDA;
  }
  if (st) {
    cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    unet_free(u);
    return xf_fail(ctx, st, "xf_unet_create: device allocation / set-up failed");
  }
  *out = u;
  return XF_OK;
}

extern "C" int xf_unet_param_count(const xf_unet* u, int64_t* n) {
  if (!u || !n) return XF_ERR_ARG;
  int64_t s = 0;
  for (const Layer& y : u->ly) s += y.nw + y.co;
  *n = s;
  return XF_OK;
}

// Parameters as one FP32 array: per layer W[27][co][ci] then b[co], layers in
// network order.  Padding weights (input channels 1..15 of the first layer,
// output channels 1..15 of the last) are forced to 0.
static int params_io(xf_unet* u, float* host, int which, bool upload) {
  xf_ctx* ctx = u->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t o = 0;
  for (int k = 0; k < NLAYER; k++) {
    Layer& y = u->ly[k];
    float* w = which == 0 ? y.w : y.gw;
    float* b = which == 0 ? y.b : y.gb;
    if (upload) {
      std::vector<float> hw(host + o, host + o + y.nw), hb(host + o + y.nw, host + o + y.nw + y.co);
      for (int t = 0; t < 27; t++)
        for (int co = 0; co < y.co; co++)
          for (int ci = 0; ci < y.ci; ci++)
            if ((k == ENC0A && ci > 0) || (k == OUTL && co > 0)) hw[((size_t)t * y.co + co) * y.ci + ci] = 0.f;
      if (k == OUTL)
        for (int co = 1; co < y.co; co++) hb[co] = 0.f;
      XF_CUDA(ctx, cudaMemcpy(w, hw.data(), y.nw * 4, cudaMemcpyHostToDevice));
      XF_CUDA(ctx, cudaMemcpy(b, hb.data(), y.co * 4, cudaMemcpyHostToDevice));
      if (which == 0)
        k_weights_bf16<<<ublocks(ctx, y.nw), 256, 0, ctx->stream>>>(y.w, y.co, y.ci, y.w16, y.wt16, y.w16t, y.wt16t);
    } else {
      XF_CUDA(ctx, cudaMemcpy(host + o, w, y.nw * 4, cudaMemcpyDeviceToHost));
      XF_CUDA(ctx, cudaMemcpy(host + o + y.nw, b, y.co * 4, cudaMemcpyDeviceToHost));
    }
    o += y.nw + y.co;
  }
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" int xf_unet_set_params(xf_unet* u, const float* host) {
  if (!u || !host) return XF_ERR_ARG;
  u->step = 0;
  for (Layer& y : u->ly) {   // a new parameter set restarts Adam
    cudaMemsetAsync(y.mw, 0, y.nw * 4, u->ctx->stream); cudaMemsetAsync(y.vw, 0, y.nw * 4, u->ctx->stream);
    cudaMemsetAsync(y.mb, 0, y.co * 4, u->ctx->stream); cudaMemsetAsync(y.vb, 0, y.co * 4, u->ctx->stream);
  }
  return params_io(u, const_cast<float*>(host), 0, true);
}
extern "C" int xf_unet_get_params(xf_unet* u, float* host) {
  if (!u || !host) return XF_ERR_ARG;
  return params_io(u, host, 0, false);
}
extern "C" int xf_unet_get_grads(xf_unet* u, float* host) {
  if (!u || !host) return XF_ERR_ARG;
  return params_io(u, host, 1, false);
}

// ---------------------------------------------------------------------------
// Forward pass on the residual box r (FP64, the grid's layout); the output
// (FP32, level-0 box) lands in u->zout.
// `in` from channel in_c0 on; `out` a plane-0 pointer with plane stride
// out_pitch (BF16), or FP32 rows of pitch out_pitch.
static int conv(xf_unet* u, int k, const Act& in, int in_c0, void* out, int64_t out_pitch, int out_ch, int out_fp32) {
  const Layer& y = u->ly[k];
  const Level& L = u->L[LLEV[k]];
  return xf_conv_launch(u->ctx, L.n1, L.n2, L.n3, in.ch(u->L, in_c0), in.ps(), y.ci, y.w16, y.w16t, y.b, y.co, L.mask,
                        out, out_pitch, out_ch, out_fp32, LRELU[k], nullptr, 0);
}
// Input gradient of layer k from its pre-activation gradient g: the convolution
// with the flipped transposed weights, x mask, x the ReLU gate of `gate` (the
// input activation) when given.
static int dgrad(xf_unet* u, int k, const Act& g, const Act& out, int out_c0, const Act* gate, int gate_c0) {
  const Layer& y = u->ly[k];
  const Level& L = u->L[LLEV[k]];
  return xf_conv_launch(u->ctx, L.n1, L.n2, L.n3, g.p0(u->L), g.ps(), y.co, y.wt16, y.wt16t, nullptr, y.ci, L.mask,
                        out.ch(u->L, out_c0), out.ps(), y.ci, 0, 0,
                        gate ? (const void*)gate->ch(u->L, gate_c0) : nullptr, gate ? gate->ps() : 0);
}
// Weight and bias gradients of layer k from its pre-activation gradient g and
// its input x (from channel x_c0 on): the weights on the tensor cores.
static int wgrad(xf_unet* u, int k, const Act& g, const Act& x, int x_c0) {
  const Layer& y = u->ly[k];
  const Level& L = u->L[LLEV[k]];
  const int st = xf_wgrad_tc(u->ctx, L.n1, L.n2, L.n3, g.p0(u->L), g.ps(), y.co, x.ch(u->L, x_c0), x.ps(), y.ci,
                             u->wpart, y.gw);
  if (st) return st;
  const int64_t chunk = wg_chunk(L.n);
  const int nchunk = (int)((L.n + chunk - 1) / chunk);
  k_bgrad<<<dim3((unsigned)nchunk, (unsigned)(y.co / 8)), 256, 0, u->ctx->stream>>>(g.p0(u->L), g.ps(), L.n,
                                                                                    (int)chunk, y.co, u->bpart);
  k_bgrad_sum<<<1, 64, 0, u->ctx->stream>>>(u->bpart, nchunk, y.co, y.gb);
  return XF_OK;
}

// Kernels one forward pass launches, with xf_unet_apply_dev's output conversion.
constexpr int UNET_FORWARD_LAUNCHES = 18;
static int forward(xf_unet* u, const double* r) {
  xf_ctx* ctx = u->ctx;
  cudaStream_t s = ctx->stream;
  const Level* L = u->L;
  int st;
  XF_CUDA(ctx, cudaMemsetAsync(u->red, 0, 8 * 8, s));
  k_sumsq<<<sumsq_blocks(ctx, L[0].n), 256, 0, s>>>(r, L[0].mask, L[0].n, u->red, 0, u->rpart, u->rtick);
  k_unet_input<<<ublocks(ctx, L[0].n), 256, 0, s>>>(r, L[0].mask, L[0].n, u->red, (double)L[0].active,
                                                    u->X0.p0(L), u->X0.ps());
  if ((st = conv(u, ENC0A, u->X0, 0, u->A0.p0(L), u->A0.ps(), 16, 0))) return st;
  if ((st = conv(u, ENC0B, u->A0, 0, u->CAT0.ch(L, 32), u->CAT0.ps(), 16, 0))) return st;   // S0
  k_pool<<<ublocks(ctx, L[1].n * 2), 256, 0, s>>>(u->CAT0.ch(L, 32), u->CAT0.ps(), L[0].n2, L[0].n3, u->P1.p0(L),
                                                  u->P1.ps(), L[1].mask, L[1].n1, L[1].n2, L[1].n3, 16);
  if ((st = conv(u, ENC1A, u->P1, 0, u->A1.p0(L), u->A1.ps(), 32, 0))) return st;
  if ((st = conv(u, ENC1B, u->A1, 0, u->CAT1.ch(L, 64), u->CAT1.ps(), 32, 0))) return st;   // S1
  k_pool<<<ublocks(ctx, L[2].n * 4), 256, 0, s>>>(u->CAT1.ch(L, 64), u->CAT1.ps(), L[1].n2, L[1].n3, u->P2.p0(L),
                                                  u->P2.ps(), L[2].mask, L[2].n1, L[2].n2, L[2].n3, 32);
  if ((st = conv(u, MIDA, u->P2, 0, u->M2a.p0(L), u->M2a.ps(), 64, 0))) return st;
  if ((st = conv(u, MIDB, u->M2a, 0, u->M2b.p0(L), u->M2b.ps(), 64, 0))) return st;
  k_upsample<<<ublocks(ctx, L[1].n * 8), 256, 0, s>>>(u->M2b.p0(L), u->M2b.ps(), L[2].n2, L[2].n3, u->CAT1.p0(L),
                                                       u->CAT1.ps(), L[1].mask, L[1].n1, L[1].n2, L[1].n3, 64);
  if ((st = conv(u, DEC1A, u->CAT1, 0, u->D1a.p0(L), u->D1a.ps(), 32, 0))) return st;
  if ((st = conv(u, DEC1B, u->D1a, 0, u->D1b.p0(L), u->D1b.ps(), 32, 0))) return st;
  k_upsample<<<ublocks(ctx, L[0].n * 4), 256, 0, s>>>(u->D1b.p0(L), u->D1b.ps(), L[1].n2, L[1].n3, u->CAT0.p0(L),
                                                       u->CAT0.ps(), L[0].mask, L[0].n1, L[0].n2, L[0].n3, 32);
  if ((st = conv(u, DEC0A, u->CAT0, 0, u->D0a.p0(L), u->D0a.ps(), 16, 0))) return st;
  if ((st = conv(u, DEC0B, u->D0a, 0, u->D0b.p0(L), u->D0b.ps(), 16, 0))) return st;
  if ((st = conv(u, OUTL, u->D0b, 0, u->zout, 1, 1, 1))) return st;
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

// Backward pass from the loss against the target e (FP64 box): weight and
// bias gradients accumulate into gw / gb.
static int backward(xf_unet* u, const double* r, const double* e, const xf_op* op) {
  xf_ctx* ctx = u->ctx;
  cudaStream_t s = ctx->stream;
  const Level* L = u->L;
  int st;
  if (op) {   // A-norm loss
    k_f2d_mask<<<ublocks(ctx, L[0].n), 256, 0, s>>>(u->zout, L[0].mask, L[0].n, u->zd);
    MvReq<double> m;
    m.x = u->zd; m.y = u->az; m.zero_inactive = 1;
    xf_mv64(op, m);
    xf_dot_async(u->g, XF_F64, u->zd, r, 10);
    xf_dot_async(u->g, XF_F64, u->zd, u->az, 11);
    xf_dot_async(u->g, XF_F64, e, r, 12);
    k_anorm_grad<<<ublocks(ctx, L[0].n), 256, 0, s>>>(r, u->az, L[0].mask, L[0].n, ctx->scratch, u->red,
                                                      u->G0_16a.p0(L), u->G0_16a.ps());
  } else {
    k_sumsq<<<sumsq_blocks(ctx, L[0].n), 256, 0, s>>>(e, L[0].mask, L[0].n, u->red, 1, u->rpart, u->rtick);
    k_unet_loss<<<ublocks(ctx, L[0].n), 256, 0, s>>>(u->zout, e, L[0].mask, L[0].n, (double)L[0].active, u->red,
                                                     u->G0_16a.p0(L), u->G0_16a.ps());
  }
  // out, dec0b, dec0a
  if ((st = wgrad(u, OUTL, u->G0_16a, u->D0b, 0))) return st;
  if ((st = dgrad(u, OUTL, u->G0_16a, u->G0_16b, 0, &u->D0b, 0))) return st;
  if ((st = wgrad(u, DEC0B, u->G0_16b, u->D0a, 0))) return st;
  if ((st = dgrad(u, DEC0B, u->G0_16b, u->G0_16a, 0, &u->D0a, 0))) return st;
  if ((st = wgrad(u, DEC0A, u->G0_16a, u->CAT0, 0))) return st;
  if ((st = dgrad(u, DEC0A, u->G0_16a, u->G0_48, 0, nullptr, 0))) return st;
  // up(D1b) part -> dec1b's pre-activation gradient
  k_upsample_bwd<<<ublocks(ctx, L[1].n * 32), 256, 0, s>>>(u->G0_48.p0(L), u->G0_48.ps(), L[0].n2, L[0].n3,
                                                           u->D1b.p0(L), u->D1b.ps(), L[1].mask, L[1].n1, L[1].n2,
                                                           L[1].n3, u->G1_32a.p0(L), u->G1_32a.ps(), 32);
  if ((st = wgrad(u, DEC1B, u->G1_32a, u->D1a, 0))) return st;
  if ((st = dgrad(u, DEC1B, u->G1_32a, u->G1_32b, 0, &u->D1a, 0))) return st;
  if ((st = wgrad(u, DEC1A, u->G1_32b, u->CAT1, 0))) return st;
  if ((st = dgrad(u, DEC1A, u->G1_32b, u->G1_96, 0, nullptr, 0))) return st;
  // up(M2b) part -> mid_b
  k_upsample_bwd<<<ublocks(ctx, L[2].n * 64), 256, 0, s>>>(u->G1_96.p0(L), u->G1_96.ps(), L[1].n2, L[1].n3,
                                                           u->M2b.p0(L), u->M2b.ps(), L[2].mask, L[2].n1, L[2].n2,
                                                           L[2].n3, u->G2_64a.p0(L), u->G2_64a.ps(), 64);
  if ((st = wgrad(u, MIDB, u->G2_64a, u->M2a, 0))) return st;
  if ((st = dgrad(u, MIDB, u->G2_64a, u->G2_64b, 0, &u->M2a, 0))) return st;
  if ((st = wgrad(u, MIDA, u->G2_64b, u->P2, 0))) return st;
  if ((st = dgrad(u, MIDA, u->G2_64b, u->G2_32, 0, nullptr, 0))) return st;
  k_pool_bwd<<<ublocks(ctx, L[1].n * 32), 256, 0, s>>>(u->G2_32.p0(L), u->G2_32.ps(), L[2].n2, L[2].n3, L[1].mask,
                                                       L[1].n1, L[1].n2, L[1].n3, u->gsum1, 32, 32);
  // S1 = enc1b output: skip gradient + pooled path
  k_skip_grad<<<ublocks(ctx, L[1].n * 32), 256, 0, s>>>(u->G1_96.ch(L, 64), u->G1_96.ps(), u->gsum1, 32,
                                                        u->CAT1.ch(L, 64), u->CAT1.ps(), L[1].mask, L[1].n,
                                                        u->G1_32a.p0(L), u->G1_32a.ps(), 32);
  if ((st = wgrad(u, ENC1B, u->G1_32a, u->A1, 0))) return st;
  if ((st = dgrad(u, ENC1B, u->G1_32a, u->G1_32b, 0, &u->A1, 0))) return st;
  if ((st = wgrad(u, ENC1A, u->G1_32b, u->P1, 0))) return st;
  if ((st = dgrad(u, ENC1A, u->G1_32b, u->G1_16, 0, nullptr, 0))) return st;
  k_pool_bwd<<<ublocks(ctx, L[0].n * 16), 256, 0, s>>>(u->G1_16.p0(L), u->G1_16.ps(), L[1].n2, L[1].n3, L[0].mask,
                                                       L[0].n1, L[0].n2, L[0].n3, u->gsum, 16, 16);
  k_skip_grad<<<ublocks(ctx, L[0].n * 16), 256, 0, s>>>(u->G0_48.ch(L, 32), u->G0_48.ps(), u->gsum, 16,
                                                        u->CAT0.ch(L, 32), u->CAT0.ps(), L[0].mask, L[0].n,
                                                        u->G0_16a.p0(L), u->G0_16a.ps(), 16);
  if ((st = wgrad(u, ENC0B, u->G0_16a, u->A0, 0))) return st;
  if ((st = dgrad(u, ENC0B, u->G0_16a, u->G0_16b, 0, &u->A0, 0))) return st;
  if ((st = wgrad(u, ENC0A, u->G0_16b, u->X0, 0))) return st;
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

static int check_box(const xf_unet* u, const xf_vec* v, const char* who) {
  if (!v || v->g != u->g || v->dtype != XF_F64)
    return xf_fail(u->ctx, XF_ERR_STATE, "%s: FP64 boxes of the network's grid expected", who);
  return XF_OK;
}

// z = U-Net(r), FP64 box (0 on inactive cells).
int xf_unet_apply_dev(xf_unet* u, const double* r, double* z) {
  int st = forward(u, r);
  if (st) return st;
  k_f2d_mask<<<ublocks(u->ctx, u->L[0].n), 256, 0, u->ctx->stream>>>(u->zout, u->L[0].mask, u->L[0].n, z);
  XF_CUDA(u->ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_unet_apply(xf_unet* u, const xf_vec* r, xf_vec* z) {
  if (!u) return XF_ERR_ARG;
  int st;
  if ((st = check_box(u, r, "xf_unet_apply")) || (st = check_box(u, z, "xf_unet_apply"))) return st;
  XF_CUDA(u->ctx, cudaSetDevice(u->ctx->device));
  if ((st = xf_unet_apply_dev(u, (const double*)r->data, (double*)z->data))) return st;
  return xf_conv_status(u->ctx);
}

extern "C" int xf_unet_train_step(xf_unet* u, const xf_op* op, const xf_vec* r, const xf_vec* e, double lr,
                                  int apply_update, double* loss) {
  if (!u) return XF_ERR_ARG;
  int st;
  if ((st = check_box(u, r, "xf_unet_train_step")) || (st = check_box(u, e, "xf_unet_train_step"))) return st;
  if (op && (op->g != u->g || op->kind == XF_OP_PACK))
    return xf_fail(u->ctx, XF_ERR_ARG, "xf_unet_train_step: the operator must be a stencil operator of the network's grid");
  if (op && (st = xf_op_ready(op))) return st;
  xf_ctx* ctx = u->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  for (Layer& y : u->ly) {
    XF_CUDA(ctx, cudaMemsetAsync(y.gw, 0, y.nw * 4, s));
    XF_CUDA(ctx, cudaMemsetAsync(y.gb, 0, y.co * 4, s));
  }
  if ((st = forward(u, (const double*)r->data))) return st;
  if ((st = backward(u, (const double*)r->data, (const double*)e->data, op))) return st;
  if (apply_update) {
    u->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)u->step), c2 = 1.f - powf(b2, (float)u->step);
    for (Layer& y : u->ly) {
      k_adam<<<ublocks(ctx, y.nw), 256, 0, s>>>(y.w, y.gw, y.mw, y.vw, y.nw, (float)lr, b1, b2, 1e-8f, c1, c2, 0);
      k_adam<<<1, 256, 0, s>>>(y.b, y.gb, y.mb, y.vb, y.co, (float)lr, b1, b2, 1e-8f, c1, c2, 0);
      k_weights_bf16<<<ublocks(ctx, y.nw), 256, 0, s>>>(y.w, y.co, y.ci, y.w16, y.wt16, y.w16t, y.wt16t);
    }
  }
  XF_CUDA(ctx, cudaGetLastError());
  if (loss) {
    XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, u->red + 2, 8, cudaMemcpyDeviceToHost, s));
  }
  if ((st = xf_conv_status(ctx))) return st;   // synchronises
  if (loss) *loss = ctx->host_scalars[0];
  return XF_OK;
}

// ---------------------------------------------------------------------------
// Flexible CG, truncated FCG(m) (Notay's flexible CG): each new preconditioned
// residual z = M(r) is A-orthogonalised against the last m search directions,
//     p = z - sum_j ((z, A p_j) / (p_j, A p_j)) p_j,
// which keeps the method robust to a preconditioner that varies from one
// application to the next (a network), then x += alpha p, r -= alpha A p with
// alpha = (p, r) / (p, A p).  FP64 vectors and dots.  Plain CG stays the
// fallback and the arbiter: an iteration whose z is no descent direction
// ((z, r) <= 0, or not finite) uses z = r; the third such iteration, or a
// residual that has not dropped by 10% over 50 iterations, switches the
// preconditioner off for the rest of the solve (all counted in
// stats->fallbacks).  The stop rule is the true relative
// residual ||b - A x|| <= rtol ||b||.  m = opts->reserved[0] (1..8, default 8).
constexpr int FCG_STRIKES = 3;   // non-descent preconditioned directions before the network is switched off
__global__ void k_fcg_update(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                             const double* __restrict__ q, double alpha, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    x[c] += alpha * p[c];
    r[c] -= alpha * q[c];
  }
}
__global__ void k_axpy_d(double* __restrict__ y, const double* __restrict__ x, double a, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    y[c] += a * x[c];
}
__global__ void k_jacobi(const double* __restrict__ r, const double* __restrict__ diag, const uint8_t* __restrict__ kind,
                         int64_t n, double* __restrict__ z) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const double d = diag[c];
    z[c] = (row_of(kind[c]) == ROW_ACTUAL && d > 0) ? r[c] / d : r[c];
  }
}

// The learned two-level preconditioner (XF_PRECOND_UNET2).  The network is
// built on a coarse grid whose interior cells are the F x F x F blocks of the
// fine interior (ghost layers match), and serves as the coarse solver; the
// FP32 Chebyshev polynomial of the mixed CG (factored, one two-level pass
// per factor) smooths what it leaves:
//   y = P N(P^T r)             P: piecewise constant over the blocks
//   omega = (y, r) / (y, A y)  the A-norm optimal step along y (the network's
//                              output scale is arbitrary)
//   z = omega y + s p(A) (r - omega A y)
// s makes lambda s p(lambda) closest to 1 on [lambda_max / ratio, lambda_max].
template <typename T>
__global__ void k_restrict_blocks(const T* __restrict__ r, int f2, int f3, int F, double* __restrict__ rc, int c1,
                                  int c2, int c3) {
  const int64_t nc = (int64_t)c1 * c2 * c3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const int K = (int)(c % c3);
    const int64_t t = c / c3;
    const int J = (int)(t % c2), I = (int)(t / c2);
    double v = 0.0;
    if (I > 0 && I < c1 - 1 && J > 0 && J < c2 - 1 && K > 0 && K < c3 - 1) {
      const int i0 = 1 + (I - 1) * F, j0 = 1 + (J - 1) * F, k0 = 1 + (K - 1) * F;
      for (int a = 0; a < F; a++)
        for (int b = 0; b < F; b++) {
          const T* row = r + ((int64_t)(i0 + a) * f2 + (j0 + b)) * f3 + k0;
          for (int q = 0; q < F; q++) v += (double)row[q];
        }
    }
    rc[c] = v;
  }
}
template <typename T>
__global__ void k_prolong_blocks(const double* __restrict__ zc, int c2, int c3, int F, const uint8_t* __restrict__ smask,
                                 int f1, int f2, int f3, T* __restrict__ y) {
  const int64_t n = (int64_t)f1 * f2 * f3;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(c % f3);
    const int64_t t = c / f3;
    const int j = (int)(t % f2), i = (int)(t / f2);
    double v = 0.0;
    if (smask[c] && i > 0 && i < f1 - 1 && j > 0 && j < f2 - 1 && k > 0 && k < f3 - 1)
      v = zc[((int64_t)(1 + (i - 1) / F) * c2 + (1 + (j - 1) / F)) * c3 + (1 + (k - 1) / F)];
    y[c] = (T)v;
  }
}
template <typename T>
__global__ void k_sub_f32(const T* __restrict__ r, const T* __restrict__ q, double om, int64_t n,
                          float* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    out[c] = (float)((double)r[c] - om * (double)q[c]);
}
template <typename T>
__global__ void k_twolevel_z(const T* __restrict__ y, const float* __restrict__ w, double om, double sc,
                             const uint8_t* __restrict__ smask, int64_t n, T* __restrict__ z) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    z[c] = smask[c] ? (T)(om * (double)y[c] + sc * (double)w[c]) : (T)0;
}
// The F = 4 transfers of the mixed path.  Restriction: one thread per coarse
// cell, its 64 loads unrolled (a warp reads 32 consecutive runs of 4 floats).
// Prolongation: 2-D grid over (j, k) plane positions and i planes, 32-bit
// index arithmetic.
__global__ void k_restrict4(const float* __restrict__ r, int f2, int f3, double* __restrict__ rc, int c1, int c2,
                            int c3) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, I = blockIdx.z;
  if (K >= c3) return;
  double v = 0.0;
  if (I > 0 && I < c1 - 1 && J > 0 && J < c2 - 1 && K > 0 && K < c3 - 1) {
    const int64_t base = ((int64_t)(1 + 4 * (I - 1)) * f2 + (1 + 4 * (J - 1))) * f3 + (1 + 4 * (K - 1));
    float part[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      float sa = 0.f;
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const float* row = r + base + ((int64_t)a * f2 + b) * f3;
        sa += (__ldg(row) + __ldg(row + 1)) + (__ldg(row + 2) + __ldg(row + 3));
      }
      part[a] = sa;
    }
    v = ((double)part[0] + (double)part[1]) + ((double)part[2] + (double)part[3]);
  }
  rc[((int64_t)I * c2 + J) * c3 + K] = v;
}
// Four consecutive cells of a plane per thread: one 4-byte mask load and one
// 16-byte store.  With F = 4 every fine interior extent is a multiple of 4, so
// n2 = 4a + 2 and n3 = 4b + 2 and the plane size n2 n3 is a multiple of 4;
// with the 256-byte aligned allocations of y and the space mask, every
// thread's group then starts on a 16-byte (y) and 4-byte (mask) boundary.
__global__ void k_prolong4v(const double* __restrict__ zc, int c2, int c3, const uint8_t* __restrict__ smask, int f1,
                            int f2, int f3, float* __restrict__ y) {
  const int P = f2 * f3;
  const int p0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x), i = blockIdx.y;
  if (p0 >= P) return;
  const int64_t c0 = (int64_t)i * P + p0;
  const uchar4 m4 = *reinterpret_cast<const uchar4*>(smask + c0);
  const unsigned char mk[4] = {m4.x, m4.y, m4.z, m4.w};
  int j = p0 / f3, k = p0 - j * f3;
  float v[4];
  const bool irow = i > 0 && i < f1 - 1;
  const int64_t ib = (int64_t)(1 + ((i - 1) >> 2)) * c2;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float t = 0.f;
    if (mk[q] && irow && j > 0 && j < f2 - 1 && k > 0 && k < f3 - 1)
      t = (float)__ldg(&zc[(ib + (1 + ((j - 1) >> 2))) * c3 + (1 + ((k - 1) >> 2))]);
    v[q] = t;
    if (++k == f3) {
      k = 0;
      j++;
    }
  }
  *reinterpret_cast<float4*>(y + c0) = make_float4(v[0], v[1], v[2], v[3]);
}
// (a, b) of FP32 boxes that are zero off the active set: exact products
// accumulated in float-float per thread and per warp, FP64 across warps and
// blocks; 16-byte loads.  -> scalars[slot]
// skip (may be null): a device flag; when set the dot is not computed
__global__ void __launch_bounds__(RED_THREADS) k_dot_f4(const float* __restrict__ a, const float* __restrict__ b,
                                                        int64_t n, DevScratch* S, int slot, const int* skip) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (skip && *skip) return;
  DotAcc<float> acc;
  const int64_t n4 = n >> 2, stride = (int64_t)gridDim.x * blockDim.x;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  const float4* b4 = reinterpret_cast<const float4*>(b);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n4; c += stride) {
    const float4 x = __ldg(a4 + c), y = __ldg(b4 + c);
    acc.add(x.x, y.x);
    acc.add(x.y, y.y);
    acc.add(x.z, y.z);
    acc.add(x.w, y.w);
  }
  for (int64_t c = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += stride) acc.add(a[c], b[c]);
  if (!publish_acc<float>(S, slot, slot, acc, sh, &last)) return;
  const double t = finish_partials(S, slot, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = t;
    S->tickets[slot] = 0;
  }
}
// mixed FCG vector kernels (FP32 vectors)
__global__ void k_fcg_update_f(float* __restrict__ e, float* __restrict__ r, const float* __restrict__ p,
                               const float* __restrict__ q, float alpha, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    e[c] = fmaf(alpha, p[c], e[c]);
    r[c] = fmaf(-alpha, q[c], r[c]);
  }
}
__global__ void k_axpy_f(float* __restrict__ y, const float* __restrict__ x, float a, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    y[c] = fmaf(a, x[c], y[c]);
}
__global__ void k_d2f(const double* __restrict__ a, int64_t n, float* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    out[c] = (float)a[c];
}
__global__ void k_fold_f2d(double* __restrict__ x, const float* __restrict__ e, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    x[c] += (double)e[c];
}

// The factor of the smoothing polynomial: 2 / (min + max) of lambda p(lambda)
// over [lmax / ratio, lmax], p the product of the quadratic factors.
static double cheb_scale(const float (*f)[3], int nf, double lmax, double ratio) {
  double gmin = 1e300, gmax = -1e300;
  const double lo = lmax / ratio;
  for (int q = 0; q <= 8192; q++) {
    const double lam = lo + (lmax - lo) * q / 8192.0;
    double p = 1.0;
    for (int k = 0; k < nf; k++) p *= (double)f[k][0] + lam * ((double)f[k][1] + lam * (double)f[k][2]);
    gmin = fmin(gmin, lam * p);
    gmax = fmax(gmax, lam * p);
  }
  return 2.0 / (gmin + gmax);
}

// scalar slots: 0..7 (z, A p_j); 8 (y, A y), 9 (y, r) of the two-level preconditioner; 10 (z, r); 11 (r, r);
// 12 (p, r); 14/15 matvec dots
enum { FS_YAY = 8, FS_YR = 9, FS_ZR = 10, FS_RR = 11, FS_PR = 12, FS_PQ = 14 };

static int read_n(xf_ctx* ctx, int first, int count, double* out) {
  XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->scalars[first], count * 8, cudaMemcpyDeviceToHost,
                               ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int q = 0; q < count; q++) out[q] = ctx->host_scalars[q];
  return XF_OK;
}

// ---------------------------------------------------------------------------
// Mixed-precision FCG(m) with the learned two-level preconditioner, driven
// entirely on the device: the correction e, the residual r, the directions
// and their images are FP32; the dots are accumulated in FP64 (exact FP32
// products summed in float-float, then FP64); alpha and the window
// coefficients are FP64.  The FP32 recursion is refreshed from the true
// residual b - A x, computed in FP64 after x += e, every `replace_every`
// iterations, whenever its (r, r) has dropped by 10^6 since the last
// refresh, and when it meets the tolerance; the window of directions is kept
// across a refresh.  The solve ends only on the true FP64 residual.
//
// Every scalar decision (alpha, the window coefficients, the fallback to
// z = r, the refresh and stop tests) is taken by one-thread control kernels
// on the device, and the whole solve is one CUDA graph with conditional
// nodes, so it needs no host round trip:
//
//   init: (b, b), the tolerance, the state
//   WHILE (not done):
//     IF (refresh):   x += e (after a cycle), e = 0, r = float(b - A x) in
//                     FP64 with (r, r); the stop, iteration-cap and stall
//                     tests
//     IF (head == 0): one iteration with direction slot 0
//     ...
//     IF (head == m): one iteration with direction slot m
//     the loop guard
//
// The m + 1 iteration blocks are the ring positions of the new direction, so
// every kernel argument is fixed at capture.  Inside an iteration block:
//   IF/ELSE (network on): z = M r (restriction, U-Net, prolongation, A y, the
//                         smoother passes reducing (z, r), (z, q_0)) /
//                         z = r with its dots
//   IF (no descent direction, (z, r) <= 0): z = r with its dots; the third
//                         time the network is switched off
//   p = z - sum_j (z, q_j) / (p_j, q_j) p_j, q = A p, (p, q), (p, r), alpha,
//   e += alpha p, r -= alpha q, (r, r), the cycle-end test.
// The loop guard ends the loop when the solve is done, and with an error
// status if a pass made no iteration (the control always runs one per pass
// until it ends the solve) or the passes exceed the iteration cap, so the
// device loop ends whatever the handles hold.  The graph, the workspace and
// the state are built once per operator, vectors and settings, and kept with
// the network.
struct TlCtl {
  double bb, thr, rr_true, rr_prev_true, rr, rr_start, alpha;
  double pq_win[9];
  float coef[8];
  int use_coef[8];
  int win_off[8];   // window dot j skipped (j >= nwin)
  int it, it_start, maxit, every, repl, prev_cycle, fallbacks, precond_on, head, nwin, done, status, brk, cycle_ran;
  int passes, it_seen;   // the loop guard
  long long launches;
};
struct TlParams {
  double rtol2;
  int maxit, every;
  // kernels per segment, for the launch count
  int n_ref, n_iter, n_on, n_off, n_fb;
};
struct TlHandles {
  cudaGraphConditionalHandle main, ref, blk[9], pre[9], fb[9];
};

struct TlGraph {
  unsigned long long op_serial = 0;
  const void *x = nullptr, *b = nullptr;
  int m = 0, F = 0, nf = 0;
  float f[6][3] = {};
  double scale = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> bufs;
  TlCtl* ctl = nullptr;
  TlParams* prm = nullptr;
  ~TlGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : bufs) cudaFree(p);
  }
};

void xf_tl_graph_free(TlGraph* t) { delete t; }

__global__ void k_tl_init(DevScratch* S, TlCtl* c, const TlParams* p, TlHandles h, int m) {
  if (threadIdx.x | blockIdx.x) return;
  cudaGraphSetConditional(h.ref, 1u);   // the loop starts with a refresh
  for (int k = 0; k <= m; k++) cudaGraphSetConditional(h.blk[k], 0u);
  c->passes = 0; c->it_seen = 0;
  c->bb = S->scalars[FS_RR];
  c->thr = p->rtol2 * c->bb;
  c->maxit = p->maxit; c->every = p->every;
  c->it = 0; c->it_start = 0; c->repl = 0; c->prev_cycle = 0; c->fallbacks = 0; c->precond_on = 1;
  c->head = 0; c->nwin = 0; c->done = 0; c->status = XF_OK; c->brk = 0; c->cycle_ran = 0;
  c->rr_true = 0; c->rr_prev_true = 0; c->rr = 0; c->rr_start = 0; c->alpha = 0;
  for (int j = 0; j < 9; j++) c->pq_win[j] = 0;
  for (int j = 0; j < 8; j++) { c->coef[j] = 0.f; c->use_coef[j] = 0; c->win_off[j] = 1; }
  c->launches = 2;
}
// x += e after a cycle (none before the first)
__global__ void k_tl_fold(double* __restrict__ x, const float* __restrict__ e, int64_t n, const TlCtl* c) {
  if (!c->cycle_ran) return;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    x[q] += (double)e[q];
}
// after the refresh: the stop, cap and stall tests; the next block
__global__ void k_tl_top(DevScratch* S, TlCtl* c, const TlParams* p, TlHandles h, int m) {
  if (threadIdx.x | blockIdx.x) return;
  c->cycle_ran = 0;
  c->launches += p->n_ref;
  const double rr = S->scalars[FS_PQ + 1];
  c->rr_true = rr;
  if (c->brk) {
    c->done = 1;
  } else if (rr <= c->thr) {
    c->done = 1;
  } else if (isnan(rr)) {
    c->done = 1; c->status = XF_NAN;
  } else if (c->it >= c->maxit) {
    c->done = 1; c->status = XF_MAXIT;
  } else {
    // no progress over a whole refresh cycle of 10 or more iterations: plain CG from here on
    if (c->repl > 0 && c->precond_on && c->prev_cycle >= 10 && !(rr < 0.81 * c->rr_prev_true)) {
      c->precond_on = 0;
      c->fallbacks++;
    }
    c->rr_prev_true = rr;
    c->rr_start = rr;
    c->rr = rr;
    c->it_start = c->it;
  }
  cudaGraphSetConditional(h.main, c->done ? 0u : 1u);
  cudaGraphSetConditional(h.ref, 0u);
  for (int k = 0; k <= m; k++) cudaGraphSetConditional(h.blk[k], (!c->done && k == c->head) ? 1u : 0u);
}
__global__ void k_tl_it(TlCtl* c, const TlParams* p, cudaGraphConditionalHandle pre, int m) {
  if (threadIdx.x | blockIdx.x) return;
  c->it++;
  for (int j = 0; j < m; j++) c->win_off[j] = j >= c->nwin;
  c->launches += p->n_iter + (c->precond_on ? p->n_on : p->n_off);
  cudaGraphSetConditional(pre, c->precond_on ? 1u : 0u);
}
__global__ void k_tl_z(DevScratch* S, TlCtl* c, const TlParams* p, cudaGraphConditionalHandle fb) {
  if (threadIdx.x | blockIdx.x) return;
  const bool bad = !(S->scalars[FS_ZR] > 0) && c->precond_on;   // no descent direction: use r this time
  if (bad) {
    if (++c->fallbacks >= FCG_STRIKES) c->precond_on = 0;   // and from the third on, for good
    c->launches += p->n_fb;
  }
  cudaGraphSetConditional(fb, bad ? 1u : 0u);
}
// the window coefficients -(z, q_j) / (p_j, q_j) of the block with direction slot hd
// The window's last term of the new direction with (p, r): p += coef_j p_j
// (when the control kept term j) and (p, r) into scalars[slot] in one pass;
// k_dot_f4's grid, mapping and order, so (p, r) is bit for bit the separate dot's.
__global__ void __launch_bounds__(RED_THREADS) k_tl_axpy_pr(float* __restrict__ y, const float* __restrict__ x,
                                                            const float* __restrict__ r, const TlCtl* c, int j,
                                                            int64_t n, DevScratch* S, int slot) {
  __shared__ double sh[32];
  __shared__ bool last;
  const bool use = c->use_coef[j] != 0;
  const float a = c->coef[j];
  DotAcc<float> acc;
  const int64_t n4 = n >> 2, stride = (int64_t)gridDim.x * blockDim.x;
  float4* y4 = reinterpret_cast<float4*>(y);
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4* r4 = reinterpret_cast<const float4*>(r);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n4; k += stride) {
    float4 v = y4[k];
    if (use) {
      const float4 xv = __ldg(x4 + k);
      v.x = fmaf(a, xv.x, v.x); v.y = fmaf(a, xv.y, v.y); v.z = fmaf(a, xv.z, v.z); v.w = fmaf(a, xv.w, v.w);
      y4[k] = v;
    }
    const float4 rv = __ldg(r4 + k);
    acc.add(v.x, rv.x);
    acc.add(v.y, rv.y);
    acc.add(v.z, rv.z);
    acc.add(v.w, rv.w);
  }
  for (int64_t k = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += stride) {
    float v = y[k];
    if (use) {
      v = fmaf(a, x[k], v);
      y[k] = v;
    }
    acc.add(v, r[k]);
  }
  if (!publish_acc<float>(S, slot, slot, acc, sh, &last)) return;
  const double t = finish_partials(S, slot, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = t;
    S->tickets[slot] = 0;
  }
}
__global__ void k_tl_coef(const DevScratch* S, TlCtl* c, int hd, int m) {
  if (threadIdx.x | blockIdx.x) return;
  for (int j = 0; j < m; j++) {
    const int sl = (hd + m - j) % (m + 1);
    const bool use = j < c->nwin && c->pq_win[sl] > 0;
    c->use_coef[j] = use;
    c->coef[j] = use ? (float)(-S->scalars[j] / c->pq_win[sl]) : 0.f;
  }
}
__global__ void k_tl_axpy(float* __restrict__ y, const float* __restrict__ x, const TlCtl* c, int j, int64_t n) {
  if (!c->use_coef[j]) return;
  const float a = c->coef[j];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    y[q] = fmaf(a, x[q], y[q]);
}
__global__ void k_tl_alpha(const DevScratch* S, TlCtl* c, int hd, int m) {
  if (threadIdx.x | blockIdx.x) return;
  const double pr = S->scalars[FS_PR], pq = S->scalars[FS_PQ];
  if (!(pq > 0)) {
    c->status = isnan(pq) ? XF_NAN : XF_BREAKDOWN;
    c->brk = 1;
    return;
  }
  c->alpha = pr / pq;
  c->pq_win[hd] = pq;
  c->head = (hd + 1) % (m + 1);
  if (c->nwin < m) c->nwin++;
}
// e += alpha p, r -= alpha q and (r, r) into scalars[slot] in the same pass;
// the grid, the thread mapping and the accumulation order are k_dot_f4's, so
// (r, r) is bit for bit the separate dot's.
__global__ void __launch_bounds__(RED_THREADS) k_tl_update(float* __restrict__ e, float* __restrict__ r,
                                                           const float* __restrict__ p, const float* __restrict__ q,
                                                           const TlCtl* c, int64_t n, DevScratch* S, int slot) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (c->brk) return;
  const float alpha = (float)c->alpha;
  DotAcc<float> acc;
  const int64_t n4 = n >> 2, stride = (int64_t)gridDim.x * blockDim.x;
  float4* e4 = reinterpret_cast<float4*>(e);
  float4* r4 = reinterpret_cast<float4*>(r);
  const float4* p4 = reinterpret_cast<const float4*>(p);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n4; k += stride) {
    float4 ev = e4[k], rv = r4[k];
    const float4 pv = __ldg(p4 + k), qv = __ldg(q4 + k);
    ev.x = fmaf(alpha, pv.x, ev.x); ev.y = fmaf(alpha, pv.y, ev.y);
    ev.z = fmaf(alpha, pv.z, ev.z); ev.w = fmaf(alpha, pv.w, ev.w);
    rv.x = fmaf(-alpha, qv.x, rv.x); rv.y = fmaf(-alpha, qv.y, rv.y);
    rv.z = fmaf(-alpha, qv.z, rv.z); rv.w = fmaf(-alpha, qv.w, rv.w);
    e4[k] = ev;
    r4[k] = rv;
    acc.add(rv.x, rv.x);
    acc.add(rv.y, rv.y);
    acc.add(rv.z, rv.z);
    acc.add(rv.w, rv.w);
  }
  for (int64_t k = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += stride) {
    e[k] = fmaf(alpha, p[k], e[k]);
    const float rv = fmaf(-alpha, q[k], r[k]);
    r[k] = rv;
    acc.add(rv, rv);
  }
  if (!publish_acc<float>(S, slot, slot, acc, sh, &last)) return;
  const double t = finish_partials(S, slot, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = t;
    S->tickets[slot] = 0;
  }
}
// The last node of the loop body: see the loop guard above.
__global__ void k_tl_guard(TlCtl* c, TlHandles h) {
  if (threadIdx.x | blockIdx.x) return;
  c->passes++;
  if (!c->done && (c->it == c->it_seen || c->passes > c->maxit + 16)) {
    c->done = 1;
    c->status = XF_ERR_CUDA;
  }
  c->it_seen = c->it;
  cudaGraphSetConditional(h.main, c->done ? 0u : 1u);
}
// the cycle-end test after the iteration in block hd; sets the next block
__global__ void k_tl_rr(const DevScratch* S, TlCtl* c, TlHandles h, int hd, int m) {
  if (threadIdx.x | blockIdx.x) return;
  bool end = c->brk != 0;
  if (!end) {
    const double rr = S->scalars[FS_RR];
    c->rr = rr;
    end = isnan(rr) || rr <= c->thr || rr <= 1e-6 * c->rr_start || c->it - c->it_start >= c->every ||
          c->it >= c->maxit;
  }
  if (end) {
    c->cycle_ran = 1;
    c->repl++;
    c->prev_cycle = c->it - c->it_start;
    cudaGraphSetConditional(h.ref, 1u);
    for (int k = hd + 1; k <= m; k++) cudaGraphSetConditional(h.blk[k], 0u);
  } else {
    cudaGraphSetConditional(h.blk[hd < m ? hd + 1 : 0], 1u);
  }
}

static int tl_graph_build(xf_op* op, xf_unet* u, int m, int F, const float (*tl_f)[3], int tl_nf, double tl_scale,
                          xf_vec* xv, const xf_vec* bv, TlGraph** out) {
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  const xf_grid* cg = u->g;
  const int64_t n = g->ncell, nc = cg->ncell;
  cudaStream_t s = ctx->stream;
  const int eb = grid_blocks(ctx, n, 256);
  const int db = red_blocks(ctx, (n + 3) / 4);
  TlGraph* t = new TlGraph();
  auto fail = [&](int code, const char* msg) {
    delete t;
    return xf_fail(ctx, code, "xf_solve_fcg: %s", msg);
  };
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    cudaMemsetAsync(p, 0, bytes, s);
    t->bufs.push_back(p);
    return p;
  };
  double *rc = (double*)alloc(nc * 8), *zc = (double*)alloc(nc * 8);
  float *r = (float*)alloc(n * 4), *e = (float*)alloc(n * 4), *z = (float*)alloc(n * 4), *y = (float*)alloc(n * 4);
  float *ay = (float*)alloc(n * 4), *w0 = (float*)alloc(n * 4), *w1 = (float*)alloc(n * 4);
  t->ctl = (TlCtl*)alloc(sizeof(TlCtl));
  t->prm = (TlParams*)alloc(sizeof(TlParams));
  float *P[9] = {nullptr}, *Q[9] = {nullptr};   // ring of m + 1: the new direction and the window
  bool ok = rc && zc && r && e && z && y && ay && w0 && w1 && t->ctl && t->prm;
  for (int j = 0; j <= m && ok; j++) ok = (P[j] = (float*)alloc(n * 4)) && (Q[j] = (float*)alloc(n * 4));
  if (!ok) return fail(XF_ERR_NOMEM, "allocation");
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(XF_ERR_CUDA, "workspace");
  double* x = (double*)xv->data;
  const double* b = (const double*)bv->data;
  DevScratch* S = ctx->scratch;
  TlCtl* c = t->ctl;
  const TlParams* prm = t->prm;
  auto fdot = [&](const float* a, const float* b2, int slot, const int* skip) {
    k_dot_f4<<<db, RED_THREADS, 0, s>>>(a, b2, n, S, slot, skip);
  };
  // the window dots j = j0 .. m-1 of block hd (skipped on the device while j >= nwin)
  auto win_dots = [&](int hd, int j0) {
    for (int j = j0; j < m; j++) fdot(z, Q[(hd + m - j) % (m + 1)], j, &c->win_off[j]);
  };
  // warm the network's kernels (attributes, first launches) outside capture
  int rcode = xf_unet_apply_dev(u, rc, zc);
  if (rcode) {
    delete t;
    return rcode;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(XF_ERR_CUDA, "warm-up");

  TlHandles H;
  cudaGraph_t top = nullptr;
  if (cudaGraphCreate(&top, 0) != cudaSuccess) return fail(XF_ERR_CUDA, "graph");
  t->graph = top;
  cudaError_t ce = cudaSuccess;
  // capture a sequence into graph gr after the nodes deps ...
  auto begin = [&](cudaGraph_t gr, const cudaGraphNode_t* deps, size_t nd) {
    if (ce == cudaSuccess) ce = cudaStreamBeginCaptureToGraph(s, gr, deps, nullptr, nd, cudaStreamCaptureModeThreadLocal);
  };
  // ... and end it, returning its tail
  auto end_tail = [&](std::vector<cudaGraphNode_t>& tail) {
    if (ce != cudaSuccess) return;
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* d = nullptr;
    size_t nd = 0;
    ce = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd);
    if (ce == cudaSuccess) tail.assign(d, d + nd);
    cudaGraph_t dummy = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &dummy);
    if (ce == cudaSuccess) ce = e2;
  };
  auto add_cond = [&](cudaGraph_t gr, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle hnd,
                      cudaGraphConditionalNodeType type, unsigned size, cudaGraph_t* bodies,
                      cudaGraphNode_t* node) {
    if (ce != cudaSuccess) return;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hnd;
    np.conditional.type = type;
    np.conditional.size = size;
    ce = cudaGraphAddNode(node, gr, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &np);
    if (ce == cudaSuccess)
      for (unsigned q = 0; q < size; q++) bodies[q] = np.conditional.phGraph_out[q];
  };
  auto handle = [&](cudaGraph_t gr, cudaGraphConditionalHandle* hnd, unsigned dflt, unsigned flags) {
    if (ce == cudaSuccess) ce = cudaGraphConditionalHandleCreate(hnd, gr, dflt, flags);
  };

  // the loop node and the handles of its body's blocks first (the init kernel sets them)
  std::vector<cudaGraphNode_t> tail, unused;
  handle(top, &H.main, 1, cudaGraphCondAssignDefault);
  cudaGraph_t wbody = nullptr;
  cudaGraphNode_t wnode = nullptr;
  add_cond(top, {}, H.main, cudaGraphCondTypeWhile, 1, &wbody, &wnode);
  handle(wbody, &H.ref, 1, 0);
  for (int k = 0; k <= m; k++) handle(wbody, &H.blk[k], 0, 0);
  // init: (b, b), the state, the block handles; before the loop
  begin(top, nullptr, 0);
  xf_dot_async(g, XF_F64, b, b, FS_RR);
  k_tl_init<<<1, 32, 0, s>>>(S, c, prm, H, m);
  end_tail(tail);
  if (ce == cudaSuccess) {
    const std::vector<cudaGraphNode_t> to(tail.size(), wnode);   // every tail node before the loop
    ce = cudaGraphAddDependencies(top, tail.data(), to.data(), nullptr, tail.size());
  }
  // refresh block
  cudaGraph_t rbody = nullptr;
  cudaGraphNode_t prev = nullptr;
  add_cond(wbody, {}, H.ref, cudaGraphCondTypeIf, 1, &rbody, &prev);
  begin(rbody, nullptr, 0);
  k_tl_fold<<<eb, 256, 0, s>>>(x, e, n, c);
  cudaMemsetAsync(e, 0, n * 4, s);
  xf_cg_res64(op, x, b, r, FS_PQ, CTL_NONE);   // r = float(b - A x), (r, r) in FP64 -> FS_PQ + 1
  k_tl_top<<<1, 32, 0, s>>>(S, c, prm, H, m);   // reads H.main, H.ref, H.blk only
  end_tail(unused);
  // iteration blocks
  int n_on = 0, n_off = 0, n_fb = 0, n_iter = 0;
  for (int hd = 0; hd <= m; hd++) {
    cudaGraph_t bbody = nullptr;
    cudaGraphNode_t bnode = nullptr;
    add_cond(wbody, {prev}, H.blk[hd], cudaGraphCondTypeIf, 1, &bbody, &bnode);
    prev = bnode;
    handle(bbody, &H.pre[hd], 0, 0);
    handle(bbody, &H.fb[hd], 0, 0);
    float* pn = P[hd];
    float* qn = Q[hd];
    const float* q_newest = Q[(hd + m) % (m + 1)];
    // it++, the network-on test
    begin(bbody, nullptr, 0);
    k_tl_it<<<1, 32, 0, s>>>(c, prm, H.pre[hd], m);
    end_tail(tail);
    cudaGraph_t ie[2] = {nullptr, nullptr};
    cudaGraphNode_t ienode = nullptr;
    add_cond(bbody, tail, H.pre[hd], cudaGraphCondTypeIf, 2, ie, &ienode);
    // network on: z = M r with (z, r) and (z, q_newest)
    begin(ie[0], nullptr, 0);
    if (F == 4)
      k_restrict4<<<dim3((cg->n3 + 63) / 64, cg->n2, cg->n1), 64, 0, s>>>(r, g->n2, g->n3, rc, cg->n1, cg->n2, cg->n3);
    else
      k_restrict_blocks<float><<<grid_blocks(ctx, nc, 256), 256, 0, s>>>(r, g->n2, g->n3, F, rc, cg->n1, cg->n2,
                                                                         cg->n3);
    if (ce == cudaSuccess && (rcode = xf_unet_apply_dev(u, rc, zc))) ce = cudaErrorUnknown;
    if (F == 4 && xf_tl_prolong_ay_supported(g)) {   // y = P zc, A y and (y, A y) in one pass
      xf_tl_prolong_ay(op, u->zout, cg->n2, cg->n3, y, ay, FS_YAY);   // the network's FP32 output
    } else {
      if (F == 4)   // n2 n3 is a multiple of 4 (see k_prolong4v)
        k_prolong4v<<<dim3((g->n2 * g->n3 / 4 + 255) / 256, g->n1), 256, 0, s>>>(zc, cg->n2, cg->n3, g->smask,
                                                                                g->n1, g->n2, g->n3, y);
      else
        k_prolong_blocks<float><<<eb, 256, 0, s>>>(zc, cg->n2, cg->n3, F, g->smask, g->n1, g->n2, g->n3, y);
      xf_cg_q32_dot(op, y, ay, FS_YAY);           // A y, (y, A y)
    }
    xf_dot_async(cg, XF_F64, zc, rc, FS_YR);   // (y, r) = (z_c, P^T r)
    {
      // the smoother: its first pass takes r - omega A y, its last writes
      // z = omega y + s p(A)(r - omega A y) (also into the direction slot) and reduces the dots
      float *src = nullptr, *dst = w0;
      for (int k = tl_nf - 1; k >= 0; k--) {
        const bool first = k == tl_nf - 1, last = k == 0;
        xf_cg_poly_tl_launch(op, first, last, first ? r : src, ay, last ? z : dst, tl_f[k], FS_YAY, FS_YR, y,
                             (float)tl_scale, pn, r, q_newest, FS_ZR, 0);
        src = dst;
        dst = dst == w0 ? w1 : w0;
      }
    }
    win_dots(hd, 1);
    end_tail(unused);
    n_on = (F == 4 && xf_tl_prolong_ay_supported(g) ? 3 : 4) + UNET_FORWARD_LAUNCHES + tl_nf + (m - 1);
    // network off: z = r with its dots
    begin(ie[1], nullptr, 0);
    cudaMemcpyAsync(z, r, n * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(pn, r, n * 4, cudaMemcpyDeviceToDevice, s);
    fdot(z, r, FS_ZR, nullptr);
    win_dots(hd, 0);
    end_tail(unused);
    n_off = 1 + m;
    // the descent test
    begin(bbody, &ienode, 1);
    k_tl_z<<<1, 32, 0, s>>>(S, c, prm, H.fb[hd]);
    end_tail(tail);
    cudaGraph_t fbody = nullptr;
    cudaGraphNode_t fnode = nullptr;
    add_cond(bbody, tail, H.fb[hd], cudaGraphCondTypeIf, 1, &fbody, &fnode);
    begin(fbody, nullptr, 0);
    cudaMemcpyAsync(z, r, n * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(pn, r, n * 4, cudaMemcpyDeviceToDevice, s);
    fdot(z, r, FS_ZR, nullptr);
    win_dots(hd, 0);
    end_tail(unused);
    n_fb = 1 + m;
    // the new direction, its image, alpha, the update, the cycle-end test
    begin(bbody, &fnode, 1);
    k_tl_coef<<<1, 32, 0, s>>>(S, c, hd, m);
    for (int j = 0; j < m - 1; j++) k_tl_axpy<<<eb, 256, 0, s>>>(pn, P[(hd + m - j) % (m + 1)], c, j, n);
    k_tl_axpy_pr<<<db, RED_THREADS, 0, s>>>(pn, P[(hd + 1) % (m + 1)], r, c, m - 1, n, S, FS_PR);   // with (p, r)
    xf_cg_q32_dot(op, pn, qn, FS_PQ);   // q = A p, (p, q)
    k_tl_alpha<<<1, 32, 0, s>>>(S, c, hd, m);
    k_tl_update<<<db, RED_THREADS, 0, s>>>(e, r, pn, qn, c, n, S, FS_RR);   // with (r, r)
    k_tl_rr<<<1, 32, 0, s>>>(S, c, H, hd, m);
    end_tail(unused);
    // it, z-test, coef, m axpys (the last with (p, r)), stencil + dot, alpha, update with (r, r), test, and
    // the loop guard
    n_iter = 3 + m + 1 + 1 + 1 + 1 + 1;
  }
  // the loop guard, last in the body
  begin(wbody, &prev, 1);
  k_tl_guard<<<1, 32, 0, s>>>(c, H);
  end_tail(unused);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return fail(rcode ? rcode : XF_ERR_CUDA, rcode ? "preconditioner" : "graph capture");
  }
  ce = cudaGraphInstantiate(&t->exec, top, 0);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return fail(XF_ERR_CUDA, cudaGetErrorString(ce));
  }
  TlParams hp = {};
  hp.n_ref = 3; hp.n_iter = n_iter; hp.n_on = n_on; hp.n_off = n_off; hp.n_fb = n_fb;
  if (cudaMemcpy(t->prm, &hp, sizeof(hp), cudaMemcpyHostToDevice) != cudaSuccess) return fail(XF_ERR_CUDA, "params");
  t->op_serial = op->serial; t->x = xv->data; t->b = bv->data; t->m = m; t->F = F; t->nf = tl_nf;
  memcpy(t->f, tl_f, sizeof(float) * 3 * tl_nf);
  t->scale = tl_scale;
  *out = t;
  return XF_OK;
}

static int fcg_mixed_two_level(xf_op* op, xf_unet* u, const xf_solve_opts& o, int m, int F, const float (*tl_f)[3],
                               int tl_nf, double tl_scale, xf_vec* xv, const xf_vec* bv, xf_solve_stats* st) {
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  cudaStream_t s = ctx->stream;
  TlGraph* t = u->tlg;
  const bool same = t && t->op_serial == op->serial && t->x == xv->data && t->b == bv->data && t->m == m &&
                    t->F == F && t->nf == tl_nf && t->scale == tl_scale &&
                    memcmp(t->f, tl_f, sizeof(float) * 3 * tl_nf) == 0;
  if (!same) {
    if (t) {
      cudaStreamSynchronize(s);
      delete t;
      u->tlg = nullptr;
    }
    int rc = tl_graph_build(op, u, m, F, tl_f, tl_nf, tl_scale, xv, bv, &u->tlg);
    if (rc) return rc;
    t = u->tlg;
  }
  // the Chebyshev passes return at once while a mixed solve's done / pause flags are set
  long long zero = 0;
  XF_CUDA(ctx, cudaMemcpyAsync(&ctx->scratch->iscalars[I_DONE], &zero, 8, cudaMemcpyHostToDevice, s));
  XF_CUDA(ctx, cudaMemcpyAsync(&ctx->scratch->iscalars[I_PAUSE], &zero, 8, cudaMemcpyHostToDevice, s));
  XF_CUDA(ctx, cudaMemcpyAsync(&ctx->scratch->iscalars[I_ERR], &zero, 8, cudaMemcpyHostToDevice, s));
  struct { double rtol2; int maxit, every; } p3 = {o.rtol * o.rtol, o.maxit, o.replace_every > 0 ? o.replace_every : 50};
  static_assert(offsetof(TlParams, rtol2) == 0 && offsetof(TlParams, maxit) == 8 && offsetof(TlParams, every) == 12,
                "TlParams layout");
  XF_CUDA(ctx, cudaMemcpyAsync(t->prm, &p3, 16, cudaMemcpyHostToDevice, s));
  XF_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  XF_CUDA(ctx, cudaGraphLaunch(t->exec, s));
  XF_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
  TlCtl hc;
  XF_CUDA(ctx, cudaMemcpyAsync(&hc, t->ctl, sizeof(hc), cudaMemcpyDeviceToHost, s));
  XF_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  int rcode;
  if ((rcode = xf_conv_status(ctx))) return rcode;
  long long err = 0;   // a bounded wait of a Chebyshev pass that gave up
  XF_CUDA(ctx, cudaMemcpy(&err, &ctx->scratch->iscalars[I_ERR], 8, cudaMemcpyDeviceToHost));
  if (err) return xf_fail(ctx, XF_ERR_CUDA, "xf_solve_fcg: a smoothing pass timed out on a copy");
  if (hc.status == XF_ERR_CUDA) return xf_fail(ctx, XF_ERR_CUDA, "xf_solve_fcg: the device loop stopped without progress");
  const double rel = hc.bb > 0 ? sqrt(hc.rr_true / hc.bb) : sqrt(hc.rr_true);
  st->status = hc.status == XF_OK && rel > o.rtol ? XF_STALL : hc.status;
  st->iterations = hc.it;
  st->replacements = hc.repl;
  st->fallbacks = hc.fallbacks;
  st->reserved[0] = (double)hc.launches;
  st->rel_resid = rel;
  st->abs_resid = sqrt(hc.rr_true);
  st->ms = ms;
  return XF_OK;
}

extern "C" int xf_solve_fcg(xf_op* op, xf_unet* u, const xf_solve_opts* opts, xf_vec* xv, const xf_vec* bv,
                            xf_solve_stats* st) {
  if (!op || !xv || !bv || !st) return XF_ERR_ARG;
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  if (xv->g != g || bv->g != g || xv->dtype != XF_F64 || bv->dtype != XF_F64)
    return xf_fail(ctx, XF_ERR_STATE, "xf_solve_fcg: x and b must be FP64 boxes of the operator's grid");
  xf_solve_opts o;
  if (opts) o = *opts;
  else xf_solve_opts_default(&o);
  if (o.maxit <= 0) o.maxit = 100000;
  if (o.rtol <= 0) o.rtol = 1e-8;
  const int m = o.reserved[0] > 0 ? (o.reserved[0] > 8 ? 8 : o.reserved[0]) : 8;
  if (o.precond == XF_PRECOND_UNET && (!u || u->g != g))
    return xf_fail(ctx, XF_ERR_ARG, "xf_solve_fcg: XF_PRECOND_UNET needs a network built on the operator's grid");
  // two-level: the network's grid is the coarse grid of F^3 blocks
  const bool two = o.precond == XF_PRECOND_UNET2;
  int F = 0;
  const xf_grid* cg = two && u ? u->g : nullptr;
  if (two) {
    if (!u || u->ctx != ctx)
      return xf_fail(ctx, XF_ERR_ARG, "xf_solve_fcg: XF_PRECOND_UNET2 needs a network on the same context");
    if (cg->n1 > 2) F = (g->n1 - 2) / (cg->n1 - 2);
    if (F < 2 || (g->n1 - 2) != F * (cg->n1 - 2) || (g->n2 - 2) != F * (cg->n2 - 2) || (g->n3 - 2) != F * (cg->n3 - 2))
      return xf_fail(ctx, XF_ERR_ARG,
                     "xf_solve_fcg: XF_PRECOND_UNET2: the network's grid must have interiors of F x F x F blocks of "
                     "the operator's (F >= 2, the same on every axis)");
    if (op->kind != XF_OP_LAPLACE || !xf_cg_poly_supported(g))
      return xf_fail(ctx, XF_ERR_UNSUPPORTED,
                     "xf_solve_fcg: XF_PRECOND_UNET2 smooths with the Chebyshev passes: a uniform Laplace grid without "
                     "boundary rows");
  }
  // smoothing polynomial: degree opts->reserved[2] (even, 2 to 12, default 8) over
  // [lambda_max / ratio, lambda_max], ratio = opts->reserved[1] (default 60)
  const int tl_deg = o.reserved[2] > 0 ? o.reserved[2] : 8;
  const double tl_ratio = o.reserved[1] > 1 ? (double)o.reserved[1] : 60.0;
  const int tl_nf = tl_deg / 2;
  float tl_f[6][3];
  double tl_scale = 0.0;
  if (two) {
    if (tl_deg < 2 || tl_deg > 12 || tl_deg % 2)
      return xf_fail(ctx, XF_ERR_ARG, "xf_solve_fcg: XF_PRECOND_UNET2 degree (opts.reserved[2]) must be even, 2 to 12");
    const double lmax = 4.0 * (g->ucx + g->ucy + g->ucz);   // Gershgorin bound of the uniform Laplace rows
    if (tl_nf == 1) xf_cheb2_coeffs(lmax, tl_ratio, tl_f[0]);
    else if (!xf_cheb_factors(lmax, tl_ratio, tl_deg, tl_f))
      return xf_fail(ctx, XF_ERR_ARG, "xf_solve_fcg: no quadratic factors of the smoothing polynomial");
    tl_scale = cheb_scale(tl_f, tl_nf, lmax, tl_ratio);
  }
  if (o.precond == XF_PRECOND_JACOBI && op->kind != XF_OP_LAPLACE)
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve_fcg: Jacobi uses the Laplace diagonal");
  int rc;
  if ((rc = xf_op_ready(op))) return rc;
  memset(st, 0, sizeof(*st));
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  if (two && o.precision == XF_PREC_MIXED) return fcg_mixed_two_level(op, u, o, m, F, tl_f, tl_nf, tl_scale, xv, bv, st);
  if (o.precision == XF_PREC_MIXED)
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve_fcg: mixed precision is for XF_PRECOND_UNET2");
  const int64_t n = g->ncell;
  std::vector<double*> bufs;
  auto buf = [&]() -> double* {
    double* p = nullptr;
    if (cudaMalloc(&p, n * 8) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    cudaMemsetAsync(p, 0, n * 8, ctx->stream);
    bufs.push_back(p);
    return p;
  };
  auto cleanup = [&]() {
    for (double* p : bufs) cudaFree(p);
  };
  double *r = buf(), *z = buf(), *pn = buf(), *qn = buf();
  double *P[8] = {nullptr}, *Q[8] = {nullptr};
  bool okb = r && z && pn && qn;
  for (int j = 0; j < m && okb; j++) okb = (P[j] = buf()) && (Q[j] = buf());
  // two-level: y, A y (fine FP64), the smoother's FP32 ping-pong pair, the coarse r and z
  double *ty = nullptr, *tqy = nullptr, *trc = nullptr, *tzc = nullptr;
  float *t32a = nullptr, *t32b = nullptr;
  if (two && okb) {
    okb = (ty = buf()) && (tqy = buf());
    for (int h = 0; h < 2 && okb; h++) {
      float* p = nullptr;
      okb = cudaMalloc(&p, n * 4) == cudaSuccess;
      if (!okb) cudaGetLastError();
      else bufs.push_back((double*)p);   // freed with the rest
      (h ? t32b : t32a) = p;
    }
    if (okb) {
      const int64_t nc = cg->ncell;
      for (int h = 0; h < 2 && okb; h++) {
        double* p = nullptr;
        okb = cudaMalloc(&p, nc * 8) == cudaSuccess;
        if (!okb) cudaGetLastError();
        else bufs.push_back(p);
        (h ? tzc : trc) = p;
      }
    }
    if (okb) {   // the Chebyshev passes return at once while a mixed solve's done / pause flags are set
      long long zero3[3] = {0, 0, 0};
      okb = cudaMemcpyAsync(&ctx->scratch->iscalars[I_DONE], zero3, 8, cudaMemcpyHostToDevice, ctx->stream) ==
                cudaSuccess &&
            cudaMemcpyAsync(&ctx->scratch->iscalars[I_PAUSE], zero3, 8, cudaMemcpyHostToDevice, ctx->stream) ==
                cudaSuccess &&
            cudaMemcpyAsync(&ctx->scratch->iscalars[I_ERR], zero3, 8, cudaMemcpyHostToDevice, ctx->stream) ==
                cudaSuccess &&
            cudaStreamSynchronize(ctx->stream) == cudaSuccess;
    }
  }
  if (!okb) {
    cleanup();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve_fcg: allocation");
  }
  double pq_win[8] = {0};
  cudaStream_t s = ctx->stream;
  const int eb = grid_blocks(ctx, n, 256);
  double* x = (double*)xv->data;
  const double* b = (const double*)bv->data;
  int precond = o.precond;
  auto fail = [&](int code, const char* msg) {
    cleanup();
    return xf_fail(ctx, code, "xf_solve_fcg: %s", msg);
  };
  auto apply_m = [&]() -> int {   // z = M r
    if (precond == XF_PRECOND_UNET) return xf_unet_apply_dev(u, r, z);
    if (precond == XF_PRECOND_UNET2) {
      k_restrict_blocks<double><<<grid_blocks(ctx, cg->ncell, 256), 256, 0, s>>>(r, g->n2, g->n3, F, trc, cg->n1,
                                                                                cg->n2, cg->n3);
      int st2 = xf_unet_apply_dev(u, trc, tzc);
      if (st2) return st2;
      k_prolong_blocks<double><<<eb, 256, 0, s>>>(tzc, cg->n2, cg->n3, F, g->smask, g->n1, g->n2, g->n3, ty);
      MvReq<double> my;   // A y, (y, A y)
      my.x = ty; my.y = tqy; my.w = ty; my.zero_inactive = 1; my.slot = FS_YAY;
      xf_mv64(op, my);
      xf_dot_async(g, XF_F64, ty, r, FS_YR);
      double v[2];
      if ((st2 = read_n(ctx, FS_YAY, 2, v))) return st2;
      const double om = (v[0] > 0 && std::isfinite(v[0]) && std::isfinite(v[1])) ? v[1] / v[0] : 0.0;
      k_sub_f32<double><<<eb, 256, 0, s>>>(r, tqy, om, n, t32a);   // r - omega A y, FP32
      float *src = t32a, *dst = t32b;
      for (int k = tl_nf - 1; k >= 0; k--) {
        xf_cg_poly_first_launch(op, src, dst, tl_f[k], nullptr, nullptr, nullptr, nullptr, nullptr);
        std::swap(src, dst);
      }
      k_twolevel_z<double><<<eb, 256, 0, s>>>(ty, src, om, tl_scale, g->smask, n, z);
      return cudaGetLastError() == cudaSuccess ? XF_OK : XF_ERR_CUDA;
    }
    if (precond == XF_PRECOND_JACOBI) {
      k_jacobi<<<eb, 256, 0, s>>>(r, g->diag, g->kind, n, z);
      return XF_OK;
    }
    return cudaMemcpyAsync(z, r, n * 8, cudaMemcpyDeviceToDevice, s) == cudaSuccess ? XF_OK : XF_ERR_CUDA;
  };
  XF_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  {
    MvReq<double> mv;   // r = b - A x (zero off the active set)
    mv.x = x; mv.y = r; mv.s = b; mv.sign = -1; mv.neg = 1; mv.zero_inactive = 1;
    xf_mv64(op, mv);
  }
  xf_dot_async(g, XF_F64, b, b, FS_RR);
  double bb;
  if ((rc = read_n(ctx, FS_RR, 1, &bb))) return fail(rc, "scalar read");
  const double thr = o.rtol * o.rtol * bb;
  xf_dot_async(g, XF_F64, r, r, FS_RR);
  double rr;
  if ((rc = read_n(ctx, FS_RR, 1, &rr))) return fail(rc, "scalar read");
  int it = 0, nwin = 0, head = 0, status = XF_OK;
  double rr_mark = rr;
  int mark_it = 0;
  while (rr > thr) {
    if (it >= o.maxit) { status = XF_MAXIT; break; }
    if (std::isnan(rr)) { status = XF_NAN; break; }
    it++;
    if ((rc = apply_m())) return fail(rc, "preconditioner");
    xf_dot_async(g, XF_F64, z, r, FS_ZR);
    double zr;
    if ((rc = read_n(ctx, FS_ZR, 1, &zr))) return fail(rc, "scalar read");
    if (!(zr > 0) && precond != XF_PRECOND_NONE) {   // no descent direction: use r this time
      if (++st->fallbacks >= FCG_STRIKES) precond = XF_PRECOND_NONE;   // and from the third on, for good
      XF_CUDA(ctx, cudaMemcpyAsync(z, r, n * 8, cudaMemcpyDeviceToDevice, s));
    }
    // p = z - sum_j (z, A p_j) / (p_j, A p_j) p_j over the window
    XF_CUDA(ctx, cudaMemcpyAsync(pn, z, n * 8, cudaMemcpyDeviceToDevice, s));
    if (nwin > 0) {
      for (int j = 0; j < nwin; j++) xf_dot_async(g, XF_F64, z, Q[j], j);
      double zq[8];
      if ((rc = read_n(ctx, 0, nwin, zq))) return fail(rc, "scalar read");
      for (int j = 0; j < nwin; j++)
        if (pq_win[j] > 0) k_axpy_d<<<eb, 256, 0, s>>>(pn, P[j], -zq[j] / pq_win[j], n);
    }
    MvReq<double> mv;   // q = A p, (p, q)
    mv.x = pn; mv.y = qn; mv.w = pn; mv.zero_inactive = 1; mv.slot = FS_PQ;
    xf_mv64(op, mv);
    xf_dot_async(g, XF_F64, pn, r, FS_PR);
    double pq, pr;
    if ((rc = read_n(ctx, FS_PQ, 1, &pq)) || (rc = read_n(ctx, FS_PR, 1, &pr))) return fail(rc, "scalar read");
    if (!(pq > 0)) { status = std::isnan(pq) ? XF_NAN : XF_BREAKDOWN; break; }
    const double alpha = pr / pq;
    k_fcg_update<<<eb, 256, 0, s>>>(x, r, pn, qn, alpha, n);
    // the new direction joins the window (ring of m)
    XF_CUDA(ctx, cudaMemcpyAsync(P[head], pn, n * 8, cudaMemcpyDeviceToDevice, s));
    XF_CUDA(ctx, cudaMemcpyAsync(Q[head], qn, n * 8, cudaMemcpyDeviceToDevice, s));
    pq_win[head] = pq;
    head = (head + 1) % m;
    if (nwin < m) nwin++;
    xf_dot_async(g, XF_F64, r, r, FS_RR);
    if ((rc = read_n(ctx, FS_RR, 1, &rr))) return fail(rc, "scalar read");
    if (it - mark_it >= 50) {   // stall watch
      if (precond != XF_PRECOND_NONE && !(rr < 0.81 * rr_mark)) {
        precond = XF_PRECOND_NONE;
        st->fallbacks++;
      }
      rr_mark = rr;
      mark_it = it;
    }
  }
  {
    MvReq<double> mv;   // true residual
    mv.x = x; mv.y = qn; mv.s = b; mv.sign = -1; mv.neg = 1; mv.zero_inactive = 1; mv.dot_self = 1; mv.slot = FS_PQ;
    xf_mv64(op, mv);
  }
  double tr[2];
  if ((rc = read_n(ctx, FS_PQ, 2, tr))) return fail(rc, "scalar read");
  XF_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
  XF_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  cleanup();
  if ((o.precond == XF_PRECOND_UNET || two) && (rc = xf_conv_status(ctx))) return rc;
  if (two) {   // a bounded wait of a Chebyshev pass that gave up
    long long err = 0;
    XF_CUDA(ctx, cudaMemcpy(&err, &ctx->scratch->iscalars[I_ERR], 8, cudaMemcpyDeviceToHost));
    if (err) return xf_fail(ctx, XF_ERR_CUDA, "xf_solve_fcg: a smoothing pass timed out on a copy");
  }
  const double rel = bb > 0 ? sqrt(tr[1] / bb) : sqrt(tr[1]);
  st->status = status == XF_OK && rel > o.rtol ? XF_STALL : status;
  st->iterations = it;
  st->rel_resid = rel;
  st->abs_resid = sqrt(tr[1]);
  st->ms = ms;
  return XF_OK;
}
