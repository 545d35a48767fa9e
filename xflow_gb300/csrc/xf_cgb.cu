// K1 of the mixed CG iteration with bulk-staged planes:
//
//   p' = r + beta p,   q = A p',   (p', q) -> alpha,   flip the p buffers
//
// on uniform Laplace grids (the CG path's "pq fused" step).  A block owns a
// tile of PQB_TILE consecutive cells of the flattened (j, k) plane and walks a
// chunk of i-planes.  For every plane, one bulk asynchronous copy
// (cp.async.bulk, the TMA engine's 1-D form) per field brings the raw r and p
// of the tile plus a halo of HA >= n3 + 1 cells on either side into a
// PQB_NS-deep shared-memory ring, completed on mbarriers.  The copies of a
// block's whole run of items form one stream, so the first planes of the next
// item load while the current item finishes.
//
// Per plane i the block turns the raw plane i+1, as soon as it has landed,
// into p'(i+1) over the whole region in a three-plane p' ring (and writes the
// own cells' p' to global memory), releases the raw slot, synchronises once,
// and computes q for its own cells of plane i: i+-1 and j+-1 from the p'
// ring (i-1 from registers), k+-1 from the neighbouring lanes.  Each thread owns two groups of
// four cells, at 4 t and at PQB_TILE / 2 + 4 t, so that consecutive lanes
// touch consecutive 16-byte words of shared memory.  The dot (p', q) keeps
// each product's rounding error (an FMA) and sums a thread's products and
// errors per plane in FP32 before the float-float accumulation.
//
// Every mbarrier wait is bounded.  A wait that runs out records I_ERR, lets
// every copy still in flight land (bounded), ends the solve with XF_ERR_CUDA
// and leaves without publishing.
#include <stdint.h>
#include <stdlib.h>

#include "xf_bulk.cuh"
#include "xf_control.cuh"
#include "xf_stencil.cuh"

namespace {

constexpr int PQB_THREADS = 256;
constexpr int PQB_TILE = 8 * PQB_THREADS;   // 2048 plane cells per tile
constexpr int PQB_HALF = PQB_TILE / 2;
constexpr int PQB_NP = 3;                   // p' plane ring: i-1, i, i+1

struct PqbArgs {
  const uint8_t* kind;
  const float* r;
  float* pb0;
  float* pb1;
  float* q;
  DevScratch* S;
  int n1, n3, P;
  int HA, RL;                 // halo width (multiple of 4, >= n3 + 1), region length TILE + 2 HA
  int tiles, chunk, nchunk;   // work items: nchunk plane chunks x tiles
  float cx, cy, cz;
  int ctl;                    // control step of the last block
};

__device__ __forceinline__ float4 fma4(float b, float4 p, float4 r) {
  return make_float4(fmaf(b, p.x, r.x), fmaf(b, p.y, r.y), fmaf(b, p.z, r.z), fmaf(b, p.w, r.w));
}
__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

template <int PQB_NS>   // raw ring depth (planes in flight)
__global__ void __launch_bounds__(PQB_THREADS, PQB_NS == 1 ? 4 : PQB_NS == 2 ? 3 : 2) k_cg_pqb(const __grid_constant__ PqbArgs a) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  float* ring = reinterpret_cast<float*>(smem + 128);          // PQB_NS x {r, p} x RL
  float* pring = ring + (size_t)PQB_NS * 2 * a.RL;             // PQB_NP x RL
  const float beta = (float)S->scalars[D_BETA];
  const int sel = (int)S->iscalars[I_PBUF];
  const float* __restrict__ po = sel ? a.pb1 : a.pb0;
  float* __restrict__ pn = sel ? a.pb0 : a.pb1;
  const float* __restrict__ r = a.r;
  const int n1 = a.n1, n3 = a.n3, P = a.P, HA = a.HA, RL = a.RL;
  const int64_t total = (int64_t)n1 * P;
  const int items = a.nchunk * a.tiles;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = a.cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + a.cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              a.cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < PQB_NS; s++) mbar_init(&mbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  // The load stream: for each of this block's items, planes lo..hi (the
  // chunk's planes and one on either side, inside the box), upwards for even
  // chunks and downwards for odd ones, so that the two blocks sharing a chunk
  // boundary read its planes at about the same time (the second read hits L2).
  auto item_range = [&](int item, int& base, int& i0, int& i1, int& lo, int& hi, int& dir) {
    const int ic = item / a.tiles;
    base = (item - ic * a.tiles) * PQB_TILE;
    i0 = ic * a.chunk;
    i1 = min(n1, i0 + a.chunk);
    lo = max(i0 - 1, 0);
    hi = min(i1, n1 - 1);
    dir = (ic & 1) ? -1 : 1;
  };
  // producer state (thread 0 only)
  int p_item = blockIdx.x, p_plane = 0, p_base = 0, p_end = 0, p_dir = 1;
  long long issued = 0;
  auto p_start_item = [&]() {
    if (p_item < items) {
      int i0, i1, lo, hi;
      item_range(p_item, p_base, i0, i1, lo, hi, p_dir);
      p_plane = p_dir > 0 ? lo : hi;
      p_end = p_dir > 0 ? hi : lo;
    }
  };
  auto issue_one = [&]() -> bool {
    if (p_item >= items) return false;
    const int s = (int)(issued % PQB_NS);
    const int64_t reg_lo = (int64_t)p_plane * P + p_base - HA, reg_hi = reg_lo + RL;
    const int64_t c_lo = reg_lo < 0 ? 0 : reg_lo, c_hi = reg_hi > total ? total : reg_hi;
    const uint32_t bytes = (uint32_t)(c_hi - c_lo) * 4u;
    float* dst = ring + (size_t)s * 2 * RL + (c_lo - reg_lo);
    mbar_expect_tx(&mbar[s], 2u * bytes);
    bulk_g2s(dst, r + c_lo, bytes, &mbar[s]);
    bulk_g2s(dst + RL, po + c_lo, bytes, &mbar[s]);
    issued++;
    if (p_plane == p_end) {
      p_item += gridDim.x;
      p_start_item();
    } else {
      p_plane += p_dir;
    }
    return true;
  };
  if (threadIdx.x == 0) {
    p_start_item();
    for (int s = 0; s < PQB_NS; s++)
      if (!issue_one()) break;
  }
  long long released = 0;   // loads whose slot is free again (all threads agree)
  auto release = [&]() {
    released++;
    if (threadIdx.x == 0) {
      fence_proxy_async();
      while (issued < released + PQB_NS && issue_one()) {
      }
    }
  };

  DotAcc<float> acc;
  bool ok = true;
  long long waited = 0;       // loads thread 0 has seen land
  long long item_first = 0;   // stream index of the current item's first plane
  for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
    int base, i0, i1, lo, hi, dir;
    item_range(item, base, i0, i1, lo, hi, dir);
    const int xa = base + 4 * threadIdx.x, xb = xa + PQB_HALF;   // this thread's two groups
    const bool va = xa < P, vb = xb < P;                         // P % 4 == 0: whole groups
    const int sa = HA + 4 * threadIdx.x, sb = sa + PQB_HALF;     // their region index
    uchar4 ka = make_uchar4(0, 0, 0, 0), kb = ka;   // row kinds of the first plane computed
    const int kfirst = dir > 0 ? i0 : i1 - 1;
    if (va) ka = *reinterpret_cast<const uchar4*>(a.kind + (int64_t)kfirst * P + xa);
    if (vb) kb = *reinterpret_cast<const uchar4*>(a.kind + (int64_t)kfirst * P + xb);
    bool wok = true;
    // own p'(i-1) in registers: the ring slot of plane i-1 is rewritten during
    // step i+1, possibly while a slower warp is still in step i
    float4 xma = make_float4(0.f, 0.f, 0.f, 0.f), xmb = xma;
    // step i: p'(j) of the region into the p' ring, j = i + dir the next
    // plane in march order, then q of plane i
    const int first = dir > 0 ? i0 - 2 : i1 + 1, stop = dir > 0 ? i1 : i0 - 1;
    for (int i = first; i != stop; i += dir) {
      const int j = i + dir;
      const bool load = j >= lo && j <= hi;
      if (load) {
        const long long L = item_first + (dir > 0 ? j - lo : hi - j);
        wok = mbar_wait_bounded(&mbar[L % PQB_NS], (uint32_t)((L / PQB_NS) & 1));
        if (wok) {
          waited = L + 1;
          const float* R = ring + (size_t)(L % PQB_NS) * 2 * RL;
          const float* Q = R + RL;
          float* pj = pring + (size_t)((j + PQB_NP) % PQB_NP) * RL;
          const float4 ga = fma4(beta, lds4(Q + sa), lds4(R + sa));
          const float4 gb = fma4(beta, lds4(Q + sb), lds4(R + sb));
          *reinterpret_cast<float4*>(pj + sa) = ga;
          *reinterpret_cast<float4*>(pj + sb) = gb;
          for (int h = threadIdx.x; h < HA / 2; h += PQB_THREADS) {   // halo groups (HA % 4 == 0), either side
            const int t = 4 * (h < HA / 4 ? h : h + PQB_TILE / 4);
            *reinterpret_cast<float4*>(pj + t) = fma4(beta, lds4(Q + t), lds4(R + t));
          }
          if (j >= i0 && j < i1) {   // p' of the chunk's own cells, written once
            const int64_t pl = (int64_t)j * P;
            if (va) *reinterpret_cast<float4*>(pn + pl + xa) = ga;
            if (vb) *reinterpret_cast<float4*>(pn + pl + xb) = gb;
          }
        }
      }
      // next plane's row kinds, in flight during this plane
      uchar4 kna = ka, knb = kb;
      if (i >= i0 && i < i1 && j >= i0 && j < i1) {
        if (va) kna = *reinterpret_cast<const uchar4*>(a.kind + (int64_t)j * P + xa);
        if (vb) knb = *reinterpret_cast<const uchar4*>(a.kind + (int64_t)j * P + xb);
      }
      if (__syncthreads_or(!wok)) { ok = false; break; }
      if (load) release();   // plane j's slot is consumed
      if (i == (dir > 0 ? i0 - 1 : i1) && i >= 0 && i < n1) {   // the plane before the chunk, written last step
        const float* pc = pring + (size_t)((i + PQB_NP) % PQB_NP) * RL;
        xma = lds4(pc + sa);
        xmb = lds4(pc + sb);
      }
      if (i >= i0 && i < i1) {
        const float* pc = pring + (size_t)((i + PQB_NP) % PQB_NP) * RL;
        const float* pp = pring + (size_t)((j + PQB_NP) % PQB_NP) * RL;
        const float4 xca = lds4(pc + sa), xcb = lds4(pc + sb);
        // k-1 / k+1 of the group ends from the neighbouring lanes (lane 0 / 31 from shared memory)
        const float la = __shfl_up_sync(0xffffffffu, xca.w, 1), lb = __shfl_up_sync(0xffffffffu, xcb.w, 1);
        const float ra = __shfl_down_sync(0xffffffffu, xca.x, 1), rb = __shfl_down_sync(0xffffffffu, xcb.x, 1);
        const int64_t pl = (int64_t)i * P;
        float psum = 0.f, esum = 0.f;   // this thread's (p', q) over the plane: FP32 sum + exact-product errors
        auto group = [&](bool v, int s0, float4 xc, float4 xm, uchar4 k4, float left, float right, int x) {
          if (!v) return;
          const float4 xp = lds4(pp + s0);
          const float km0 = lane == 0 ? pc[s0 - 1] : left;
          const float kp3 = lane == 31 ? pc[s0 + 4] : right;
          const float2 jm01 = *reinterpret_cast<const float2*>(pc + s0 - n3);
          const float2 jm23 = *reinterpret_cast<const float2*>(pc + s0 - n3 + 2);
          const float2 jp01 = *reinterpret_cast<const float2*>(pc + s0 + n3);
          const float2 jp23 = *reinterpret_cast<const float2*>(pc + s0 + n3 + 2);
          const float c[4] = {xc.x, xc.y, xc.z, xc.w};
          const float m[4] = {xm.x, xm.y, xm.z, xm.w};
          const float pq[4] = {xp.x, xp.y, xp.z, xp.w};
          const float jm[4] = {jm01.x, jm01.y, jm23.x, jm23.y};
          const float jp[4] = {jp01.x, jp01.y, jp23.x, jp23.y};
          const float km[4] = {km0, c[0], c[1], c[2]};
          const float kp[4] = {c[1], c[2], c[3], kp3};
          const uint8_t kk[4] = {k4.x, k4.y, k4.z, k4.w};
          float out[4];
#pragma unroll
          for (int v2 = 0; v2 < 4; v2++) {
            float o = fmaf(dtab[kk[v2] & 63], c[v2],
                           -fmaf(a.cx, pq[v2] + m[v2], fmaf(a.cy, jp[v2] + jm[v2], a.cz * (kp[v2] + km[v2]))));
            if ((kk[v2] >> K_ROW_SHIFT) == ROW_NONE) o = 0.f;
            out[v2] = o;
            const float pr = c[v2] * o;
            esum += fmaf(c[v2], o, -pr);
            psum += pr;
          }
          *reinterpret_cast<float4*>(a.q + pl + x) = make_float4(out[0], out[1], out[2], out[3]);
        };
        group(va, sa, xca, xma, ka, la, ra, xa);
        group(vb, sb, xcb, xmb, kb, lb, rb, xb);
        acc.add(psum, 1.f);
        acc.add(esum, 1.f);
        xma = xca;
        xmb = xcb;
      }
      ka = kna; kb = knb;
    }
    if (!ok) break;
    item_first += hi - lo + 1;
    __syncthreads();   // the next item rewrites the p' ring
  }
  if (!ok) {
    // A copy did not land in time: record it, let every copy still in flight
    // land (bounded) so none writes into released shared memory, and leave.
    if (threadIdx.x == 0) {
      atomicExch((unsigned long long*)&S->iscalars[I_ERR], 1ull);
      for (long long L = waited; L < issued; L++) mbar_wait_bounded(&mbar[L % PQB_NS], (uint32_t)((L / PQB_NS) & 1));
      S->iscalars[I_DONE] = 1;
      S->iscalars[I_STATUS] = XF_ERR_CUDA;
    }
    __syncthreads();
    return;
  }
  if (!publish_acc<float>(S, SL_A, SL_A, acc, sh, &last)) return;
  double tot = finish_partials(S, SL_A, sh);
  if (threadIdx.x == 0) {
    S->scalars[SL_A] = tot;
    S->tickets[SL_A] = 0;
    control_step(S, a.ctl);
  }
}

size_t pqb_smem(int RL, int ns) { return 128 + (size_t)(ns * 2 + PQB_NP) * RL * sizeof(float); }

}  // namespace

// The bulk-staged kernel needs P % 4 == 0 (16-byte groups and copy bounds) and
// n3 even (8-byte aligned j+-1 reads), and its ring must fit in shared memory.
bool xf_cg_pqb_supported(const xf_grid* g) {
  const int64_t P = (int64_t)g->n2 * g->n3;
  if (P % 4 != 0 || g->n3 % 2 != 0 || g->n3 < 2 || g->n2 < 2 || P > (1 << 30)) return false;
  const int HA = (g->n3 + 1 + 3) & ~3;
  return pqb_smem(PQB_TILE + 2 * HA, 2) <= 227 * 1024 - 1024;
}

void xf_cg_pqb_launch(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int ctl) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  PqbArgs a;
  a.kind = g->kind;
  a.r = r; a.pb0 = pb0; a.pb1 = pb1; a.q = q; a.S = ctx->scratch;
  a.n1 = g->n1; a.n3 = g->n3; a.P = g->n2 * g->n3;
  a.HA = (g->n3 + 1 + 3) & ~3;
  a.RL = PQB_TILE + 2 * a.HA;
  a.tiles = (a.P + PQB_TILE - 1) / PQB_TILE;
  a.cx = (float)g->ucx; a.cy = (float)g->ucy; a.cz = (float)g->ucz;
  a.ctl = ctl;
  // ring depth 2 (3 blocks per SM)
  const int ns = 2;
  const size_t smem = pqb_smem(a.RL, ns);
  static size_t attr_smem[5][64] = {};   // per ring depth and device
  size_t& at = attr_smem[ns][ctx->device & 63];
  if (at < smem) {
    cudaFuncSetAttribute(k_cg_pqb<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    at = smem;
  }
  // resident blocks per SM from shared memory (1 KB reserved per block) and the launch bounds
  int resident = (int)((228 * 1024) / (smem + 1024 + 1024));
  if (resident > 3) resident = 3;
  if (resident < 1) resident = 1;
  const int64_t B = (int64_t)ctx->sm_count * resident;
  // plane chunk: the length whose last wave wastes least (cost ~ waves x (chunk + 1))
  int best = 8;
  double best_cost = 1e30;
  for (int L = 4; L <= 48; L++) {
    const int64_t items = (int64_t)a.tiles * ((g->n1 + L - 1) / L);
    const double cost = (double)((items + B - 1) / B) * (L + 1);
    if (cost < best_cost) { best_cost = cost; best = L; }
  }
  a.chunk = best;
  a.nchunk = (g->n1 + a.chunk - 1) / a.chunk;
  int64_t blocks = B, items = (int64_t)a.tiles * a.nchunk;
  if (blocks > items) blocks = items;
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  // XF_PQB_BLOCKS caps the grid (several items per block: the cross-item load stream)
  if (const char* env = getenv("XF_PQB_BLOCKS")) {
    const long cap = strtol(env, nullptr, 10);
    if (cap >= 1 && cap < blocks) blocks = cap;
  }
  k_cg_pqb<2><<<(int)blocks, PQB_THREADS, smem, ctx->stream>>>(a);
}
