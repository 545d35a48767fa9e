// K0 of the polynomially preconditioned mixed CG:
//
//   z = p(A) r,   (r, z) -> beta
//
// on uniform Laplace grids, p the degree-2 polynomial of two steps of the
// Chebyshev iteration for A z = r over [lambda_max / ratio, lambda_max]
// (positive on the spectrum, so p(A) is symmetric positive definite), in
// Horner form
//
//   y1 = a1 r + a2 (A r),   z = a0 r + A y1,
//
// both stencil levels in one pass over memory.  A block owns a tile of
// CP_TILE consecutive cells of the flattened (j, k) plane and marches a chunk
// of i-planes.  The raw r of each plane (tile plus a halo of 2 HA cells,
// HA >= n3 + 1, on either side) arrives by bulk asynchronous copy
// (cp.async.bulk) into a CP_NS-deep ring; at step t the block
//   - computes level 1 for plane t-1 over the tile plus one halo (y1 into a
//     four-plane ring),
//   - computes level 2 for plane t-3 on its own cells (z to global memory,
//     the (r, z) partial),
//   - waits for raw plane t+1 (its row kinds over the level-1 region come
//     with it, by a second bulk copy on the same barrier),
// and synchronises once.  The stencil is the fast Laplace row of the CG
// kernels (open-face diagonal, uniform coefficients); rows without an
// equation give 0, so inactive cells keep z = 0.  Halo cells outside the box
// hold stale values that only rows without an equation read.
//
// The fused form (FUSE) also carries the previous iteration's update: when
// raw plane t+1 lands, the block applies r -= alpha q to it in shared memory
// (q of the same region arrives by bulk copy into a one-plane buffer),
// writes the updated residual of its own cells to the other residual buffer,
// updates the FP32 correction e += alpha p' there and accumulates (r, r).  Halo
// cells are updated redundantly with the same FMA as their owners, so every
// block sees bit-identical values.  One launch then does the work of the
// residual update kernel and of K0, and the iteration needs two kernels.
//
// The learned two-level preconditioner's smoother (xf_unet.cu) uses two more
// forms around its factor passes: the first pass takes its input as
// r - omega q (q = A y of the prolongated coarse correction y, omega from the
// device scalars), applied to each raw plane as it lands and to the own cells
// of level 2; the last pass writes z = omega y + s w of its output w (zero
// off the active set) to two buffers and reduces (z, r) and (z, q_w) with q_w
// the flexible CG's last direction image.  They replace the separate
// subtraction, combination and dot kernels.
//
// Every mbarrier wait is bounded; a wait that runs out records I_ERR, lets the
// copies in flight land (bounded), ends the solve with XF_ERR_CUDA and leaves.
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <array>
#include <complex>
#include <vector>

#include "xf_bulk.cuh"
#include "xf_control.cuh"
#include "xf_stencil.cuh"

namespace {

constexpr int CP_THREADS = 256;
constexpr int CP_TILE = 8 * CP_THREADS;   // 2048 plane cells
constexpr int CP_NS = 4;                  // raw ring: planes t-2, t-1, t and one in flight
constexpr int CP_NY = 4;                  // y1 ring: planes t-4 .. t-1

struct CpArgs {
  const uint8_t* kind;
  const float* r;             // residual (FUSE: before this launch's update)
  float* z;
  DevScratch* S;
  const float* q;             // FUSE: A p' of the iteration
  const float *pa, *pb;       // FUSE: direction buffers (I_PBUF names the current one)
  float* e;                   // FUSE: FP32 correction
  float* rout;                // FUSE: updated residual (own cells)
  const float* dr;            // CP_SECOND / two-level last pass: the residual of the (r, z) dot
  // two-level forms (CP_TL_*): omega = tl_omega(scalars, s_yay, s_yr)
  int s_yay, s_yr;
  const float* ty;            // last pass: the prolongated coarse correction y
  const uint8_t* smask;       // last pass: space mask
  float* z2;                  // last pass: second copy of z
  const float* qw;            // last pass: the last direction image (nullptr: no second dot)
  float tsc;                  // last pass: the smoother's scale s
  int s_zr, s_zq;             // last pass: slots of (z, r) and (z, q_w)
  int n1, n3, P;
  int HA, R0, R1;             // halo unit (multiple of 4), raw region TILE + 4 HA, level-1 region TILE + 2 HA
  int KS;                     // bytes of a row-kind slot: R1 + 32 rounded up to 16
  int tiles, chunk, nchunk;   // work items: nchunk plane chunks x tiles
  float cx, cy, cz;           // uniform Laplace coefficients
  float a0, a1, a2;           // Horner coefficients of p
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// Fast Laplace row (uniform grid) of four consecutive cells whose centres are
// c[0..3]: i-neighbours m, p; j-neighbours at -+n3 from s (shared memory,
// 8-byte aligned); k-neighbours from the neighbouring lanes' groups (the
// caller's consecutive lanes hold consecutive groups), s[-1] / s[4] at the
// warp's ends.
__device__ __forceinline__ void lap4(const float* dtab, uchar4 k4, float4 c, float4 m, float4 p, const float* s, int n3,
                                     float cx, float cy, float cz, float out[4], bool last_group = false) {
  const int lane = threadIdx.x & 31;
  float left = __shfl_up_sync(0xffffffffu, c.w, 1), right = __shfl_down_sync(0xffffffffu, c.x, 1);
  if (lane == 0) left = s[-1];
  if (lane == 31 || last_group) right = s[4];   // the next lane holds no following group
  const float2 jm01 = *reinterpret_cast<const float2*>(s - n3), jm23 = *reinterpret_cast<const float2*>(s - n3 + 2);
  const float2 jp01 = *reinterpret_cast<const float2*>(s + n3), jp23 = *reinterpret_cast<const float2*>(s + n3 + 2);
  const float cc[4] = {c.x, c.y, c.z, c.w};
  const float mm[4] = {m.x, m.y, m.z, m.w};
  const float pp[4] = {p.x, p.y, p.z, p.w};
  const float jm[4] = {jm01.x, jm01.y, jm23.x, jm23.y};
  const float jp[4] = {jp01.x, jp01.y, jp23.x, jp23.y};
  const float km[4] = {left, cc[0], cc[1], cc[2]};
  const float kp[4] = {cc[1], cc[2], cc[3], right};
  const uint8_t kk[4] = {k4.x, k4.y, k4.z, k4.w};
#pragma unroll
  for (int v = 0; v < 4; v++) {
    float o = fmaf(dtab[kk[v] & 63], cc[v], -fmaf(cx, pp[v] + mm[v], fmaf(cy, jp[v] + jm[v], cz * (kp[v] + km[v]))));
    if ((kk[v] >> K_ROW_SHIFT) == ROW_NONE) o = 0.f;
    out[v] = o;
  }
}

// Launch modes.  A degree-2 preconditioner is one pass (CP_POLY, or
// CP_POLY_FUSED carrying the residual update); a degree-4 one is the product
// of two quadratic factors, z = p1(A) p2(A) r, in two passes: w = p2(A) r
// (CP_FIRST, or CP_FIRST_FUSED with the update), then z = p1(A) w with the
// (r, z) dot against the residual buffer dr (CP_SECOND).
// CP_TL_FIRST, CP_TL_LAST and CP_TL_BOTH are the two-level forms (see the
// top of this file) of a first, last or only factor pass.
enum { CP_POLY = 0, CP_POLY_FUSED = 1, CP_FIRST = 2, CP_FIRST_FUSED = 3, CP_SECOND = 4, CP_TL_FIRST = 5,
       CP_TL_LAST = 6, CP_TL_BOTH = 7 };

template <int MODE>
__global__ void __launch_bounds__(CP_THREADS, 2) k_cg_poly2(const __grid_constant__ CpArgs a) {
  constexpr bool FUSE = MODE == CP_POLY_FUSED || MODE == CP_FIRST_FUSED;
  constexpr bool IN_SUB = MODE == CP_TL_FIRST || MODE == CP_TL_BOTH;   // input r - omega q
  constexpr bool OUT_TL = MODE == CP_TL_LAST || MODE == CP_TL_BOTH;    // output omega y + s w, two dots
  constexpr bool QBUF = FUSE || IN_SUB;        // q of each raw plane arrives by bulk copy
  constexpr bool DOTZ = MODE == CP_POLY || MODE == CP_POLY_FUSED || MODE == CP_SECOND || OUT_TL;   // (r, z)
  constexpr bool DOTSEP = MODE == CP_SECOND || OUT_TL;   // r of the dot is not the input
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  const int n1 = a.n1, n3 = a.n3, P = a.P, HA = a.HA, R0 = a.R0, R1 = a.R1;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);          // CP_NS raw-plane barriers, then the q barrier
  uint64_t* qbar = mbar + CP_NS;
  float* ring = reinterpret_cast<float*>(smem + 128);          // CP_NS x R0 raw r
  float* yring = ring + (size_t)CP_NS * R0;                     // CP_NY x R1 level-1 planes
  float* qbuf = yring + (size_t)CP_NY * R1;                     // QBUF: R0 cells of q
  uint8_t* kring = reinterpret_cast<uint8_t*>(qbuf + (QBUF ? (size_t)R0 : 0));   // CP_NS x KS row kinds
  const int KS = a.KS;
  const int64_t total = (int64_t)n1 * P;
  const int64_t total16 = (total + 15) & ~(int64_t)15;   // the kind array holds zero bytes up to here
  const int items = a.nchunk * a.tiles;
  float alpha = 0.f;   // FUSE: the update's step; IN_SUB: omega
  const float* pdir = a.pa;
  if (FUSE) {
    alpha = (float)S->scalars[D_ALPHA];
    if (S->iscalars[I_PBUF]) pdir = a.pb;
  }
  float om = 0.f;
  if (IN_SUB || OUT_TL) om = (float)tl_omega(S->scalars, a.s_yay, a.s_yr);
  if (IN_SUB) alpha = om;
  const float* r2src = FUSE ? a.rout : a.r;   // own-cell residual of level 2
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = a.cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + a.cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              a.cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < CP_NS + (QBUF ? 1 : 0); s++) mbar_init(&mbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  auto item_range = [&](int item, int& base, int& i0, int& i1, int& lo, int& hi) {
    const int ic = item / a.tiles;
    base = (item - ic * a.tiles) * CP_TILE;
    i0 = ic * a.chunk;
    i1 = min(n1, i0 + a.chunk);
    lo = max(i0 - 2, 0);
    hi = min(i1 + 1, n1 - 1);
  };
  // the box cells [c_lo, c_hi) of the raw region of a plane, and its start
  auto region = [&](int plane, int base, int64_t& reg_lo, int64_t& c_lo, int64_t& c_hi) {
    reg_lo = (int64_t)plane * P + base - 2 * HA;
    const int64_t reg_hi = reg_lo + R0;
    c_lo = reg_lo < 0 ? 0 : reg_lo;
    c_hi = reg_hi > total ? total : reg_hi;
  };
  // producer (thread 0): the stream of raw planes over this block's items
  int p_item = blockIdx.x, p_plane = 0, p_base = 0, p_hi = -1;
  long long issued = 0;
  auto p_start_item = [&]() {
    if (p_item < items) {
      int i0, i1, lo;
      item_range(p_item, p_base, i0, i1, lo, p_hi);
      p_plane = lo;
    }
  };
  auto issue_one = [&]() -> bool {
    if (p_item >= items) return false;
    const int s = (int)(issued % CP_NS);
    int64_t reg_lo, c_lo, c_hi;
    region(p_plane, p_base, reg_lo, c_lo, c_hi);
    const uint32_t bytes = (uint32_t)(c_hi - c_lo) * 4u;
    // row kinds of the level-1 region, widened to 16-byte boundaries
    const int64_t x0 = (int64_t)p_plane * P + p_base - HA;
    const int64_t k_lo = x0 & ~(int64_t)15, k_hi = (x0 + R1 + 15) & ~(int64_t)15;
    const int64_t kc_lo = k_lo < 0 ? 0 : k_lo, kc_hi = k_hi > total16 ? total16 : k_hi;
    const uint32_t kbytes = (uint32_t)(kc_hi - kc_lo);
    mbar_expect_tx(&mbar[s], bytes + kbytes);
    bulk_g2s(ring + (size_t)s * R0 + (c_lo - reg_lo), a.r + c_lo, bytes, &mbar[s]);
    bulk_g2s(kring + (size_t)s * KS + (kc_lo - k_lo), a.kind + kc_lo, kbytes, &mbar[s]);
    issued++;
    if (++p_plane > p_hi) {
      p_item += gridDim.x;
      p_start_item();
    }
    return true;
  };
  if (threadIdx.x == 0) {
    p_start_item();
    for (int s = 0; s < CP_NS; s++)
      if (!issue_one()) break;
  }
  long long released = 0;
  auto release = [&]() {
    released++;
    if (threadIdx.x == 0) {
      fence_proxy_async();
      while (issued < released + CP_NS && issue_one()) {
      }
    }
  };
  // FUSE: q of one raw plane into the one-plane buffer (thread 0; the previous
  // reader of the buffer has passed a block barrier)
  long long q_issued = 0, q_waited = 0;
  auto issue_q = [&](int plane, int base) {
    int64_t reg_lo, c_lo, c_hi;
    region(plane, base, reg_lo, c_lo, c_hi);
    const uint32_t bytes = (uint32_t)(c_hi - c_lo) * 4u;
    fence_proxy_async();
    mbar_expect_tx(qbar, bytes);
    bulk_g2s(qbuf + (c_lo - reg_lo), a.q + c_lo, bytes, qbar);
    q_issued++;
  };

  DotAcc<float> acc, acc_rr;
  bool ok = true;
  long long waited = 0;
  long long item_first = 0;
  for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
    int base, i0, i1, lo, hi;
    item_range(item, base, i0, i1, lo, hi);
    const int l1lo = max(i0 - 1, 0), l1hi = min(i1, n1 - 1);   // planes of level 1
    auto rslot = [&](int pl) {   // raw slot of a loaded plane (any slot for planes not loaded)
      const int q = pl < lo ? lo : pl > hi ? hi : pl;
      return ring + (size_t)((item_first + (q - lo)) % CP_NS) * R0;
    };
    auto yslot = [&](int pl) { return yring + (size_t)(((pl % CP_NY) + CP_NY) % CP_NY) * R1; };
    // own cells of level 2: two groups of four at 4 t and TILE/2 + 4 t
    const int xa = base + 4 * threadIdx.x, xb = xa + CP_TILE / 2;
    const bool va = xa < P, vb = xb < P;
    const int ya = HA + 4 * threadIdx.x, yb = ya + CP_TILE / 2;   // their index in the level-1 region
    // level-2 inputs of the next plane, prefetched one step ahead (FUSE: the
    // updated residual this thread wrote three steps earlier, read through L2)
    float4 rpa = make_float4(0.f, 0.f, 0.f, 0.f), rpb = rpa, dpa = rpa, dpb = rpa;
    float4 qpa = rpa, qpb = rpa, ypa = rpa, ypb = rpa, wpa = rpa, wpb = rpa;   // IN_SUB: q; OUT_TL: y, q_w
    uchar4 kpa = make_uchar4(0, 0, 0, 0), kpb = kpa, mpa = kpa, mpb = kpa;   // OUT_TL: space mask
    auto prefetch2 = [&](int pl) {
      if (pl < i0 || pl >= i1) return;
      const int64_t o = (int64_t)pl * P;
      if (DOTSEP) {
        if (va) dpa = __ldg(reinterpret_cast<const float4*>(a.dr + o + xa));
        if (vb) dpb = __ldg(reinterpret_cast<const float4*>(a.dr + o + xb));
      }
      if (IN_SUB) {
        if (va) qpa = __ldg(reinterpret_cast<const float4*>(a.q + o + xa));
        if (vb) qpb = __ldg(reinterpret_cast<const float4*>(a.q + o + xb));
      }
      if (OUT_TL) {
        if (va) {
          ypa = __ldg(reinterpret_cast<const float4*>(a.ty + o + xa));
          mpa = *reinterpret_cast<const uchar4*>(a.smask + o + xa);
          if (a.qw) wpa = __ldg(reinterpret_cast<const float4*>(a.qw + o + xa));
        }
        if (vb) {
          ypb = __ldg(reinterpret_cast<const float4*>(a.ty + o + xb));
          mpb = *reinterpret_cast<const uchar4*>(a.smask + o + xb);
          if (a.qw) wpb = __ldg(reinterpret_cast<const float4*>(a.qw + o + xb));
        }
      }
      if (FUSE) {
        if (va) rpa = __ldcg(reinterpret_cast<const float4*>(r2src + o + xa));
        if (vb) rpb = __ldcg(reinterpret_cast<const float4*>(r2src + o + xb));
      } else {
        if (va) rpa = __ldg(reinterpret_cast<const float4*>(r2src + o + xa));
        if (vb) rpb = __ldg(reinterpret_cast<const float4*>(r2src + o + xb));
      }
      if (va) kpa = *reinterpret_cast<const uchar4*>(a.kind + o + xa);
      if (vb) kpb = *reinterpret_cast<const uchar4*>(a.kind + o + xb);
    };
    // row kinds of a loaded plane over its level-1 region (stale outside the
    // box, where only rows without an equation read the level-1 values)
    auto kslot = [&](int pl) {
      const int64_t x0 = (int64_t)pl * P + base - HA;
      return kring + (size_t)((item_first + (pl - lo)) % CP_NS) * KS + (int)(x0 & 15);
    };
    // raw plane pl has landed (and, FUSE, its q)
    auto wait_plane = [&](int pl) -> bool {
      const long long L = item_first + (pl - lo);
      bool w = mbar_wait_bounded(&mbar[L % CP_NS], (uint32_t)((L / CP_NS) & 1));
      if (w) waited = L + 1;
      if (QBUF && w) {
        w = mbar_wait_bounded(qbar, (uint32_t)(q_waited & 1));
        if (w) q_waited++;
      }
      return w;
    };
    // FUSE: e and p' of the own cells of the plane the step's update reaches,
    // loaded at the top of the step so that their latency hides under the
    // stencil levels
    const int own_n = min(CP_TILE, P - base);   // own cells of the tile in a plane
    float4 ep[2], pp[2];
    auto prefetch_e = [&](int pl) {
      if (pl < i0 || pl >= i1) return;
      const int64_t o = (int64_t)pl * P + base;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = 4 * (int)threadIdx.x + h * (CP_TILE / 2);
        if (c < own_n) {
          ep[h] = *reinterpret_cast<const float4*>(a.e + o + c);
          pp[h] = __ldg(reinterpret_cast<const float4*>(pdir + o + c));
        }
      }
    };
    // FUSE: r -= alpha q over the box cells of raw plane pl; own cells of own
    // planes also go to rout with e += alpha p' and (r, r)
    auto update = [&](int pl) {
      float* R = rslot(pl);
      const int64_t reg_lo = (int64_t)pl * P + base - 2 * HA;
      const int s_lo = reg_lo < 0 ? (int)(-reg_lo) : 0;                          // box cells: raw [s_lo, s_hi)
      const int s_hi = total - reg_lo < R0 ? (int)(total - reg_lo) : R0;
      const bool own_plane = pl >= i0 && pl < i1;
      float* rown = a.rout + (int64_t)pl * P + base;
      float* eown = a.e + (int64_t)pl * P + base;
      float psum = 0.f, esum = 0.f;   // (r, r) of the own cells: products and their rounding errors
      auto upd = [&](int s) -> float4 {
        float4 rv = ld4(R + s);
        const float4 qv = ld4(qbuf + s);
        rv.x = fmaf(-alpha, qv.x, rv.x);
        rv.y = fmaf(-alpha, qv.y, rv.y);
        rv.z = fmaf(-alpha, qv.z, rv.z);
        rv.w = fmaf(-alpha, qv.w, rv.w);
        *reinterpret_cast<float4*>(R + s) = rv;
        return rv;
      };
#pragma unroll
      for (int h = 0; h < 2; h++) {   // the own-cell groups of level 2's mapping
        const int c = 4 * (int)threadIdx.x + h * (CP_TILE / 2);
        const int s = 2 * HA + c;
        if (s >= s_hi) continue;
        const float4 rv = upd(s);
        if (FUSE && own_plane && c < own_n) {
          *reinterpret_cast<float4*>(rown + c) = rv;
          float4 ev = ep[h];
          const float4 pv = pp[h];
          ev.x = fmaf(alpha, pv.x, ev.x);
          ev.y = fmaf(alpha, pv.y, ev.y);
          ev.z = fmaf(alpha, pv.z, ev.z);
          ev.w = fmaf(alpha, pv.w, ev.w);
          *reinterpret_cast<float4*>(eown + c) = ev;
          const float rr[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const float pr = rr[k] * rr[k];
            esum += fmaf(rr[k], rr[k], -pr);
            psum += pr;
          }
        }
      }
      if (FUSE && own_plane) {
        acc_rr.add(psum, 1.f);
        acc_rr.add(esum, 1.f);
      }
      for (int hg = threadIdx.x; hg < HA; hg += CP_THREADS) {   // halo groups, either side
        const int s = 4 * (hg < HA / 2 ? hg : hg + CP_TILE / 4);
        if (s >= s_lo && s < s_hi) upd(s);
      }
    };
    long long rel_next = lo;   // next plane whose raw slot is released
    // the item's first raw plane
    if (QBUF && threadIdx.x == 0) issue_q(lo, base);
    if (FUSE) prefetch_e(lo);
    bool wok = wait_plane(lo);
    if (QBUF && wok) update(lo);
    if (__syncthreads_or(!wok)) { ok = false; break; }
    for (int t = i0 - 2; t <= i1 + 2; t++) {
      const int pn = t + 1;   // the raw plane that lands during this step
      const bool has_next = pn > lo && pn <= hi;
      if (QBUF && has_next) {
        if (threadIdx.x == 0) issue_q(pn, base);
        if (FUSE) prefetch_e(pn);
      }
      // (B) level 1 for plane t-1: y1 = a1 r + a2 (A r) over the level-1 region
      const int p1 = t - 1;
      if (p1 >= l1lo && p1 <= l1hi) {
        const float* Rc = rslot(p1);
        const float* Rm = rslot(p1 - 1);
        const float* Rp = rslot(p1 + 1);
        const uint8_t* kb = kslot(p1);
        float* Y = yslot(p1);
        // warp-uniform trip count (the shuffles need every lane); groups past
        // the region end compute on in-bounds cells and are not stored
        for (int g0 = 0; g0 < R1 / 4; g0 += CP_THREADS) {
          const int g = g0 + (int)threadIdx.x;
          const int gg = g < R1 / 4 ? g : R1 / 4 - 1;
          const int s = HA + 4 * gg;   // raw index of the group's first cell
          const float4 c = ld4(Rc + s);
          float ar[4];
          lap4(dtab, *reinterpret_cast<const uchar4*>(kb + 4 * gg), c, ld4(Rm + s), ld4(Rp + s), Rc + s, n3, a.cx,
               a.cy, a.cz, ar, g + 1 >= R1 / 4);
          if (g < R1 / 4)
            *reinterpret_cast<float4*>(Y + 4 * g) =
                make_float4(fmaf(a.a2, ar[0], a.a1 * c.x), fmaf(a.a2, ar[1], a.a1 * c.y),
                            fmaf(a.a2, ar[2], a.a1 * c.z), fmaf(a.a2, ar[3], a.a1 * c.w));
        }
      }
      // (C) level 2 for plane t-3: z = a0 r + A y1 on the own cells, (r, z)
      const int p2 = t - 3;
      if (p2 >= i0 && p2 < i1) {
        const float* Yc = yslot(p2);
        const float* Ym = yslot(p2 - 1);
        const float* Yp = yslot(p2 + 1);
        const int64_t o = (int64_t)p2 * P;
        // (r, z) of this thread's cells: FP32 sum of the products plus the sum of
        // their exact rounding errors, into the float-float accumulator per plane
        float psum = 0.f, esum = 0.f, psum2 = 0.f, esum2 = 0.f;
        auto group = [&](bool v, int s, float4 rr, float4 dd, uchar4 k4, int x, float4 qq, float4 yy, uchar4 mm,
                         float4 ww) {
          float ay[4];
          lap4(dtab, k4, ld4(Yc + s), ld4(Ym + s), ld4(Yp + s), Yc + s, n3, a.cx, a.cy, a.cz, ay);
          if (!v) return;
          if (IN_SUB) {   // the pass input r - omega q, as the raw planes got it
            rr.x = fmaf(-om, qq.x, rr.x);
            rr.y = fmaf(-om, qq.y, rr.y);
            rr.z = fmaf(-om, qq.z, rr.z);
            rr.w = fmaf(-om, qq.w, rr.w);
          }
          float zz[4] = {fmaf(a.a0, rr.x, ay[0]), fmaf(a.a0, rr.y, ay[1]), fmaf(a.a0, rr.z, ay[2]),
                         fmaf(a.a0, rr.w, ay[3])};
          if (OUT_TL) {   // z = omega y + s w on the active set, 0 elsewhere
            const float yv[4] = {yy.x, yy.y, yy.z, yy.w};
            const unsigned char mv[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
            for (int q = 0; q < 4; q++) zz[q] = mv[q] ? fmaf(om, yv[q], a.tsc * zz[q]) : 0.f;
            *reinterpret_cast<float4*>(a.z2 + o + x) = make_float4(zz[0], zz[1], zz[2], zz[3]);
          }
          *reinterpret_cast<float4*>(a.z + o + x) = make_float4(zz[0], zz[1], zz[2], zz[3]);
          if (!DOTZ) return;
          if (DOTSEP) rr = dd;
          const float rv[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const float pr = rv[q] * zz[q];
            esum += fmaf(rv[q], zz[q], -pr);
            psum += pr;
          }
          if (OUT_TL) {
            const float wv[4] = {ww.x, ww.y, ww.z, ww.w};
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float pr = wv[q] * zz[q];
              esum2 += fmaf(wv[q], zz[q], -pr);
              psum2 += pr;
            }
          }
        };
        group(va, ya, rpa, dpa, kpa, xa, qpa, ypa, mpa, wpa);
        group(vb, yb, rpb, dpb, kpb, xb, qpb, ypb, mpb, wpb);
        if (DOTZ) {
          acc.add(psum, 1.f);
          acc.add(esum, 1.f);
        }
        if (OUT_TL) {
          acc_rr.add(psum2, 1.f);
          acc_rr.add(esum2, 1.f);
        }
      }
      // (D) level-2 inputs of the next step
      prefetch2(t - 2);
      // (E) raw plane t+1 for the next step's level 1
      if (has_next) {
        wok = wait_plane(pn);
        if (QBUF && wok) update(pn);
      }
      // (F) one barrier per step; a timed-out wait anywhere stops the block
      if (__syncthreads_or(!wok)) { ok = false; break; }
      // (G) raw plane t-2 has had its last reader
      while (rel_next <= t - 2 && rel_next <= hi) { release(); rel_next++; }
    }
    if (!ok) break;
    while (rel_next <= hi) { release(); rel_next++; }
    item_first += hi - lo + 1;
    __syncthreads();   // the next item rewrites the rings
  }
  if (!ok) {
    if (threadIdx.x == 0) {
      atomicExch((unsigned long long*)&S->iscalars[I_ERR], 1ull);
      for (long long L = waited; L < issued; L++) mbar_wait_bounded(&mbar[L % CP_NS], (uint32_t)((L / CP_NS) & 1));
      if (QBUF && q_issued > q_waited) mbar_wait_bounded(qbar, (uint32_t)(q_waited & 1));
      S->iscalars[I_DONE] = 1;
      S->iscalars[I_STATUS] = XF_ERR_CUDA;
    }
    __syncthreads();
    return;
  }
  if (MODE == CP_FIRST || MODE == CP_TL_FIRST) return;   // a later pass reduces
  if (OUT_TL) {   // (z, r) and (z, q_w), one ticket; no control step (the flexible CG reads them)
    const double bzr = block_sum_acc<float>(acc, sh);
    const double bzq = block_sum_acc<float>(acc_rr, sh);
    if (threadIdx.x == 0) {
      S->partials[a.s_zr][lin_block()] = bzr;
      S->partials[a.s_zq][lin_block()] = bzq;
      __threadfence();
      const unsigned int tk = atomicAdd(&S->tickets[a.s_zr], 1u);
      last = (tk == (unsigned)num_blocks() - 1);
    }
    __syncthreads();
    if (!last) return;
    const double zr = finish_partials(S, a.s_zr, sh);
    const double zq = finish_partials(S, a.s_zq, sh);
    if (threadIdx.x == 0) {
      S->scalars[a.s_zr] = zr;
      if (a.qw) S->scalars[a.s_zq] = zq;
      S->tickets[a.s_zr] = 0;
    }
    return;
  }
  if (MODE == CP_FIRST_FUSED) {   // (r, r) of the updated residual: the stop test
    if (!publish_acc<float>(S, SL_B, SL_B, acc_rr, sh, &last)) return;
    double tot = finish_partials(S, SL_B, sh);
    if (threadIdx.x == 0) {
      S->scalars[SL_B] = tot;
      S->tickets[SL_B] = 0;
      control_step(S, CTL_PCG_RR);
    }
    return;
  }
  if (!FUSE) {
    if (!publish_acc<float>(S, SL_D, SL_D, acc, sh, &last)) return;
    double tot = finish_partials(S, SL_D, sh);
    if (threadIdx.x == 0) {
      S->scalars[SL_D] = tot;
      S->tickets[SL_D] = 0;
      control_step(S, CTL_PCG_BETA);
    }
    return;
  }
  // FUSE: (r, r) of the updated residual and (r, z), one ticket
  const double brr = block_sum_acc<float>(acc_rr, sh);
  const double brz = block_sum_acc<float>(acc, sh);
  if (threadIdx.x == 0) {
    S->partials[SL_B][lin_block()] = brr;
    S->partials[SL_D][lin_block()] = brz;
    __threadfence();
    const unsigned int tk = atomicAdd(&S->tickets[SL_D], 1u);
    last = (tk == (unsigned)num_blocks() - 1);
  }
  __syncthreads();
  if (!last) return;
  const double rr = finish_partials(S, SL_B, sh);
  const double rz = finish_partials(S, SL_D, sh);
  if (threadIdx.x == 0) {
    S->scalars[SL_B] = rr;
    S->scalars[SL_D] = rz;
    S->tickets[SL_D] = 0;
    control_step(S, CTL_PCG_RR_BETA);
  }
}

int cp_kslot(int R1) { return (R1 + 32 + 15) & ~15; }

size_t cp_smem(int R0, int R1, bool fuse) {
  return 128 + (size_t)CP_NS * R0 * 4 + (size_t)CP_NY * R1 * 4 + (fuse ? (size_t)R0 * 4 : 0) +
         (size_t)CP_NS * cp_kslot(R1);
}

int cp_halo(int n3) { return (n3 + 1 + 3) & ~3; }

}  // namespace

// Monomial coefficients, in mu = lambda / lmax, of the Chebyshev-iteration
// polynomial after `deg` steps for A z = r over [lmax / ratio, lmax] (the
// iteration z_{k+1} = z_k + d_{k+1}, d_{k+1} = rho_{k+1} rho_k d_k +
// 2 rho_{k+1} / delta (r - A z_k)), scaled so that the constant term is 1 (a
// positive multiple of a preconditioner leaves preconditioned CG unchanged).
static std::vector<double> cheb_mu_coeffs(double ratio, int deg) {
  const double lo = 1.0 / ratio, hi = 1.0;
  const double theta = (hi + lo) / 2, delta = (hi - lo) / 2, sigma = theta / delta;
  double rho = 1 / sigma;
  std::vector<double> d = {1 / theta}, z = d;
  for (int it = 0; it < deg; it++) {
    std::vector<double> res(z.size() + 1, 0.0);
    res[0] = 1.0;
    for (size_t j = 0; j < z.size(); j++) res[j + 1] -= z[j];   // 1 - mu z
    const double rho_new = 1 / (2 * sigma - rho);
    std::vector<double> dn(res.size(), 0.0);
    for (size_t j = 0; j < d.size(); j++) dn[j] += rho_new * rho * d[j];
    for (size_t j = 0; j < res.size(); j++) dn[j] += 2 * rho_new / delta * res[j];
    d = dn;
    z.resize(d.size(), 0.0);
    for (size_t j = 0; j < d.size(); j++) z[j] += d[j];
    rho = rho_new;
  }
  const double c0 = z[0];
  for (double& c : z) c /= c0;
  return z;
}

// Degree 2: p(A) = out[0] + out[1] A + out[2] A^2.
void xf_cheb2_coeffs(double lmax, double ratio, float out[3]) {
  const std::vector<double> z = cheb_mu_coeffs(ratio, 2);
  for (int j = 0; j < 3; j++) out[j] = (float)(z[j] / pow(lmax, j));
}

// An even degree d = 2 m (4 to 12) as m real quadratic factors
// p(A) = p_1(A) ... p_m(A), each with constant term 1: the roots of p
// (Durand-Kerner iteration in complex double) paired as conjugates, real
// roots with their real neighbours.  f[k] holds factor k+1 as (1, b1, b2) in
// A.  Returns false if the factors do not reproduce p to 1e-9 (relative to
// the largest coefficient).
bool xf_cheb_factors(double lmax, double ratio, int deg, float (*f)[3]) {
  if (deg < 4 || deg > 12 || deg % 2) return false;
  const std::vector<double> c = cheb_mu_coeffs(ratio, deg);
  typedef std::complex<double> cd;
  std::vector<cd> root(deg);
  for (int k = 0; k < deg; k++) root[k] = 2.0 * std::pow(cd(0.4, 0.9), k);
  auto eval = [&](cd x) {
    cd v = c[deg];
    for (int j = deg - 1; j >= 0; j--) v = v * x + c[j];
    return v;
  };
  for (int it = 0; it < 5000; it++) {
    double change = 0;
    for (int k = 0; k < deg; k++) {
      cd den = c[deg];
      for (int m = 0; m < deg; m++)
        if (m != k) den *= root[k] - root[m];
      const cd step = eval(root[k]) / den;
      root[k] -= step;
      change = std::max(change, std::abs(step) / std::max(1.0, std::abs(root[k])));
    }
    if (change < 1e-15) break;
  }
  std::sort(root.begin(), root.end(), [](const cd& x, const cd& y) { return x.real() < y.real(); });
  // pairs: a complex root with the root nearest its conjugate, a real root
  // with the next unused real root (real roots come in an even number)
  auto is_real = [&](int k) { return std::abs(root[k].imag()) <= 1e-12 * std::max(1.0, std::abs(root[k])); };
  std::vector<int> pair;
  std::vector<bool> used(deg, false);
  for (int k = 0; k < deg; k++) {
    if (used[k]) continue;
    int best = -1;
    for (int m = k + 1; m < deg; m++) {
      if (used[m] || is_real(m) != is_real(k)) continue;
      if (best < 0 || std::abs(root[m] - std::conj(root[k])) < std::abs(root[best] - std::conj(root[k]))) best = m;
      if (is_real(k)) break;
    }
    if (best < 0) return false;
    used[k] = used[best] = true;
    pair.push_back(k);
    pair.push_back(best);
  }
  const int nf = deg / 2;
  std::vector<double> prod = {1.0};
  std::vector<std::array<double, 3>> q(nf);
  for (int fi = 0; fi < nf; fi++) {
    const cd ra = root[pair[2 * fi]], rb = root[pair[2 * fi + 1]];
    const cd s1 = 1.0 / ra + 1.0 / rb, s2 = 1.0 / (ra * rb);
    if (std::abs(s1.imag()) > 1e-9 * std::max(1.0, std::abs(s1)) || std::abs(s2.imag()) > 1e-9 * std::max(1.0, std::abs(s2)))
      return false;
    q[fi] = {1.0, -s1.real(), s2.real()};
    std::vector<double> np(prod.size() + 2, 0.0);
    for (size_t i = 0; i < prod.size(); i++)
      for (int j = 0; j < 3; j++) np[i + j] += prod[i] * q[fi][j];
    prod = np;
  }
  double cmax = 0;
  for (double v : c) cmax = std::max(cmax, std::abs(v));
  for (int j = 0; j <= deg; j++)
    if (std::abs(prod[j] - c[j]) > 1e-9 * cmax) return false;
  for (int fi = 0; fi < nf; fi++)
    for (int j = 0; j < 3; j++) f[fi][j] = (float)(q[fi][j] / pow(lmax, j));
  return true;
}

// C ABI: the preconditioner's factors as the solver builds them.  degree 2:
// the Horner coefficients (one factor); 4 to 12: the quadratic factors in the
// order p_1 ... p_m (the solver applies p_m first).
extern "C" int xf_cheb_factors_host(double lmax, double ratio, int degree, float* factors) {
  if (!factors || !(lmax > 0) || !(ratio > 1) || degree < 2 || degree > 12 || degree % 2) return XF_ERR_ARG;
  if (degree == 2) {
    xf_cheb2_coeffs(lmax, ratio, factors);
    return XF_OK;
  }
  float f[6][3];
  if (!xf_cheb_factors(lmax, ratio, degree, f)) return XF_ERR_ARG;
  for (int k = 0; k < degree / 2; k++)
    for (int j = 0; j < 3; j++) factors[3 * k + j] = f[k][j];
  return XF_OK;
}

bool xf_cheb4_factors(double lmax, double ratio, float f1[3], float f2[3]) {
  float f[2][3];
  if (!xf_cheb_factors(lmax, ratio, 4, f)) return false;
  for (int j = 0; j < 3; j++) {
    f1[j] = f[0][j];
    f2[j] = f[1][j];
  }
  return true;
}

bool xf_cg_poly_supported(const xf_grid* g) {
  const int64_t P = (int64_t)g->n2 * g->n3;
  if (!g->uniform || g->nbrow != 0 || P % 4 != 0 || g->n3 % 2 != 0 || g->n3 < 2 || g->n2 < 2) return false;
  const int HA = cp_halo(g->n3);
  return cp_smem(CP_TILE + 4 * HA, CP_TILE + 2 * HA, true) <= 226 * 1024;
}

namespace {

template <int MODE>
void poly_launch(const xf_op* op, CpArgs& a, const float coeffs[3]) {
  // a one-plane q buffer in shared memory: the fused update and the two-level first pass
  constexpr bool FUSE = MODE == CP_POLY_FUSED || MODE == CP_FIRST_FUSED || MODE == CP_TL_FIRST || MODE == CP_TL_BOTH;
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  a.kind = g->kind; a.S = ctx->scratch;
  a.n1 = g->n1; a.n3 = g->n3; a.P = g->n2 * g->n3;
  a.HA = cp_halo(g->n3);
  a.R0 = CP_TILE + 4 * a.HA;
  a.R1 = CP_TILE + 2 * a.HA;
  a.KS = cp_kslot(a.R1);
  a.tiles = (a.P + CP_TILE - 1) / CP_TILE;
  a.cx = (float)g->ucx; a.cy = (float)g->ucy; a.cz = (float)g->ucz;
  a.a0 = coeffs[0]; a.a1 = coeffs[1]; a.a2 = coeffs[2];
  const size_t smem = cp_smem(a.R0, a.R1, FUSE);
  static size_t attr[64] = {};   // per device: the attribute belongs to the device's copy of the kernel
  size_t& at = attr[ctx->device & 63];
  if (at < smem) {
    cudaFuncSetAttribute(k_cg_poly2<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    at = smem;
  }
  int resident = (int)((228 * 1024) / (smem + 2048));
  if (resident > 2) resident = 2;
  if (resident < 1) resident = 1;
  const int64_t B = (int64_t)ctx->sm_count * resident;
  int best = 8;
  double best_cost = 1e30;
  for (int L = 4; L <= 64; L++) {   // one wave where possible; cost ~ waves x (chunk + 5 pipeline steps)
    const int64_t items = (int64_t)a.tiles * ((g->n1 + L - 1) / L);
    const double cost = (double)((items + B - 1) / B) * (L + 5);
    if (cost < best_cost) { best_cost = cost; best = L; }
  }
  a.chunk = best;
  a.nchunk = (g->n1 + a.chunk - 1) / a.chunk;
  int64_t blocks = B, items = (int64_t)a.tiles * a.nchunk;
  if (blocks > items) blocks = items;
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  if (const char* env = getenv("XF_POLY_BLOCKS")) {   // grid cap: several items per block (tests)
    const long cap = strtol(env, nullptr, 10);
    if (cap >= 1 && cap < blocks) blocks = cap;
  }
  k_cg_poly2<MODE><<<(int)blocks, CP_THREADS, smem, ctx->stream>>>(a);
}

}  // namespace

void xf_cg_poly_launch(const xf_op* op, const float* r, float* z, const float coeffs[3]) {
  CpArgs a = {};
  a.r = r; a.z = z;
  poly_launch<CP_POLY>(op, a, coeffs);
}

// The fused launch: r_out = r - alpha q on the own cells, e += alpha p' (p' the
// current direction buffer of pa / pb), z = p(A) r_out, (r_out, r_out) and
// (r_out, z) -> the stop test and beta.  r and r_out are different buffers.
void xf_cg_polyr_launch(const xf_op* op, const float* r, float* r_out, const float* q, const float* pa,
                        const float* pb, float* e, float* z, const float coeffs[3]) {
  CpArgs a = {};
  a.r = r; a.z = z; a.q = q; a.pa = pa; a.pb = pb; a.e = e; a.rout = r_out;
  poly_launch<CP_POLY_FUSED>(op, a, coeffs);
}

// The two passes of a factored degree-4 preconditioner z = p1(A) p2(A) r:
// the first gives w = p2(A) r (with the residual update fused in when q is
// given: r_out = r - alpha q, e += alpha p', (r_out, r_out) -> the stop test),
// the second z = p1(A) w with (r, z) -> beta, r the residual after the update.
void xf_cg_poly_first_launch(const xf_op* op, const float* r, float* w, const float coeffs[3], const float* q,
                             const float* pa, const float* pb, float* e, float* r_out) {
  CpArgs a = {};
  a.r = r; a.z = w; a.q = q; a.pa = pa; a.pb = pb; a.e = e; a.rout = r_out;
  if (q) poly_launch<CP_FIRST_FUSED>(op, a, coeffs);
  else poly_launch<CP_FIRST>(op, a, coeffs);
}

void xf_cg_poly_second_launch(const xf_op* op, const float* w, const float* r, float* z, const float coeffs[3]) {
  CpArgs a = {};
  a.r = w; a.z = z; a.dr = r;
  poly_launch<CP_SECOND>(op, a, coeffs);
}

// The two-level smoother's first (input r - omega q) and last (output
// z = omega y + s w into z and z2, (z, r) -> s_zr and, with qw, (z, qw) ->
// s_zq) factor passes, or both in one (a single factor).  omega comes from
// the device scalars s_yay, s_yr.
void xf_cg_poly_tl_launch(const xf_op* op, bool first, bool last, const float* in, const float* q, float* out,
                          const float coeffs[3], int s_yay, int s_yr, const float* y, float tsc, float* z2,
                          const float* r, const float* qw, int s_zr, int s_zq) {
  CpArgs a = {};
  a.r = in; a.z = out; a.q = q;
  a.s_yay = s_yay; a.s_yr = s_yr;
  a.ty = y; a.smask = op->g->smask; a.z2 = z2; a.dr = r; a.qw = qw; a.tsc = tsc; a.s_zr = s_zr; a.s_zq = s_zq;
  if (first && last) poly_launch<CP_TL_BOTH>(op, a, coeffs);
  else if (first) poly_launch<CP_TL_FIRST>(op, a, coeffs);
  else if (last) poly_launch<CP_TL_LAST>(op, a, coeffs);
  else poly_launch<CP_FIRST>(op, a, coeffs);
}
