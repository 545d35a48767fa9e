// Stencil kernels of the CG iterations (Laplace operator, fast rows).
//
//  q-mode:   q = A p, (p, q) -> SL_A, control CTL_CG_ALPHA (FP32 or FP64).
//  res-mode: r32 = float(b - A x) in FP64 with (r, r) -> slot+1 and a control
//            step: the mixed solver's start and its true-residual replacements.
//
// Plane march: a thread owns a (j, k) column (two consecutive cells when the
// row length is even: 8/16-byte vector loads along k) and walks i with
// x[i-1], x[i], x[i+1] in registers, prefetching plane i+2.  FP64 rows use the
// precomputed diagonal: one DMUL and six DFMA per cell, the FP64 issue rate
// being the bound on GB300.
#include <stdlib.h>

#include <type_traits>

#include "xf_control.cuh"
#include "xf_stencil.cuh"

template <typename T> struct V2;
template <> struct V2<float> { typedef float2 type; };
template <> struct V2<double> { typedef double2 type; };

constexpr int CGK_THREADS = 256;

template <typename T>
struct CgqArgs {
  StencilGrid<T> g;
  const T* __restrict__ x;
  T* __restrict__ y;
  const double* __restrict__ diag;
  const T* __restrict__ b;     // res-mode right-hand side
  float* __restrict__ y32;     // res-mode output
  DevScratch* S;
  int chunk, slot, ctl;
};

// PreDefined / PreNormal rows (rare: a branch that is warp-uniform off the
// boundary).
template <typename T>
__device__ __forceinline__ T slow_row(const StencilGrid<T>& g, const T* __restrict__ x, int i, int j, int k, int c,
                                      uint8_t kb) {
  return apply_row<T, XF_OP_LAPLACE, false>(g, x, i, j, k, c, kb);
}

template <typename T, bool USE_D>
__device__ __forceinline__ T lap_fast(uint8_t kb, T cxm, T cxp, T cym, T cyp, T czm, T czp, T d, T xm, T xc, T xp,
                                      T xjm, T xjp, T xkm, T xkp) {
  if (USE_D) {
    const T kpx = (kb & K_PX) ? cxp : T(0), kmx = (kb & K_MX) ? cxm : T(0);
    const T kpy = (kb & K_PY) ? cyp : T(0), kmy = (kb & K_MY) ? cym : T(0);
    const T kpz = (kb & K_PZ) ? czp : T(0), kmz = (kb & K_MZ) ? czm : T(0);
    T s = kpx * xp;
    s = fma(kmx, xm, s);
    s = fma(kpy, xjp, s);
    s = fma(kmy, xjm, s);
    s = fma(kpz, xkp, s);
    s = fma(kmz, xkm, s);
    return fma(d, xc, -s);
  } else {
    const T tpx = (kb & K_PX) ? cxp * (xp - xc) : T(0);
    const T tmx = (kb & K_MX) ? cxm * (xc - xm) : T(0);
    const T tpy = (kb & K_PY) ? cyp * (xjp - xc) : T(0);
    const T tmy = (kb & K_MY) ? cym * (xc - xjm) : T(0);
    const T tpz = (kb & K_PZ) ? czp * (xkp - xc) : T(0);
    const T tmz = (kb & K_MZ) ? czm * (xc - xkm) : T(0);
    return -(((tpx - tmx) + (tpy - tmy)) + (tpz - tmz));
  }
}

// Publishes the block's dot (into SL_A, or slot+1 in res-mode under slot's
// ticket) and, in the last block, totals it and runs the control step.
template <typename T, bool RES>
__device__ __forceinline__ void finish_cg_kernel(DevScratch* S, const CgqArgs<T>& a, const DotAcc<T>& acc, double* sh,
                                                 bool* last) {
  // RES: (r, r) -> slot + 1; otherwise (p, q) -> slot (SL_A for the CG's own launches)
  const int slot = RES ? a.slot + 1 : a.slot;
  const int ticket = a.slot;
  if (!publish_acc<T>(S, slot, ticket, acc, sh, last)) return;
  double tot = finish_partials(S, slot, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = tot;
    S->tickets[ticket] = 0;
    control_step(S, a.ctl);
  }
}

// Two cells (k0, k0+1) per thread; needs n3 even (then P is even and every
// cell pair is 2*sizeof(T)-aligned and inside one k-row).
template <typename T, bool USE_D, bool RES>
__global__ void __launch_bounds__(CGK_THREADS, 4) k_cg_q2(CgqArgs<T> a) {
  __shared__ double sh[32];
  __shared__ bool last;
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || (!RES && S->iscalars[I_PAUSE])) return;
  typedef typename V2<T>::type VT;
  const StencilGrid<T>& g = a.g;
  const int P = g.n2 * g.n3;
  const int p0 = 2 * (blockIdx.x * CGK_THREADS + threadIdx.x);
  const int i0 = blockIdx.y * a.chunk, i1 = min(g.n1, i0 + a.chunk);
  DotAcc<T> acc;
  if (p0 < P) {
    const int j = p0 / g.n3, k0 = p0 - j * g.n3;
    const int ojm = j > 0 ? -g.n3 : 0, ojp = j < g.n2 - 1 ? g.n3 : 0;
    const int okm = k0 > 0 ? -1 : 0, okp = k0 + 1 < g.n3 - 1 ? 2 : 1;
    const T cym = g.cym[j], cyp = g.cyp[j];
    const T czm0 = g.czm[k0], czp0 = g.czp[k0], czm1 = g.czm[k0 + 1], czp1 = g.czp[k0 + 1];
    const T* __restrict__ x = a.x;
    int c = i0 * P + p0;
    const VT zero = {T(0), T(0)};
    VT xm = i0 > 0 ? *reinterpret_cast<const VT*>(x + c - P) : zero;
    VT xc = *reinterpret_cast<const VT*>(x + c);
    VT xp = i0 + 1 < g.n1 ? *reinterpret_cast<const VT*>(x + c + P) : zero;
    uchar2 kc = *reinterpret_cast<const uchar2*>(g.kind + c);
    for (int i = i0; i < i1; i++, c += P) {
      const VT xpp = i + 2 < g.n1 ? *reinterpret_cast<const VT*>(x + c + 2 * P) : zero;
      const uchar2 kn = i + 1 < g.n1 ? *reinterpret_cast<const uchar2*>(g.kind + c + P) : make_uchar2(0, 0);
      const VT xjm = *reinterpret_cast<const VT*>(x + c + ojm);
      const VT xjp = *reinterpret_cast<const VT*>(x + c + ojp);
      const T xkm = x[c + okm], xkp = x[c + okp];
      const T cxm = g.cxm[i], cxp = g.cxp[i];
      T d0 = 0, d1 = 0;
      if (USE_D) {
        const VT dd = *reinterpret_cast<const VT*>(a.diag + c);
        d0 = dd.x; d1 = dd.y;
      }
      VT out;
      out.x = lap_fast<T, USE_D>(kc.x, cxm, cxp, cym, cyp, czm0, czp0, d0, xm.x, xc.x, xp.x, xjm.x, xjp.x, xkm, xc.y);
      out.y = lap_fast<T, USE_D>(kc.y, cxm, cxp, cym, cyp, czm1, czp1, d1, xm.y, xc.y, xp.y, xjm.y, xjp.y, xc.x, xkp);
      const int r0 = row_of(kc.x), r1 = row_of(kc.y);
      if (r0 > ROW_ACTUAL) out.x = slow_row<T>(g, x, i, j, k0, c, kc.x);
      if (r1 > ROW_ACTUAL) out.y = slow_row<T>(g, x, i, j, k0 + 1, c + 1, kc.y);
      if (RES) {
        const VT bb = *reinterpret_cast<const VT*>(a.b + c);
        out.x = bb.x - out.x;
        out.y = bb.y - out.y;
      }
      if (r0 == ROW_NONE) out.x = T(0);
      if (r1 == ROW_NONE) out.y = T(0);
      if (RES) {
        acc.add(out.x, out.x);
        acc.add(out.y, out.y);
        *reinterpret_cast<float2*>(a.y32 + c) = make_float2((float)out.x, (float)out.y);
      } else {
        acc.add(xc.x, out.x);
        acc.add(xc.y, out.y);
        *reinterpret_cast<VT*>(a.y + c) = out;
      }
      xm = xc; xc = xp; xp = xpp; kc = kn;
    }
  }
  finish_cg_kernel<T, RES>(S, a, acc, sh, &last);
}

// One cell per thread (any n3).
template <typename T, bool USE_D, bool RES>
__global__ void __launch_bounds__(CGK_THREADS, 4) k_cg_q1(CgqArgs<T> a) {
  __shared__ double sh[32];
  __shared__ bool last;
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || (!RES && S->iscalars[I_PAUSE])) return;
  const StencilGrid<T>& g = a.g;
  const int P = g.n2 * g.n3;
  const int p = blockIdx.x * CGK_THREADS + threadIdx.x;
  const int i0 = blockIdx.y * a.chunk, i1 = min(g.n1, i0 + a.chunk);
  DotAcc<T> acc;
  if (p < P) {
    const int j = p / g.n3, k = p - j * g.n3;
    const int ojm = j > 0 ? -g.n3 : 0, ojp = j < g.n2 - 1 ? g.n3 : 0;
    const int okm = k > 0 ? -1 : 0, okp = k < g.n3 - 1 ? 1 : 0;
    const T cym = g.cym[j], cyp = g.cyp[j], czm = g.czm[k], czp = g.czp[k];
    const T* __restrict__ x = a.x;
    int c = i0 * P + p;
    T xm = i0 > 0 ? x[c - P] : T(0);
    T xc = x[c];
    T xp = i0 + 1 < g.n1 ? x[c + P] : T(0);
    uint8_t kc = g.kind[c];
    for (int i = i0; i < i1; i++, c += P) {
      const T xpp = i + 2 < g.n1 ? x[c + 2 * P] : T(0);
      const uint8_t kn = i + 1 < g.n1 ? g.kind[c + P] : (uint8_t)0;
      const T xjm = x[c + ojm], xjp = x[c + ojp], xkm = x[c + okm], xkp = x[c + okp];
      const T d = USE_D ? (T)a.diag[c] : T(0);
      T v = lap_fast<T, USE_D>(kc, g.cxm[i], g.cxp[i], cym, cyp, czm, czp, d, xm, xc, xp, xjm, xjp, xkm, xkp);
      const int r = row_of(kc);
      if (r > ROW_ACTUAL) v = slow_row<T>(g, x, i, j, k, c, kc);
      if (RES) v = a.b[c] - v;
      if (r == ROW_NONE) v = T(0);
      if (RES) {
        acc.add(v, v);
        a.y32[c] = (float)v;
      } else {
        acc.add(xc, v);
        a.y[c] = v;
      }
      xm = xc; xc = xp; xp = xpp; kc = kn;
    }
  }
  finish_cg_kernel<T, RES>(S, a, acc, sh, &last);
}

// FP32 q = A p, software-pipelined plane march for uniform grids: two cells
// per thread; the centre column is loaded three planes ahead, the j+-1 / k+-1
// neighbours and the kind bytes of the next plane one step ahead, so no load
// is consumed in the step that issues it.  Per-axis constant coefficients.
struct Side2 { float2 jm, jp; float km, kp; };

// Read-only loads go through the non-coherent path explicitly (__ldg): the
// pointers travel in a parameter struct, where __restrict__ does not reach
// the compiler.
__device__ __forceinline__ Side2 load_side2(const float* __restrict__ x, int c, int ojm, int ojp, int okm, int okp) {
  Side2 s;
  s.jm = __ldg(reinterpret_cast<const float2*>(x + c + ojm));
  s.jp = __ldg(reinterpret_cast<const float2*>(x + c + ojp));
  s.km = __ldg(x + c + okm);
  s.kp = __ldg(x + c + okp);
  return s;
}

// Actual rows use A p = D p_c - (cx (p_i+1 + p_i-1) + cy (..) + cz (..)): the
// CG direction is zero on every inactive cell, so a closed (Fictive) face's
// neighbour term vanishes by itself and only the diagonal D depends on the
// open faces; D comes from a 64-entry table indexed by the face bits.
// BROWS: the grid has PreDefined/PreNormal rows.  Without them the (never
// taken) boundary-row branch is compiled out: its mere presence costs ~15% here.
// Prefetch addresses are clamped to the box instead of bounds-checked: a
// clamped (out-of-box) plane only ever feeds rows on the box faces, which are
// never Actual rows, so its values are never used.
template <bool BROWS>
__global__ void __launch_bounds__(CGK_THREADS, 4) k_cg_q2u(CgqArgs<float> a, float cx, float cy, float cz) {
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  __syncthreads();
  const StencilGrid<float>& g = a.g;
  const int n1 = g.n1, n3 = g.n3;
  const int P = g.n2 * n3;
  const int p0 = 2 * (blockIdx.x * CGK_THREADS + threadIdx.x);
  const int i0 = blockIdx.y * a.chunk, i1 = min(n1, i0 + a.chunk);
  DotAcc<float> acc;
  if (p0 < P) {
    const int j = p0 / n3, k0 = p0 - j * n3;
    const int ojm = j > 0 ? -n3 : 0, ojp = j < g.n2 - 1 ? n3 : 0;
    const int okm = k0 > 0 ? -1 : 0, okp = k0 + 1 < n3 - 1 ? 2 : 1;
    const float* __restrict__ x = a.x;
    const int last_plane = n1 - 1;
    auto ld = [&](int i) -> float2 {
      const int ic = min(max(i, 0), last_plane);
      return __ldg(reinterpret_cast<const float2*>(x + ic * P + p0));
    };
    auto ldk = [&](int i) -> uchar2 {
      return __ldg(reinterpret_cast<const uchar2*>(g.kind + min(i, last_plane) * P + p0));
    };
    float2 xm = ld(i0 - 1), xc = ld(i0), xp = ld(i0 + 1), xpp = ld(i0 + 2);
    uchar2 kc = ldk(i0), kn = ldk(i0 + 1);
    Side2 sc = load_side2(x, i0 * P + p0, ojm, ojp, okm, okp);
    for (int i = i0; i < i1; i++) {
      const int c = i * P + p0;
      // loads for later steps, in flight during this step's arithmetic
      const float2 x3 = ld(i + 3);
      const uchar2 kn2 = ldk(i + 2);
      const Side2 sn = load_side2(x, min(i + 1, last_plane) * P + p0, ojm, ojp, okm, okp);
      float2 out;
      out.x = fmaf(dtab[kc.x & 63], xc.x, -fmaf(cx, xp.x + xm.x, fmaf(cy, sc.jp.x + sc.jm.x, cz * (xc.y + sc.km))));
      out.y = fmaf(dtab[kc.y & 63], xc.y, -fmaf(cx, xp.y + xm.y, fmaf(cy, sc.jp.y + sc.jm.y, cz * (sc.kp + xc.x))));
      const int r0 = row_of(kc.x), r1 = row_of(kc.y);
      if (BROWS) {
        if (r0 > ROW_ACTUAL) out.x = slow_row<float>(g, x, i, j, k0, c, kc.x);
        if (r1 > ROW_ACTUAL) out.y = slow_row<float>(g, x, i, j, k0 + 1, c + 1, kc.y);
      }
      if (r0 == ROW_NONE) out.x = 0.f;
      if (r1 == ROW_NONE) out.y = 0.f;
      acc.add(xc.x, out.x);
      acc.add(xc.y, out.y);
      *reinterpret_cast<float2*>(a.y + c) = out;
      xm = xc; xc = xp; xp = xpp; xpp = x3;
      kc = kn; kn = kn2;
      sc = sn;
    }
  }
  finish_cg_kernel<float, false>(S, a, acc, sh, &last);
}

// ---------------------------------------------------------------------------
// FP32 direction update fused into the stencil, for uniform grids without
// PreDefined/PreNormal rows:
//     p' = r + beta p   (every cell; r and p are zero off the active set),
//     q  = A p',  (p', q) -> SL_A, control CTL_CG_ALPHA_FLIP.
// p' is formed on the fly wherever the stencil needs it (the centre column
// and its four side neighbours), so p' must not overwrite p while other
// threads still read p: the direction ping-pongs between two buffers and the
// device flag I_PBUF names the one holding the current p (flipped by the
// control step once every block has read it).
// The grid is one wave of resident blocks; each block walks work items
// (plane chunk, column group) round-robin, plane-chunk major so that blocks
// on neighbouring column groups march the same planes at the same time (their
// shared halo rows stay in L2), and publishes its dot once.
struct PqArgs {
  StencilGrid<float> g;
  const float* r;
  float* pb0;
  float* pb1;
  float* q;
  DevScratch* S;
  int chunk, nchunk, bx;
};

struct SideRaw { float2 rjm, rjp, pjm, pjp; float rkm, rkp, pkm, pkp; };

__device__ __forceinline__ SideRaw load_side_raw(const float* __restrict__ r, const float* __restrict__ p, int c,
                                                 int ojm, int ojp, int okm, int okp) {
  SideRaw s;
  s.rjm = __ldg(reinterpret_cast<const float2*>(r + c + ojm));
  s.rjp = __ldg(reinterpret_cast<const float2*>(r + c + ojp));
  s.pjm = __ldg(reinterpret_cast<const float2*>(p + c + ojm));
  s.pjp = __ldg(reinterpret_cast<const float2*>(p + c + ojp));
  s.rkm = __ldg(r + c + okm);
  s.rkp = __ldg(r + c + okp);
  s.pkm = __ldg(p + c + okm);
  s.pkp = __ldg(p + c + okp);
  return s;
}

__device__ __forceinline__ float2 dir2(float beta, float2 r, float2 p) {
  return make_float2(fmaf(beta, p.x, r.x), fmaf(beta, p.y, r.y));
}

__device__ __forceinline__ Side2 dir_side(float beta, const SideRaw& s) {
  Side2 o;
  o.jm = dir2(beta, s.rjm, s.pjm);
  o.jp = dir2(beta, s.rjp, s.pjp);
  o.km = fmaf(beta, s.pkm, s.rkm);
  o.kp = fmaf(beta, s.pkp, s.rkp);
  return o;
}

__global__ void __launch_bounds__(CGK_THREADS, 3) k_cg_pq2u(PqArgs a, float cx, float cy, float cz) {
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  const float beta = (float)S->scalars[D_BETA];
  const int sel = (int)S->iscalars[I_PBUF];
  const float* __restrict__ po = sel ? a.pb1 : a.pb0;
  float* __restrict__ pn = sel ? a.pb0 : a.pb1;
  const float* __restrict__ r = a.r;
  float* __restrict__ q = a.q;
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  __syncthreads();
  const StencilGrid<float>& g = a.g;
  const int n1 = g.n1, n3 = g.n3;
  const int P = g.n2 * n3;
  const int last_plane = n1 - 1;
  const int items = a.nchunk * a.bx;
  DotAcc<float> acc;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int ic = item / a.bx, gx = item - ic * a.bx;
    const int p0 = 2 * (gx * CGK_THREADS + threadIdx.x);
    if (p0 >= P) continue;
    const int i0 = ic * a.chunk, i1 = min(n1, i0 + a.chunk);
    const int j = p0 / n3, k0 = p0 - j * n3;
    const int ojm = j > 0 ? -n3 : 0, ojp = j < g.n2 - 1 ? n3 : 0;
    const int okm = k0 > 0 ? -1 : 0, okp = k0 + 1 < n3 - 1 ? 2 : 1;
    // Plane addresses clamped to the box: a clamped plane only feeds rows on
    // the box faces, which are never Actual rows (their outputs are zeroed).
    auto pl = [&](int i) { return min(max(i, 0), last_plane) * P + p0; };
    auto ldr = [&](int i) { return __ldg(reinterpret_cast<const float2*>(r + pl(i))); };
    auto ldp = [&](int i) { return __ldg(reinterpret_cast<const float2*>(po + pl(i))); };
    auto ldk = [&](int i) { return __ldg(reinterpret_cast<const uchar2*>(g.kind + pl(i))); };
    float2 xm = dir2(beta, ldr(i0 - 1), ldp(i0 - 1));
    float2 xc = dir2(beta, ldr(i0), ldp(i0));
    float2 xp = dir2(beta, ldr(i0 + 1), ldp(i0 + 1));
    float2 r2 = ldr(i0 + 2), p2 = ldp(i0 + 2);
    uchar2 kc = ldk(i0), kn = ldk(i0 + 1);
    Side2 sc = dir_side(beta, load_side_raw(r, po, pl(i0), ojm, ojp, okm, okp));
    for (int i = i0; i < i1; i++) {
      const int c = i * P + p0;
      // loads for later steps, in flight during this step's arithmetic
      const float2 r3 = ldr(i + 3), p3 = ldp(i + 3);
      const uchar2 kn2 = ldk(i + 2);
      const SideRaw sn = load_side_raw(r, po, pl(i + 1), ojm, ojp, okm, okp);
      float2 out;
      out.x = fmaf(dtab[kc.x & 63], xc.x, -fmaf(cx, xp.x + xm.x, fmaf(cy, sc.jp.x + sc.jm.x, cz * (xc.y + sc.km))));
      out.y = fmaf(dtab[kc.y & 63], xc.y, -fmaf(cx, xp.y + xm.y, fmaf(cy, sc.jp.y + sc.jm.y, cz * (sc.kp + xc.x))));
      if (row_of(kc.x) == ROW_NONE) out.x = 0.f;
      if (row_of(kc.y) == ROW_NONE) out.y = 0.f;
      acc.add(xc.x, out.x);
      acc.add(xc.y, out.y);
      *reinterpret_cast<float2*>(pn + c) = xc;
      *reinterpret_cast<float2*>(q + c) = out;
      xm = xc; xc = xp; xp = dir2(beta, r2, p2);
      r2 = r3; p2 = p3;
      kc = kn; kn = kn2;
      sc = dir_side(beta, sn);
    }
  }
  if (!publish_acc<float>(S, SL_A, SL_A, acc, sh, &last)) return;
  double tot = finish_partials(S, SL_A, sh);
  if (threadIdx.x == 0) {
    S->scalars[SL_A] = tot;
    S->tickets[SL_A] = 0;
    control_step(S, CTL_CG_ALPHA_FLIP);
  }
}

// ---------------------------------------------------------------------------
// The same fused step with the plane staged in shared memory.  A block owns a
// tile of PQT_V * 256 consecutive cells of the flattened (j, k) plane (8 per
// thread, two 16-byte vectors per field) and marches along i.  Per plane it
// forms p' = r + beta p once: its own cells in registers (x-neighbours stay in
// registers across the march) and a halo of n3 + 1 cells on either side, then
// writes the plane's p' tile to shared memory, from where the j+-1 and k+-1
// neighbours are read.  The raw r and p of plane i+2 (own cells) and of the
// halo of plane i+1 are in flight while plane i is computed.  Shared memory is
// double-buffered: one barrier per plane.
// Layout of a buffer: [pad | left halo (H) | own tile | right halo (H)], with
// H = n3 + 1 and the own tile at a 16-byte aligned offset.
constexpr int PQT_V = 8;
constexpr int PQT_TILE = CGK_THREADS * PQT_V;

struct PqtArgs {
  StencilGrid<float> g;
  const float* r;
  float* pb0;
  float* pb1;
  float* q;
  DevScratch* S;
  int chunk, nchunk, tiles;   // work items: nchunk plane chunks x tiles per plane
  int H, off, stride;         // halo width, own-tile offset, floats per buffer
};

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__global__ void __launch_bounds__(CGK_THREADS, 2) k_cg_pqt(PqtArgs a, float cx, float cy, float cz) {
  extern __shared__ float4 smem4[];
  float* sbuf = reinterpret_cast<float*>(smem4);
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  const float beta = (float)S->scalars[D_BETA];
  const int sel = (int)S->iscalars[I_PBUF];
  const float* __restrict__ po = sel ? a.pb1 : a.pb0;
  float* __restrict__ pn = sel ? a.pb0 : a.pb1;
  const float* __restrict__ r = a.r;
  float* __restrict__ q = a.q;
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  const StencilGrid<float>& g = a.g;
  const int n1 = g.n1, n3 = g.n3;
  const int P = g.n2 * n3;
  const int last_plane = n1 - 1;
  const int H = a.H, OFF = a.off;
  const int nhalo = 2 * H;                    // halo cells per plane
  const int items = a.nchunk * a.tiles;
  DotAcc<float> acc;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int ic = item / a.tiles, tile = item - ic * a.tiles;
    const int base = tile * PQT_TILE;
    const int t0 = base + threadIdx.x * PQT_V;   // first own plane cell
    // P is a multiple of 4: the low four cells are valid or none, and so are the high four
    const bool own = t0 < P, own_hi = t0 + 4 < P;
    const int i0 = ic * a.chunk, i1 = min(n1, i0 + a.chunk);
    auto pl = [&](int i) { return min(max(i, 0), last_plane) * P; };
    // own raw loads (8 cells: two float4 of r and of p)
    auto ld_own = [&](int i, float4& r0, float4& r1, float4& p0, float4& p1) {
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      const int c = pl(i) + t0;
      r0 = own ? ldg4(r + c) : z;
      p0 = own ? ldg4(po + c) : z;
      r1 = own_hi ? ldg4(r + c + 4) : z;
      p1 = own_hi ? ldg4(po + c + 4) : z;
    };
    auto dir4 = [&](float4 rr, float4 pp) {
      return make_float4(fmaf(beta, pp.x, rr.x), fmaf(beta, pp.y, rr.y), fmaf(beta, pp.z, rr.z), fmaf(beta, pp.w, rr.w));
    };
    // halo: up to HPT cells per thread, plane positions base-H.. and base+TILE..
    constexpr int HPT = 4;   // covers 2H <= 4 * 256, i.e. n3 <= 511 (checked on the host)
    auto halo_pos = [&](int h) { return h < H ? base - H + h : base + PQT_TILE + (h - H); };
    float hr[HPT], hp[HPT];
    auto ld_halo = [&](int i) {
      const int pi = pl(i);
#pragma unroll
      for (int u = 0; u < HPT; u++) {
        const int h = threadIdx.x + u * CGK_THREADS;
        const int x = halo_pos(h);
        const bool ok = h < nhalo && x >= 0 && x < P;
        hr[u] = ok ? __ldg(r + pi + x) : 0.f;
        hp[u] = ok ? __ldg(po + pi + x) : 0.f;
      }
    };
    float4 xm0, xm1, xc0, xc1, xp0, xp1;
    float4 r2a, r2b, p2a, p2b;
    {
      float4 a0, a1, b0, b1;
      ld_own(i0 - 1, a0, a1, b0, b1);
      xm0 = dir4(a0, b0); xm1 = dir4(a1, b1);
      ld_own(i0, a0, a1, b0, b1);
      xc0 = dir4(a0, b0); xc1 = dir4(a1, b1);
      ld_own(i0 + 1, a0, a1, b0, b1);
      xp0 = dir4(a0, b0); xp1 = dir4(a1, b1);
      ld_own(i0 + 2, r2a, r2b, p2a, p2b);
    }
    ld_halo(i0);
    auto ld_kind = [&](int i) {
      const uint32_t* kp = reinterpret_cast<const uint32_t*>(g.kind + pl(i) + t0);
      return make_uint2(own ? __ldg(kp) : 0u, own_hi ? __ldg(kp + 1) : 0u);
    };
    uint2 kc = ld_kind(i0);
    for (int i = i0; i < i1; i++) {
      float* buf = sbuf + (i & 1) * a.stride;
      // p' of plane i into shared memory: own tile and halo
      *reinterpret_cast<float4*>(buf + OFF + threadIdx.x * PQT_V) = xc0;
      *reinterpret_cast<float4*>(buf + OFF + threadIdx.x * PQT_V + 4) = xc1;
#pragma unroll
      for (int u = 0; u < HPT; u++) {
        const int h = threadIdx.x + u * CGK_THREADS;
        if (h < nhalo) buf[h < H ? OFF - H + h : OFF + PQT_TILE + (h - H)] = fmaf(beta, hp[u], hr[u]);
      }
      // loads for later planes, in flight during this plane's arithmetic
      float4 r3a, r3b, p3a, p3b;
      ld_own(i + 3, r3a, r3b, p3a, p3b);
      ld_halo(i + 1);
      const uint2 kn = ld_kind(i + 1);
      __syncthreads();
      if (own) {
        const float* s0 = buf + OFF + threadIdx.x * PQT_V;
        float c[8] = {xc0.x, xc0.y, xc0.z, xc0.w, xc1.x, xc1.y, xc1.z, xc1.w};
        const float m[8] = {xm0.x, xm0.y, xm0.z, xm0.w, xm1.x, xm1.y, xm1.z, xm1.w};
        const float pp[8] = {xp0.x, xp0.y, xp0.z, xp0.w, xp1.x, xp1.y, xp1.z, xp1.w};
        float jm[8], jp[8];
#pragma unroll
        for (int v = 0; v < 8; v += 2) {
          const float2 a2 = *reinterpret_cast<const float2*>(s0 + v - n3);
          const float2 b2 = *reinterpret_cast<const float2*>(s0 + v + n3);
          jm[v] = a2.x; jm[v + 1] = a2.y; jp[v] = b2.x; jp[v + 1] = b2.y;
        }
        const float km0 = s0[-1], kp7 = s0[8];
        const uint32_t kw[2] = {kc.x, kc.y};
        float out[8];
#pragma unroll
        for (int v = 0; v < 8; v++) {
          const uint32_t kb = (kw[v >> 2] >> (8 * (v & 3))) & 0xffu;
          const float km = v == 0 ? km0 : c[v - 1];
          const float kp = v == 7 ? kp7 : c[v + 1];
          float o = fmaf(dtab[kb & 63], c[v], -fmaf(cx, pp[v] + m[v], fmaf(cy, jp[v] + jm[v], cz * (kp + km))));
          if ((kb >> K_ROW_SHIFT) == ROW_NONE) o = 0.f;
          out[v] = o;
          acc.add(c[v], o);
        }
        const int cg = i * P + t0;
        *reinterpret_cast<float4*>(pn + cg) = xc0;
        *reinterpret_cast<float4*>(q + cg) = make_float4(out[0], out[1], out[2], out[3]);
        if (own_hi) {
          *reinterpret_cast<float4*>(pn + cg + 4) = xc1;
          *reinterpret_cast<float4*>(q + cg + 4) = make_float4(out[4], out[5], out[6], out[7]);
        }
      }
      xm0 = xc0; xm1 = xc1; xc0 = xp0; xc1 = xp1;
      xp0 = dir4(r2a, p2a); xp1 = dir4(r2b, p2b);
      r2a = r3a; r2b = r3b; p2a = p3a; p2b = p3b;
      kc = kn;
    }
    __syncthreads();   // the next item rewrites both buffers
  }
  if (!publish_acc<float>(S, SL_A, SL_A, acc, sh, &last)) return;
  double tot = finish_partials(S, SL_A, sh);
  if (threadIdx.x == 0) {
    S->scalars[SL_A] = tot;
    S->tickets[SL_A] = 0;
    control_step(S, CTL_CG_ALPHA_FLIP);
  }
}

// The tiled kernel needs P to be a multiple of 4 (16-byte own vectors in
// every plane), n3 even (8-byte aligned j+-1 reads from shared memory) and
// 2 (n3 + 1) <= 4 * 256 halo cells.
static bool pqt_supported(const xf_grid* g) {
  const int64_t P = (int64_t)g->n2 * g->n3;
  return (P % 4) == 0 && (g->n3 % 2) == 0 && 2 * (g->n3 + 1) <= 4 * CGK_THREADS && g->n3 >= 2 && g->n2 >= 2;
}

bool xf_cg_pq_supported(const xf_grid* g) {
  return g->uniform && g->nbrow == 0 && (g->n3 % 2) == 0 && g->n1 >= 2;
}

static void launch_pqt(const xf_op* op, const float* r, float* pb0, float* pb1, float* q) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  PqtArgs a;
  a.g = make_stencil_grid<float>(g, nullptr);
  a.r = r; a.pb0 = pb0; a.pb1 = pb1; a.q = q; a.S = ctx->scratch;
  const int P = g->n2 * g->n3;
  a.H = g->n3 + 1;
  a.off = (a.H + 3) & ~3;
  a.stride = (a.off + PQT_TILE + a.H + 3) & ~3;
  a.tiles = (P + PQT_TILE - 1) / PQT_TILE;
  const size_t smem = 2 * (size_t)a.stride * sizeof(float);
  static int resident = 0;   // blocks per SM at this kernel's launch bounds and shared memory
  static size_t resident_smem = 0;
  if (!resident || resident_smem != smem) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_cg_pqt, CGK_THREADS, smem) != cudaSuccess ||
        resident < 1)
      resident = 1;
    resident_smem = smem;
  }
  const int64_t B = (int64_t)ctx->sm_count * resident;
  // plane chunk: the length whose last wave wastes least (cost ~ waves x
  // (chunk + 2 start-up planes))
  int best = 8;
  double best_cost = 1e30;
  for (int L = 4; L <= 32; L++) {
    const int64_t items = (int64_t)a.tiles * ((g->n1 + L - 1) / L);
    const double cost = (double)((items + B - 1) / B) * (L + 2);
    if (cost < best_cost) { best_cost = cost; best = L; }
  }
  a.chunk = best;
  a.nchunk = (g->n1 + a.chunk - 1) / a.chunk;
  int64_t blocks = B, items = (int64_t)a.tiles * a.nchunk;
  if (blocks > items) blocks = items;
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  k_cg_pqt<<<(int)blocks, CGK_THREADS, smem, ctx->stream>>>(a, (float)g->ucx, (float)g->ucy, (float)g->ucz);
}

// p' = r + beta p (p in pb[I_PBUF]), q = A p', (p', q), alpha, flip: the
// bulk-staged kernel (xf_cgb.cu) where the plane allows it, else the
// shared-memory tiled kernel, else the register march.  variant: 0
// automatic, 1 register march, 2 tiled, 3 bulk-staged.
bool xf_cg_pqb_supported(const xf_grid* g);
void xf_cg_pqb_launch(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int ctl = CTL_CG_ALPHA_FLIP);
void xf_cg_pq32_variant(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int variant);
void xf_cg_pq32(const xf_op* op, const float* r, float* pb0, float* pb1, float* q) {
  // XF_PQT: "0" the register march, "1" the tiled kernel, "2" the bulk-staged
  // kernel (each where the plane allows it); unset: automatic
  const char* env = getenv("XF_PQT");
  const int v = !env ? 0 : env[0] == '0' ? 1 : env[0] == '1' ? 2 : env[0] == '2' ? 3 : 0;
  xf_cg_pq32_variant(op, r, pb0, pb1, q, v);
}
bool xf_cg_pqt_supported(const xf_grid* g) { return pqt_supported(g); }

void xf_cg_pq32_variant(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int variant) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  if ((variant == 0 || variant == 3) && xf_cg_pqb_supported(g)) {
    xf_cg_pqb_launch(op, r, pb0, pb1, q);
    return;
  }
  if (variant != 1 && pqt_supported(g)) {
    launch_pqt(op, r, pb0, pb1, q);
    return;
  }
  static int resident = 0;   // blocks per SM at this kernel's launch bounds
  if (!resident) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_cg_pq2u, CGK_THREADS, 0) != cudaSuccess ||
        resident < 1)
      resident = 1;
  }
  PqArgs a;
  a.g = make_stencil_grid<float>(g, nullptr);
  a.r = r; a.pb0 = pb0; a.pb1 = pb1; a.q = q; a.S = ctx->scratch;
  const int P = g->n2 * g->n3;
  a.bx = (P / 2 + CGK_THREADS - 1) / CGK_THREADS;
  a.chunk = 8;
  a.nchunk = (g->n1 + a.chunk - 1) / a.chunk;
  int64_t items = (int64_t)a.bx * a.nchunk;
  int64_t blocks = (int64_t)ctx->sm_count * resident;
  if (blocks > items) blocks = items;
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  k_cg_pq2u<<<(int)blocks, CGK_THREADS, 0, ctx->stream>>>(a, (float)g->ucx, (float)g->ucy, (float)g->ucz);
}

template <typename T, bool RES>
static void launch_cg_q(const xf_op* op, const T* x, T* y, const T* b, float* y32, int slot, int ctl) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  CgqArgs<T> a;
  a.g = make_stencil_grid<T>(g, nullptr);
  a.x = x; a.y = y; a.b = b; a.y32 = y32; a.diag = g->diag; a.S = ctx->scratch; a.slot = slot; a.ctl = ctl;
  const int P = g->n2 * g->n3;
  const bool two = (g->n3 % 2) == 0;
  const int per = two ? 2 : 1;
  const int bx = (P / per + CGK_THREADS - 1) / CGK_THREADS;
  int chunk = 16;
  while ((int64_t)bx * ((g->n1 + chunk - 1) / chunk) > RED_MAX_BLOCKS) chunk *= 2;
  a.chunk = chunk;
  dim3 grid(bx, (g->n1 + chunk - 1) / chunk);
  constexpr bool D = std::is_same<T, double>::value;
  if constexpr (!D && !RES) {
    if (two && g->uniform) {
      if (g->nbrow > 0) k_cg_q2u<true><<<grid, CGK_THREADS, 0, ctx->stream>>>(a, (float)g->ucx, (float)g->ucy, (float)g->ucz);
      else k_cg_q2u<false><<<grid, CGK_THREADS, 0, ctx->stream>>>(a, (float)g->ucx, (float)g->ucy, (float)g->ucz);
      return;
    }
  }
  if (two) k_cg_q2<T, D, RES><<<grid, CGK_THREADS, 0, ctx->stream>>>(a);
  else k_cg_q1<T, D, RES><<<grid, CGK_THREADS, 0, ctx->stream>>>(a);
}

// q = A p with (p, q) -> SL_A and the CG alpha step.  Laplace operators only.
void xf_cg_q64(const xf_op* op, const double* p, double* q) {
  launch_cg_q<double, false>(op, p, q, nullptr, nullptr, SL_A, CTL_CG_ALPHA);
}
void xf_cg_q32(const xf_op* op, const float* p, float* q) {
  launch_cg_q<float, false>(op, p, q, nullptr, nullptr, SL_A, CTL_CG_ALPHA);
}
// q = A p with (p, q) -> scalars[slot] and no control step (the flexible CG's
// host loop reads the dot).  Laplace operators only.
void xf_cg_q32_dot(const xf_op* op, const float* p, float* q, int slot) {
  launch_cg_q<float, false>(op, p, q, nullptr, nullptr, slot, CTL_NONE);
}

// The coarse correction of the learned two-level preconditioner, prolongated
// and multiplied by A in one pass: y = P zc (the value of the cell's
// 4 x 4 x 4 block, 0 on inactive cells), q = A y and (y, q) -> scalars[slot].
// zc is the network's FP32 output (its FP64 copy is an exact widening, and a
// conversion from FP64 per fine cell would run on the FP64 pipe, 1/58 of the
// FP32 rate here).  Every value y takes at a stencil point is a coarse value
// (0 behind a closed face), and the row is k_cg_q2u's expression with
// k_cg_q2u's thread mapping and accumulation order, so y, q and (y, q) are bit
// for bit those of the prolongation followed by xf_cg_q32_dot.  Uniform
// Laplace grids without boundary rows, n3 even.
__global__ void __launch_bounds__(CGK_THREADS, 4) k_tl_prolong_ay(CgqArgs<float> a, const float* __restrict__ zc,
                                                                  int c2, int c3, float* __restrict__ yout,
                                                                  float cx, float cy, float cz) {
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ float dtab[64];
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  if (threadIdx.x < 64) {
    const int b = threadIdx.x;
    dtab[b] = cx * (float)(((b >> 0) & 1) + ((b >> 1) & 1)) + cy * (float)(((b >> 2) & 1) + ((b >> 3) & 1)) +
              cz * (float)(((b >> 4) & 1) + ((b >> 5) & 1));
  }
  __syncthreads();
  const StencilGrid<float>& g = a.g;
  const int n1 = g.n1, n3 = g.n3;
  const int P = g.n2 * n3;
  const int p0 = 2 * (blockIdx.x * CGK_THREADS + threadIdx.x);
  const int i0 = blockIdx.y * a.chunk, i1 = min(n1, i0 + a.chunk);
  DotAcc<float> acc;
  if (p0 < P) {
    const int j = p0 / n3, k0 = p0 - j * n3;
    // block coordinates and block-face flags of this thread's row and its two
    // cells (interior cells only; ghost cells take the ROW_NONE branch): a
    // neighbour across a block face is the next block's value, else the own
    const int sJ = c3, sI = c2 * c3;
    const int Jb = 1 + ((j - 1) >> 2);
    const bool jlo = ((j - 1) & 3) == 0, jhi = ((j - 1) & 3) == 3;
    int Kb[2];
    bool klo[2], khi[2];
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int k = k0 + t;
      Kb[t] = 1 + ((k - 1) >> 2);
      klo[t] = ((k - 1) & 3) == 0;
      khi[t] = ((k - 1) & 3) == 3;
    }
    for (int i = i0; i < i1; i++) {
      const int c = i * P + p0;
      const uchar2 kk = __ldg(reinterpret_cast<const uchar2*>(g.kind + c));
      const uint8_t kbs[2] = {kk.x, kk.y};
      const int Ib = 1 + ((i - 1) >> 2);
      const bool ilo = ((i - 1) & 3) == 0, ihi = ((i - 1) & 3) == 3;
      const int brow = (Ib * c2 + Jb) * c3;
      float yv[2], out[2];
#pragma unroll
      for (int t = 0; t < 2; t++) {
        const uint8_t kb = kbs[t];
        if (row_of(kb) == ROW_NONE) {
          yv[t] = 0.f;
          out[t] = 0.f;
          continue;
        }
        const int bc = brow + Kb[t];
        const float yc = __ldg(zc + bc);
        // a neighbour's value: the next block's across a block face, else the own; 0 behind a closed face
        auto nb = [&](uint8_t bit, bool cross, int off) -> float {
          if (!(kb & bit)) return 0.f;
          return cross ? __ldg(zc + bc + off) : yc;
        };
        const float ypx = nb(K_PX, ihi, sI), ymx = nb(K_MX, ilo, -sI);
        const float ypy = nb(K_PY, jhi, sJ), ymy = nb(K_MY, jlo, -sJ);
        const float ypz = nb(K_PZ, khi[t], 1), ymz = nb(K_MZ, klo[t], -1);
        yv[t] = yc;
        out[t] = fmaf(dtab[kb & 63], yc, -fmaf(cx, ypx + ymx, fmaf(cy, ypy + ymy, cz * (ypz + ymz))));
      }
      acc.add(yv[0], out[0]);
      acc.add(yv[1], out[1]);
      *reinterpret_cast<float2*>(yout + c) = make_float2(yv[0], yv[1]);
      *reinterpret_cast<float2*>(a.y + c) = make_float2(out[0], out[1]);
    }
  }
  finish_cg_kernel<float, false>(S, a, acc, sh, &last);
}

bool xf_tl_prolong_ay_supported(const xf_grid* g) { return g->uniform && g->nbrow == 0 && g->n3 % 2 == 0; }

void xf_tl_prolong_ay(const xf_op* op, const float* zc, int c2, int c3, float* y, float* ay, int slot) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  CgqArgs<float> a;
  a.g = make_stencil_grid<float>(g, nullptr);
  a.x = nullptr; a.y = ay; a.b = nullptr; a.y32 = nullptr; a.diag = g->diag; a.S = ctx->scratch; a.slot = slot;
  a.ctl = CTL_NONE;
  const int P = g->n2 * g->n3;
  const int bx = (P / 2 + CGK_THREADS - 1) / CGK_THREADS;
  int chunk = 16;
  while ((int64_t)bx * ((g->n1 + chunk - 1) / chunk) > RED_MAX_BLOCKS) chunk *= 2;
  a.chunk = chunk;
  dim3 grid(bx, (g->n1 + chunk - 1) / chunk);
  k_tl_prolong_ay<<<grid, CGK_THREADS, 0, ctx->stream>>>(a, zc, c2, c3, y, (float)g->ucx, (float)g->ucy,
                                                          (float)g->ucz);
}
// r32 = float(b - A x) in FP64, (r, r) -> scalars[slot + 1], then control `ctl`.
void xf_cg_res64(const xf_op* op, const double* x, const double* b, float* r32, int slot, int ctl) {
  launch_cg_q<double, true>(op, x, nullptr, b, r32, slot, ctl);
}
