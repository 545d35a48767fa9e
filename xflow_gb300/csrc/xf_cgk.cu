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
  const int slot = RES ? a.slot + 1 : SL_A;
  const int ticket = RES ? a.slot : SL_A;
  if (!publish_acc<T>(S, slot, ticket, acc, sh, last)) return;
  double tot = finish_partials(S, slot, sh);
  if (threadIdx.x == 0) {
    S->scalars[slot] = tot;
    S->tickets[ticket] = 0;
    control_step(S, RES ? a.ctl : CTL_CG_ALPHA);
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

bool xf_cg_pq_supported(const xf_grid* g) {
  return g->uniform && g->nbrow == 0 && (g->n3 % 2) == 0 && g->n1 >= 2;
}

// p' = r + beta p (p in pb[I_PBUF]), q = A p', (p', q), alpha, flip.
void xf_cg_pq32(const xf_op* op, const float* r, float* pb0, float* pb1, float* q) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
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
    if (two && g->uniform && !(getenv("XF_Q2_PLAIN") && getenv("XF_Q2_PLAIN")[0] == '1')) {
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
// r32 = float(b - A x) in FP64, (r, r) -> scalars[slot + 1], then control `ctl`.
void xf_cg_res64(const xf_op* op, const double* x, const double* b, float* r32, int slot, int ctl) {
  launch_cg_q<double, true>(op, x, nullptr, b, r32, slot, ctl);
}
