// Fused FP32 CG iteration for the Laplace operator, with shared-memory staged
// planes.
//
//  K1: p <- r + beta p (formed on the fly at every stencil point), q = A p,
//      (p, q) -> alpha (CTL_CG_ALPHA); writes p.
//  K2: q = A p recomputed, e += alpha p, r -= alpha q, (r, r) -> beta
//      (CTL_CG_BETA_FLIP).
// q is never stored: 13 + 21 = 34 bytes per cell per iteration instead of
// 9 + 24 + 12 = 45 for separate matvec / update / direction kernels.
//
// Staging: a work item is a contiguous range of CF_TP plane positions
// (p = j*n3 + k) over CF_CHUNK consecutive i-planes.  For each plane one bulk
// copy per field brings [range - H, range + H) (H >= n3 + 1, so the j-1 and
// j+1 rows come along) into a 4-deep shared-memory ring completed on
// mbarriers, two planes ahead of the plane being computed.  i+-1 come from the
// neighbouring ring slots, j+-1 and k+-1 from the same slot.  The per-cell
// kind byte (and, in K2, e and r) are prefetched one plane ahead in registers.
// The grid is persistent (resident blocks only) and loops over work items.
// Requires n2*n3 % 4 == 0.
#include "xf_bulk.cuh"
#include "xf_control.cuh"
#include "xf_stencil.cuh"

constexpr int CF_THREADS = 256;
constexpr int CF_TP = 1024;    // plane positions per work item (4 per thread)
constexpr int CF_NB = 4;       // ring depth
constexpr int CF_CHUNK = 16;   // planes per work item

struct CgfArgs {
  StencilGrid<float> g;
  float* r;                        // K1 input, K2 in/out
  float* pbuf0;                    // direction ping-pong buffers
  float* pbuf1;
  float* e;                        // K2 in/out
  DevScratch* S;
  int H, W, nx, items;             // halo, tile width (floats), items along the plane, total items
  float ucx, ucy, ucz;             // uniform grids: per-axis coefficients
};

// Staged-plane accessor for the boundary rows.
template <int MODE>
struct SmemAcc {
  const float *m0, *m1, *m2;   // planes i-1, i, i+1 of field 0 (r or p)
  const float *o0, *o1, *o2;   // planes of field 1 (p_old) in MODE 1
  float beta;
  int s, n3;
  __device__ __forceinline__ float operator()(int a, int b, int d) const {
    const int idx = s + b * n3 + d;
    const float* m = a < 0 ? m0 : (a == 0 ? m1 : m2);
    if (MODE == 1) {
      const float* o = a < 0 ? o0 : (a == 0 ? o1 : o2);
      return fmaf(beta, o[idx], m[idx]);
    }
    return m[idx];
  }
};

template <int MODE>
__device__ __noinline__ float staged_boundary_row(const StencilGrid<float>* g, SmemAcc<MODE> A, int i, int j, int k,
                                                  int c, int row) {
  return boundary_row_acc<float, false>(*g, A, i, j, k, c, row);
}

__device__ __forceinline__ float lap_row_f(uint8_t kb, float cxm, float cxp, float cym, float cyp, float czm,
                                           float czp, float xm, float xc, float xp, float xjm, float xjp, float xkm,
                                           float xkp) {
  const float tpx = (kb & K_PX) ? cxp * (xp - xc) : 0.f;
  const float tmx = (kb & K_MX) ? cxm * (xc - xm) : 0.f;
  const float tpy = (kb & K_PY) ? cyp * (xjp - xc) : 0.f;
  const float tmy = (kb & K_MY) ? cym * (xc - xjm) : 0.f;
  const float tpz = (kb & K_PZ) ? czp * (xkp - xc) : 0.f;
  const float tmz = (kb & K_MZ) ? czm * (xc - xkm) : 0.f;
  return -(((tpx - tmx) + (tpy - tmy)) + (tpz - tmz));
}

template <int MODE, bool UNI>
__global__ void __launch_bounds__(CF_THREADS, 3) k_cgf(const __grid_constant__ CgfArgs a) {
  constexpr int NF = MODE == 1 ? 2 : 1;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ int issued_hi;
  DevScratch* S = a.S;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  const StencilGrid<float>& g = a.g;
  const int n1 = g.n1, n3 = g.n3;
  const int P = g.n2 * n3;
  const int H = a.H, W = a.W;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  float* tiles = reinterpret_cast<float*>(smem + 128);
  const int pb = (int)S->iscalars[I_PBUF];
  const float* pin = pb ? a.pbuf1 : a.pbuf0;     // p_old (K1)
  float* pout = pb ? a.pbuf0 : a.pbuf1;          // p written by K1, staged by K2
  const float* f0 = MODE == 1 ? a.r : pout;
  const float* f1 = pin;
  const float beta = (float)S->scalars[D_BETA];
  const float alpha = (float)S->scalars[D_ALPHA];
  DotAcc<float> acc;
  bool ok = true;
  int waited_hi = 0, ifirst = 0;

  for (int item = blockIdx.x; item < a.items && ok; item += gridDim.x) {
    const int pb0 = (item % a.nx) * CF_TP;
    const int i0 = (item / a.nx) * CF_CHUNK, i1 = min(n1, i0 + CF_CHUNK);
    const int t0 = pb0 - H;
    const int lo = max(0, t0), hi = min(P, t0 + W);
    const int soff = lo - t0, len = hi - lo;
    const uint32_t nbytes = (uint32_t)len * 4u;
    ifirst = max(0, i0 - 1);
    const int ilast = min(n1 - 1, i1);

    __syncthreads();   // the previous item is done with every slot
    // Tile parts no copy writes (outside the box's plane) stay zero.
    for (int b = 0; b < CF_NB * NF; b++) {
      float* t = tiles + b * W;
      for (int q = threadIdx.x; q < W; q += CF_THREADS)
        if (q < soff || q >= soff + len) t[q] = 0.f;
    }
    if (threadIdx.x == 0) {
      for (int b = 0; b < CF_NB; b++) {
        if (item != (int)blockIdx.x) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&mbar[b])) : "memory");
        mbar_init(&mbar[b], 1);
      }
      fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int q) {
      const int b = (q - ifirst) % CF_NB;
      mbar_expect_tx(&mbar[b], nbytes * NF);
      bulk_g2s(tiles + (b * NF + 0) * W + soff, f0 + (size_t)q * P + lo, nbytes, &mbar[b]);
      if (NF == 2) bulk_g2s(tiles + (b * NF + 1) * W + soff, f1 + (size_t)q * P + lo, nbytes, &mbar[b]);
    };
    if (threadIdx.x == 0) {
      int q = ifirst;
      for (; q <= ilast && q < ifirst + CF_NB; q++) issue(q);
      issued_hi = q - 1;
    }
    waited_hi = ifirst - 1;

    // This thread's four consecutive positions.
    const int pbase = pb0 + 4 * threadIdx.x;
    const bool active = pbase < P;   // P % 4 == 0: all four or none
    int j0 = 0, k0 = 0;
    if (active) { j0 = pbase / n3; k0 = pbase - j0 * n3; }
    const int s = pbase - t0;   // tile index of the first position
    // register prefetch of the plain (unstaged) inputs of plane i0
    uchar4 kb4 = make_uchar4(0, 0, 0, 0);
    float4 e4 = make_float4(0.f, 0.f, 0.f, 0.f), r4 = e4;
    if (active) {
      const int c = i0 * P + pbase;
      kb4 = *reinterpret_cast<const uchar4*>(g.kind + c);
      if (MODE == 2) { e4 = *reinterpret_cast<const float4*>(a.e + c); r4 = *reinterpret_cast<const float4*>(a.r + c); }
    }
    bool wait_ok = true;
    for (int i = i0; i < i1; i++) {
      const int qa = (i == i0) ? max(i - 1, ifirst) : i + 1, qb = min(i + 1, ilast);
      for (int q = qa; q <= qb; q++) {
        wait_ok = mbar_wait_bounded(&mbar[(q - ifirst) % CF_NB], ((q - ifirst) / CF_NB) & 1) && wait_ok;
        waited_hi = q;
      }
      // next plane's plain inputs, in flight while this plane is computed
      uchar4 kbn = kb4;
      float4 en = e4, rn = r4;
      if (active && i + 1 < i1) {
        const int cn = (i + 1) * P + pbase;
        kbn = *reinterpret_cast<const uchar4*>(g.kind + cn);
        if (MODE == 2) { en = *reinterpret_cast<const float4*>(a.e + cn); rn = *reinterpret_cast<const float4*>(a.r + cn); }
      }
      const int bc = (i - ifirst) % CF_NB;
      const int bm = i - 1 >= ifirst ? (i - 1 - ifirst) % CF_NB : bc;
      const int bp = i + 1 <= ilast ? (i + 1 - ifirst) % CF_NB : bc;
      const float* Rm = tiles + (bm * NF) * W;
      const float* Rc = tiles + (bc * NF) * W;
      const float* Rp = tiles + (bp * NF) * W;
      const float* Om = tiles + (bm * NF + 1) * W;
      const float* Oc = tiles + (bc * NF + 1) * W;
      const float* Op = tiles + (bp * NF + 1) * W;
      if (active && wait_ok) {
        const int c = i * P + pbase;
        const float cxm = UNI ? a.ucx : g.cxm[i], cxp = UNI ? a.ucx : g.cxp[i];
        auto V = [&](const float* R, const float* O, int t) -> float {
          return MODE == 1 ? fmaf(beta, O[t], R[t]) : R[t];
        };
        float4 xc4 = *reinterpret_cast<const float4*>(Rc + s);
        float4 xm4 = *reinterpret_cast<const float4*>(Rm + s);
        float4 xp4 = *reinterpret_cast<const float4*>(Rp + s);
        if (MODE == 1) {
          const float4 oc4 = *reinterpret_cast<const float4*>(Oc + s);
          const float4 om4 = *reinterpret_cast<const float4*>(Om + s);
          const float4 op4 = *reinterpret_cast<const float4*>(Op + s);
          xc4.x = fmaf(beta, oc4.x, xc4.x); xc4.y = fmaf(beta, oc4.y, xc4.y);
          xc4.z = fmaf(beta, oc4.z, xc4.z); xc4.w = fmaf(beta, oc4.w, xc4.w);
          xm4.x = fmaf(beta, om4.x, xm4.x); xm4.y = fmaf(beta, om4.y, xm4.y);
          xm4.z = fmaf(beta, om4.z, xm4.z); xm4.w = fmaf(beta, om4.w, xm4.w);
          xp4.x = fmaf(beta, op4.x, xp4.x); xp4.y = fmaf(beta, op4.y, xp4.y);
          xp4.z = fmaf(beta, op4.z, xp4.z); xp4.w = fmaf(beta, op4.w, xp4.w);
        }
        const float xl = V(Rc, Oc, s - 1), xr = V(Rc, Oc, s + 4);
        const float xcv[6] = {xl, xc4.x, xc4.y, xc4.z, xc4.w, xr};
        const float xmv[4] = {xm4.x, xm4.y, xm4.z, xm4.w};
        const float xpv[4] = {xp4.x, xp4.y, xp4.z, xp4.w};
        const uint8_t kbs[4] = {kb4.x, kb4.y, kb4.z, kb4.w};
        float out[4];
        int j = j0, k = k0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float xjm = V(Rc, Oc, s + u - n3), xjp = V(Rc, Oc, s + u + n3);
          const float cym = UNI ? a.ucy : g.cym[j], cyp = UNI ? a.ucy : g.cyp[j];
          const float czm = UNI ? a.ucz : g.czm[k], czp = UNI ? a.ucz : g.czp[k];
          float v = lap_row_f(kbs[u], cxm, cxp, cym, cyp, czm, czp, xmv[u], xcv[u + 1], xpv[u],
                              xjm, xjp, xcv[u], xcv[u + 2]);
          const int row = row_of(kbs[u]);
          if (row > ROW_ACTUAL) {
            SmemAcc<MODE> A{Rm, Rc, Rp, Om, Oc, Op, beta, s + u, n3};
            v = staged_boundary_row<MODE>(&g, A, i, j, k, c + u, row);
          }
          out[u] = row == ROW_NONE ? 0.f : v;
          if (++k == n3) { k = 0; j++; }
        }
        if (MODE == 1) {
          *reinterpret_cast<float4*>(pout + c) = xc4;
          acc.add(xc4.x, out[0]); acc.add(xc4.y, out[1]); acc.add(xc4.z, out[2]); acc.add(xc4.w, out[3]);
        } else {
          e4.x = fmaf(alpha, xc4.x, e4.x); e4.y = fmaf(alpha, xc4.y, e4.y);
          e4.z = fmaf(alpha, xc4.z, e4.z); e4.w = fmaf(alpha, xc4.w, e4.w);
          r4.x = fmaf(-alpha, out[0], r4.x); r4.y = fmaf(-alpha, out[1], r4.y);
          r4.z = fmaf(-alpha, out[2], r4.z); r4.w = fmaf(-alpha, out[3], r4.w);
          *reinterpret_cast<float4*>(a.e + c) = e4;
          *reinterpret_cast<float4*>(a.r + c) = r4;
          acc.add(r4.x, r4.x); acc.add(r4.y, r4.y); acc.add(r4.z, r4.z); acc.add(r4.w, r4.w);
        }
      }
      kb4 = kbn; e4 = en; r4 = rn;
      // every thread is done with plane i-1's slot; a timed-out wait anywhere
      // stops the whole block
      if (__syncthreads_or(!wait_ok)) { ok = false; break; }
      if (threadIdx.x == 0 && i - 1 >= ifirst && i - 1 + CF_NB <= ilast) {
        fence_proxy_async();
        issue(i - 1 + CF_NB);
        issued_hi = i - 1 + CF_NB;
      }
    }
  }
  if (!ok) {
    // A copy did not land in time: record it, let every copy still in flight
    // finish (bounded) so none writes into released shared memory, and leave.
    if (threadIdx.x == 0) {
      atomicExch((unsigned long long*)&S->iscalars[I_ERR], 1ull);
      for (int q = waited_hi + 1; q <= issued_hi; q++)
        mbar_wait_bounded(&mbar[(q - ifirst) % CF_NB], ((q - ifirst) / CF_NB) & 1);
      S->iscalars[I_DONE] = 1;
      S->iscalars[I_STATUS] = XF_ERR_CUDA;
    }
    __syncthreads();
    return;
  }
  double vals[1] = {acc.value()};
  const int slot = MODE == 1 ? SL_A : SL_B;
  if (publish_partials<1>(S, slot, vals, sh, &last)) {
    double t = finish_partials(S, slot, sh);
    if (threadIdx.x == 0) {
      S->scalars[slot] = t;
      S->tickets[slot] = 0;
      control_step(S, MODE == 1 ? CTL_CG_ALPHA : CTL_CG_BETA_FLIP);
    }
  }
}

static size_t cgf_smem(int W, int NF) { return 128 + (size_t)CF_NB * NF * W * sizeof(float); }

static int cgf_halo(const xf_grid* g) { return ((g->n3 + 1) + 3) / 4 * 4; }

// True when the staged fused iteration applies to this grid.
bool xf_cgf_supported(const xf_grid* g) {
  const int64_t P = (int64_t)g->n2 * g->n3;
  if (P % 4 != 0) return false;
  return cgf_smem(CF_TP + 2 * cgf_halo(g), 2) <= 200 * 1024;
}

static int g_cgf_grid[2] = {0, 0};

// Outside any stream capture: allow the large dynamic shared-memory tiles and
// size the persistent grids to the resident-block count.
template <bool UNI>
static int cgf_prepare_t(xf_ctx* ctx, int W) {
  XF_CUDA(ctx, cudaFuncSetAttribute(k_cgf<1, UNI>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  XF_CUDA(ctx, cudaFuncSetAttribute(k_cgf<2, UNI>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  int b1 = 0, b2 = 0;
  XF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_cgf<1, UNI>, CF_THREADS, cgf_smem(W, 2)));
  XF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_cgf<2, UNI>, CF_THREADS, cgf_smem(W, 1)));
  g_cgf_grid[0] = (b1 > 0 ? b1 : 1) * ctx->sm_count;
  g_cgf_grid[1] = (b2 > 0 ? b2 : 1) * ctx->sm_count;
  return XF_OK;
}

int xf_cgf_prepare(xf_ctx* ctx, const xf_grid* g) {
  const int W = CF_TP + 2 * cgf_halo(g);
  return g->uniform ? cgf_prepare_t<true>(ctx, W) : cgf_prepare_t<false>(ctx, W);
}

// One fused iteration (K1 then K2).  r is updated in place; e accumulates the
// correction; p0/p1 are the direction ping-pong buffers selected on the device.
void xf_cgf_iteration(const xf_op* op, float* r, float* e, float* p0, float* p1) {
  const xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  CgfArgs a;
  a.g = make_stencil_grid<float>(g, nullptr);
  a.r = r; a.pbuf0 = p0; a.pbuf1 = p1; a.e = e; a.S = ctx->scratch;
  a.H = cgf_halo(g);
  a.W = CF_TP + 2 * a.H;
  const int P = g->n2 * g->n3;
  a.nx = (P + CF_TP - 1) / CF_TP;
  a.items = a.nx * ((g->n1 + CF_CHUNK - 1) / CF_CHUNK);
  a.ucx = (float)g->ucx; a.ucy = (float)g->ucy; a.ucz = (float)g->ucz;
  const int grid1 = min(a.items, min(g_cgf_grid[0], RED_MAX_BLOCKS));
  const int grid2 = min(a.items, min(g_cgf_grid[1], RED_MAX_BLOCKS));
  if (g->uniform) {
    k_cgf<1, true><<<grid1, CF_THREADS, cgf_smem(a.W, 2), ctx->stream>>>(a);
    k_cgf<2, true><<<grid2, CF_THREADS, cgf_smem(a.W, 1), ctx->stream>>>(a);
  } else {
    k_cgf<1, false><<<grid1, CF_THREADS, cgf_smem(a.W, 2), ctx->stream>>>(a);
    k_cgf<2, false><<<grid2, CF_THREADS, cgf_smem(a.W, 1), ctx->stream>>>(a);
  }
}
