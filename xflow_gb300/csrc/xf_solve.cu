// Krylov solvers of TSLAE (XSLAE.cpp) on the GPU.
//
//  XF_CG            Hestenes-Stiefel CG, relative tolerance; FP64, or mixed
//                   (FP32 matvec / vectors, FP64 dots and scalars, true FP64
//                   residual replacement every `replace_every` iterations and
//                   at convergence - reliable updates).
//  XF_CG_REFERENCE  TSLAE::SolveByConjugateGradients (three-term form).
//  XF_BICGSTAB      TSLAE::SolveByBiConjugateGradientsStab.
//  XF_MINRES        TSLAE::SolveByMinimalResiduals.
//
// Every iteration is a short chain of kernels whose scalar recurrences run on
// the device (xf_control.cuh); chunks of iterations are captured in a CUDA
// graph and the host only polls the device "done" flag between chunks.
#include <math.h>
#include <stdlib.h>

#include <functional>
#include <utility>
#include <vector>

#include "xf_control.cuh"
#include "xf_stencil.cuh"

void xf_mv64(const xf_op* op, const MvReq<double>& q);
void xf_mv32(const xf_op* op, const MvReq<float>& q);
void xf_cg_q64(const xf_op* op, const double* p, double* q);
void xf_cg_q32(const xf_op* op, const float* p, float* q);
void xf_cg_res64(const xf_op* op, const double* x, const double* b, float* r32, int slot, int ctl);
bool xf_cg_pq_supported(const xf_grid* g);
void xf_cg_pq32(const xf_op* op, const float* r, float* pb0, float* pb1, float* q);
bool xf_cg_pqb_supported(const xf_grid* g);
void xf_cg_pqb_launch(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int ctl);
bool xf_cg_poly_supported(const xf_grid* g);
void xf_cg_poly_launch(const xf_op* op, const float* r, float* z, const float coeffs[3]);
void xf_cg_polyr_launch(const xf_op* op, const float* r, float* r_out, const float* q, const float* pa,
                        const float* pb, float* e, float* z, const float coeffs[3]);
void xf_cheb2_coeffs(double lmax, double ratio, float out[3]);
bool xf_cheb4_factors(double lmax, double ratio, float f1[3], float f2[3]);
bool xf_cheb_factors(double lmax, double ratio, int deg, float (*f)[3]);
bool xf_tl_prolong_ay_supported(const xf_grid* g);
void xf_tl_prolong_ay(const xf_op* op, const float* zc, int c2, int c3, float* y, float* ay, int slot);
void xf_cg_poly_tl_launch(const xf_op* op, bool first, bool last, const float* in, const float* q, float* out,
                          const float coeffs[3], int s_yay, int s_yr, const float* y, float tsc, float* z2,
                          const float* r, const float* qw, int s_zr, int s_zq);
void xf_cg_poly_first_launch(const xf_op* op, const float* r, float* w, const float coeffs[3], const float* q,
                             const float* pa, const float* pb, float* e, float* r_out);
void xf_cg_poly_second_launch(const xf_op* op, const float* w, const float* r, float* z, const float coeffs[3]);
void xf_cg_pq32_variant(const xf_op* op, const float* r, float* pb0, float* pb1, float* q, int variant);
bool xf_cg_pqt_supported(const xf_grid* g);
int xf_op_ready(const xf_op* op);
int xf_op_jacobi(const xf_op* op, const double** dinv);

#define GUARD_DONE(S) \
  if ((S)->iscalars[I_DONE]) return;

// ---------------------------------------------------------------------------
// x += alpha p; r -= alpha q; (r, r) -> SL_B; control CTL_CG_BETA.  Unmasked:
// the solver keeps p, q, r at zero on inactive cells.
// 16-byte vector view of T (cudaMalloc'd boxes are 256-byte aligned).
template <typename T> struct V16;
template <> struct V16<float> { typedef float4 type; };
template <> struct V16<double> { typedef double2 type; };

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_cg_xr(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                                       const T* __restrict__ q, int64_t n, DevScratch* S,
                                                       const T* __restrict__ p_alt = nullptr, int ctl = CTL_CG_BETA) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (S->iscalars[I_DONE] || S->iscalars[I_PAUSE]) return;
  // fused direction update: p ping-pongs and I_PBUF names the current buffer
  if (p_alt && S->iscalars[I_PBUF]) p = p_alt;
  typedef typename V16<T>::type VT;
  constexpr int L = 16 / sizeof(T);
  const T alpha = (T)S->scalars[D_ALPHA];
  DotAcc<T> acc;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nv = n / L;
  for (int64_t v = tid; v < nv; v += stride) {
    VT xv = reinterpret_cast<const VT*>(x)[v], rv = reinterpret_cast<const VT*>(r)[v];
    const VT pv = reinterpret_cast<const VT*>(p)[v], qv = reinterpret_cast<const VT*>(q)[v];
    T* xa = reinterpret_cast<T*>(&xv);
    T* ra = reinterpret_cast<T*>(&rv);
    const T* pa = reinterpret_cast<const T*>(&pv);
    const T* qa = reinterpret_cast<const T*>(&qv);
#pragma unroll
    for (int l = 0; l < L; l++) {
      xa[l] = fma(alpha, pa[l], xa[l]);
      ra[l] = fma(-alpha, qa[l], ra[l]);
      acc.add(ra[l], ra[l]);
    }
    reinterpret_cast<VT*>(x)[v] = xv;
    reinterpret_cast<VT*>(r)[v] = rv;
  }
  for (int64_t c = nv * L + tid; c < n; c += stride) {
    x[c] = fma(alpha, p[c], x[c]);
    T rv = fma(-alpha, q[c], r[c]);
    r[c] = rv;
    acc.add(rv, rv);
  }
  if (publish_acc<T>(S, SL_B, SL_B, acc, sh, &last)) {
    double t = finish_partials(S, SL_B, sh);
    if (threadIdx.x == 0) {
      S->scalars[SL_B] = t;
      S->tickets[SL_B] = 0;
      control_step(S, ctl);
    }
  }
}

// One wave of resident blocks for the x/r update (its grid-stride loop then
// has no partial second wave), capped by the reduction table.
template <typename T>
static int xr_blocks(xf_ctx* ctx, int64_t n) {
  static int per_sm[2] = {0, 0};
  int& r = per_sm[sizeof(T) == 8];
  if (!r && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_cg_xr<T>, RED_THREADS, 0) != cudaSuccess || r < 1))
    r = 1;
  int64_t b = (int64_t)ctx->sm_count * r;
  const int64_t need = (n + RED_THREADS - 1) / RED_THREADS;
  if (b > need) b = need;
  if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
  return (int)(b < 1 ? 1 : b);
}

// p = r + beta p.  `after_replace`: the step that follows a true-residual
// replacement runs even while the inner recursion is paused.
template <typename T>
__global__ void k_cg_p(T* __restrict__ p, const T* __restrict__ r, int64_t n, DevScratch* S, int after_replace) {
  if (S->iscalars[I_DONE] || (!after_replace && S->iscalars[I_PAUSE])) return;
  typedef typename V16<T>::type VT;
  constexpr int L = 16 / sizeof(T);
  const T beta = (T)S->scalars[D_BETA];
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nv = n / L;
  for (int64_t v = tid; v < nv; v += stride) {
    VT pv = reinterpret_cast<const VT*>(p)[v];
    const VT rv = reinterpret_cast<const VT*>(r)[v];
    T* pa = reinterpret_cast<T*>(&pv);
    const T* ra = reinterpret_cast<const T*>(&rv);
#pragma unroll
    for (int l = 0; l < L; l++) pa[l] = fma(beta, pa[l], ra[l]);
    reinterpret_cast<VT*>(p)[v] = pv;
  }
  for (int64_t c = nv * L + tid; c < n; c += stride) p[c] = fma(beta, p[c], r[c]);
}

// Mixed: fold the FP32 correction into the FP64 iterate (x += e; e = 0).
// mode 0: always; mode 2: unless the solve is done.
__global__ void k_fold(double* __restrict__ x, float* __restrict__ e, int64_t n, DevScratch* S, int mode) {
  if (mode == 2 && S->iscalars[I_DONE]) return;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nv = n / 2;
  for (int64_t v = tid; v < nv; v += stride) {
    double2 xv = reinterpret_cast<const double2*>(x)[v];
    const float2 ev = reinterpret_cast<const float2*>(e)[v];
    xv.x += (double)ev.x;
    xv.y += (double)ev.y;
    reinterpret_cast<double2*>(x)[v] = xv;
    reinterpret_cast<float2*>(e)[v] = make_float2(0.f, 0.f);
  }
  for (int64_t c = nv * 2 + tid; c < n; c += stride) {
    x[c] += (double)e[c];
    e[c] = 0.f;
  }
}

// Masked FP64 dot with a control step.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot_ctl(const T* __restrict__ a, const T* __restrict__ b,
                                                         const uint8_t* __restrict__ m, int64_t n, DevScratch* S,
                                                         int slot, int ctl, int guard) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (guard && S->iscalars[I_DONE]) return;
  double acc = 0.0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    if (m[c]) acc += (double)a[c] * (double)b[c];
  double v[1] = {acc};
  if (publish_partials<1>(S, slot, v, sh, &last)) {
    double t = finish_partials(S, slot, sh);
    if (threadIdx.x == 0) {
      S->scalars[slot] = t;
      S->tickets[slot] = 0;
      control_step(S, ctl);
    }
  }
}

// ---- reference-semantics helpers (masked, device scalars) -------------------
// z = a - d[ci] * s   (TSLAE CG start: xk |= xk_1 - tauk*rk_1)
__global__ void k_axmy_dev(double* __restrict__ z, const double* __restrict__ a, const double* __restrict__ s,
                           const uint8_t* __restrict__ m, int64_t n, DevScratch* S, int ci) {
  GUARD_DONE(S);
  const double c1 = S->scalars[ci];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (m[i]) z[i] = a[i] - c1 * s[i];
}

// XSLAE.cpp:124-134: result = alfak1*xk + (1-alfak1)*xk_1; result -= (tauk1*alfak1)*rk;
// xk_1 = xk; xk = result.
__global__ void k_rcg_update(double* __restrict__ xk, double* __restrict__ xk_1, const double* __restrict__ rk,
                             const uint8_t* __restrict__ m, int64_t n, DevScratch* S) {
  GUARD_DONE(S);
  const double c1 = S->scalars[D_C1], c2 = S->scalars[D_C2], c3 = S->scalars[D_C3];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!m[i]) continue;
    double res = c1 * xk[i] + c2 * xk_1[i];
    res = res - c3 * rk[i];
    xk_1[i] = xk[i];
    xk[i] = res;
  }
}

// BiCGStab's vector steps come in two forms: the reference's steps (EXACT,
// for XF_EXACT solves) and FMA forms with fewer FP64 operations (GB300's FP64
// rate, not memory, bounds these passes).
// XSLAE.cpp:723-727: Pn1 = Rn + bn*(Pn - wn*Vn).  With a Jacobi
// preconditioner (dinv non-null) also Ph = dinv Pn1, the vector A sees.
template <bool EXACT>
__global__ void k_bcgs_p(double* __restrict__ Pn1, const double* __restrict__ Rn, const double* __restrict__ Pn,
                         const double* __restrict__ Vn, const uint8_t* __restrict__ m, int64_t n, DevScratch* S,
                         const double* __restrict__ dinv, double* __restrict__ Ph) {
  GUARD_DONE(S);
  const double wn = S->scalars[D_WN], bn = S->scalars[D_BN];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!m[i]) continue;
    double p;
    if (EXACT) {
      double t = wn * Vn[i];
      t = Pn[i] - t;
      t = bn * t;
      p = Rn[i] + t;
    } else {
      p = fma(bn, fma(-wn, Vn[i], Pn[i]), Rn[i]);
    }
    Pn1[i] = p;
    if (dinv) Ph[i] = dinv[i] * p;
  }
}

// XSLAE.cpp:732-733: Sn = Rn - an*Vn (and Sh = dinv Sn).
template <bool EXACT>
__global__ void k_bcgs_s(double* __restrict__ Sn, const double* __restrict__ Rn, const double* __restrict__ Vn,
                         const uint8_t* __restrict__ m, int64_t n, DevScratch* S, const double* __restrict__ dinv,
                         double* __restrict__ Sh) {
  GUARD_DONE(S);
  const double an = S->scalars[D_AN];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!m[i]) continue;
    const double s = EXACT ? Rn[i] - an * Vn[i] : fma(-an, Vn[i], Rn[i]);
    Sn[i] = s;
    if (dinv) Sh[i] = dinv[i] * s;
  }
}

__device__ __forceinline__ double max_nan_skip(double a, double b) { return b > a ? b : a; }
__device__ double block_max(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max_nan_skip(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max_nan_skip(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// XSLAE.cpp:738-749: Un += an*Pn1 + wn*Sn; Rn = Sn - wn*Tn; Pn = Pn1 (no
// copy when Pn is null: the caller alternates the two direction buffers);
// then ||Rn||_inf (NaN never wins, XSpace.cpp:3455-3463) with control `ctl`.
// With a Jacobi preconditioner Un moves along the preconditioned vectors:
// Un += an*Ph + wn*Sh (Xp, Xs; otherwise Pn1 and Sn).
template <bool EXACT>
__global__ void __launch_bounds__(RED_THREADS) k_bcgs_end(double* __restrict__ Un, double* __restrict__ Rn,
                                                          double* __restrict__ Pn, const double* __restrict__ Pn1,
                                                          const double* __restrict__ Sn, const double* __restrict__ Tn,
                                                          const uint8_t* __restrict__ m, int64_t n, DevScratch* S,
                                                          int update, int ctl, const double* __restrict__ Xp = nullptr,
                                                          const double* __restrict__ Xs = nullptr) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (update) GUARD_DONE(S);
  const double an = S->scalars[D_AN], wn = S->scalars[D_WN];
  double best = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!m[i]) continue;
    double r;
    if (update && EXACT) {
      double tmp1 = an * (Xp ? Xp[i] : Pn1[i]);
      double tmp2 = tmp1 + wn * (Xs ? Xs[i] : Sn[i]);
      Un[i] = Un[i] + tmp2;
      double t = wn * Tn[i];
      r = Sn[i] - t;
      Rn[i] = r;
      if (Pn) Pn[i] = Pn1[i];
    } else if (update) {
      const double sn = Sn[i];
      Un[i] = Un[i] + fma(an, Xp ? Xp[i] : Pn1[i], wn * (Xs ? Xs[i] : sn));
      r = fma(-wn, Tn[i], sn);
      Rn[i] = r;
      if (Pn) Pn[i] = Pn1[i];
    } else {
      r = Rn[i];
    }
    best = max_nan_skip(best, fabs(r));
  }
  double bm = block_max(best, sh);
  if (threadIdx.x == 0) {
    S->partials[SL_D][blockIdx.x] = bm;
    __threadfence();
    unsigned int t = atomicAdd(&S->tickets[SL_D], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double q = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) q = max_nan_skip(q, __ldcg(&S->partials[SL_D][b]));
  q = block_max(q, sh);
  if (threadIdx.x == 0) {
    S->scalars[SL_D] = q;
    S->tickets[SL_D] = 0;
    control_step(S, ctl);
  }
}

// XSLAE.cpp:387: xk = xk + alfa*rk.
__global__ void k_mr_x(double* __restrict__ xk, const double* __restrict__ rk, const uint8_t* __restrict__ m, int64_t n,
                       DevScratch* S) {
  GUARD_DONE(S);
  const double alfa = S->scalars[D_ALFA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (m[i]) xk[i] = xk[i] + alfa * rk[i];
}

// ---- TSLAE::SolveByBiConjugateGradients (XSLAE.cpp:159-348) -------------
// Start (:169-189): xk = 0 whatever x held, rk = A(0) - b = -b, rt = -rk = b,
// rk = rt, pk = rk, pt = rt; everything off the active set stays as it is.
__global__ void k_bicg_init(double* __restrict__ x, double* __restrict__ rk, double* __restrict__ rt,
                            double* __restrict__ pk, double* __restrict__ pt, const double* __restrict__ b,
                            const uint8_t* __restrict__ m, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (m[i]) {
      const double r = (0.0 - b[i]) * (-1);
      x[i] = 0;
      rk[i] = r; rt[i] = r; pk[i] = r; pt[i] = r;
    }
}

// :237-251: xk += alpha pk; rk = (-alpha) A pk + rk; rt = (-alpha) A^T pt + rt;
// then (rk, rt) -> SL_C and (rk, rk) -> SL_C+1 with the beta step.
__global__ void __launch_bounds__(RED_THREADS) k_bicg_update(double* __restrict__ x, double* __restrict__ rk,
                                                             double* __restrict__ rt, const double* __restrict__ pk,
                                                             const double* __restrict__ Ap,
                                                             const double* __restrict__ Atp,
                                                             const uint8_t* __restrict__ m, int64_t n, DevScratch* S) {
  __shared__ double sh[32];
  __shared__ bool last;
  GUARD_DONE(S);
  const double alpha = S->scalars[D_ALPHA];
  DotAcc<double> a1, a2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (m[i]) {
      x[i] = x[i] + alpha * pk[i];
      const double r = (-alpha) * Ap[i] + rk[i];
      const double t = (-alpha) * Atp[i] + rt[i];
      rk[i] = r;
      rt[i] = t;
      a1.add(r, t);
      a2.add(r, r);
    }
  double v[2] = {a1.value(), a2.value()};
  if (publish_partials<2>(S, SL_C, v, sh, &last)) {
    double t1 = finish_partials(S, SL_C, sh);
    double t2 = finish_partials(S, SL_C + 1, sh);
    if (threadIdx.x == 0) {
      S->scalars[SL_C] = t1;
      S->scalars[SL_C + 1] = t2;
      S->tickets[SL_C] = 0;
      control_step(S, CTL_BICG_BETA);
    }
  }
}

// :282-291: pk = rk + beta pk; pt = rt + beta pt.
__global__ void k_bicg_p(double* __restrict__ pk, double* __restrict__ pt, const double* __restrict__ rk,
                         const double* __restrict__ rt, const uint8_t* __restrict__ m, int64_t n, DevScratch* S) {
  GUARD_DONE(S);
  const double beta = S->scalars[D_BETA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (m[i]) {
      pk[i] = rk[i] + beta * pk[i];
      pt[i] = rt[i] + beta * pt[i];
    }
}

__global__ void k_reset_state(DevScratch* S, double rtol2, double eps, long long maxit, long long repevery, long long mixed) {
  for (int q = 0; q < 16; q++) S->iscalars[q] = 0;
  S->iscalars[I_STATUS] = XF_OK;
  S->iscalars[I_MAXIT] = maxit;
  S->iscalars[I_REPEVERY] = repevery;
  S->iscalars[I_MIXED] = mixed;
  S->scalars[D_RTOL2] = rtol2;
  S->scalars[D_EPS] = eps;
  for (int q = 0; q < NUM_SLOTS; q++) S->tickets[q] = 0;
}

// ---------------------------------------------------------------------------
// Device buffers owned for the duration of one solve.
struct Bufs {
  xf_ctx* ctx;
  std::vector<void*> ptrs;
  explicit Bufs(xf_ctx* c) : ctx(c) {}
  template <typename T>
  T* get(int64_t n, bool zero = true) {
    void* p = nullptr;
    if (cudaMallocAsync(&p, n * sizeof(T), ctx->stream) != cudaSuccess) return nullptr;
    if (zero) cudaMemsetAsync(p, 0, n * sizeof(T), ctx->stream);
    ptrs.push_back(p);
    return (T*)p;
  }
  ~Bufs() {
    for (void* p : ptrs) cudaFreeAsync(p, ctx->stream);
  }
};

struct HostState { long long done, status, it, repl, kernels; };

static int read_state(xf_ctx* ctx, HostState* hs) {
  long long tmp[4];
  XF_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, ctx->scratch->iscalars, 4 * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  memcpy(tmp, ctx->host_scalars, sizeof(tmp));
  hs->done = tmp[0]; hs->status = tmp[1]; hs->it = tmp[2]; hs->repl = tmp[3];
  return XF_OK;
}

// Runs `iter` (which enqueues one iteration) until the device flags done:
// chunks of `chunk` iterations are captured once into a CUDA graph; the state
// of chunk k is read while chunk k+1 is already queued.
static int run_loop(xf_ctx* ctx, const std::function<void(int)>& iter, int chunk, int maxit, HostState* hs) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  XF_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int c = 0; c < chunk; c++) iter(c);
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (ce != cudaSuccess) return xf_fail(ctx, XF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return xf_fail(ctx, XF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
  }
  long long* hbuf = (long long*)(ctx->host_scalars + 128);  // two 4-entry state slots
  cudaEvent_t ev[2];
  cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  const int max_chunks = maxit / chunk + 3;
  int st = XF_OK;
  int launched = 0;
  size_t nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nodes);
  bool done = false;
  // keep two chunks in flight
  for (int k = 0; k < max_chunks && !done; k++) {
    ce = cudaGraphLaunch(exec, ctx->stream);
    if (ce != cudaSuccess) { st = xf_fail(ctx, XF_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce)); break; }
    cudaMemcpyAsync(hbuf + 4 * (k & 1), ctx->scratch->iscalars, 4 * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
    cudaEventRecord(ev[k & 1], ctx->stream);
    launched++;
    if (k >= 1) {
      cudaEventSynchronize(ev[(k - 1) & 1]);
      if (hbuf[4 * ((k - 1) & 1)]) done = true;
    }
  }
  cudaStreamSynchronize(ctx->stream);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  if (st) return st;
  XF_CUDA(ctx, cudaGetLastError());
  long long kernels = hs->kernels + (long long)launched * (long long)nodes;
  int rs = read_state(ctx, hs);
  hs->kernels = kernels;
  return rs;
}

static double read_scalar(xf_ctx* ctx, int idx) {
  cudaMemcpyAsync(ctx->host_scalars, &ctx->scratch->scalars[idx], 8, cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return ctx->host_scalars[0];
}

// True relative residual ||b - A x||_2 / ||b||_2 in FP64 (fast rows).
static int true_residual(const xf_op* op, const double* x, const double* b, double* tmp, double* rel, double* bbout) {
  xf_ctx* ctx = op->g->ctx;
  DevScratch* S = ctx->scratch;
  k_dot_ctl<double><<<red_blocks(ctx, op->g->ncell), RED_THREADS, 0, ctx->stream>>>(b, b, op->g->smask, op->g->ncell, S, SL_B, CTL_NONE, 0);
  MvReq<double> q;
  q.x = x; q.y = tmp; q.s = b; q.sign = -1; q.neg = 1; q.zero_inactive = 1; q.dot_self = 1; q.slot = SL_C;
  xf_mv64(op, q);
  XF_CUDA(ctx, cudaGetLastError());
  double bb = read_scalar(ctx, SL_B), rr = read_scalar(ctx, SL_C + 1);
  *rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  if (bbout) *bbout = bb;
  return XF_OK;
}

// ---------------------------------------------------------------------------
static int solve_cg(xf_op* op, const xf_solve_opts& o, xf_vec* xv, const xf_vec* bv, xf_solve_stats* st) {
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  DevScratch* S = ctx->scratch;
  const int64_t n = g->ncell;
  const bool mixed = o.precision == XF_PREC_MIXED;
  double* x = (double*)xv->data;
  const double* b = (const double*)bv->data;
  Bufs B(ctx);
  const int rb = red_blocks(ctx, n), eb = grid_blocks(ctx, n, 256);
  const int xb32 = xr_blocks<float>(ctx, n), xb64 = xr_blocks<double>(ctx, n);
  int total_it = 0, total_repl = 0;
  HostState hs = {0, 0, 0, 0, 0};
  double rel = 0;
  double *r = nullptr, *p = nullptr, *q = nullptr;
  float *e32 = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr, *p32b = nullptr, *z32 = nullptr;
  float *r32b = nullptr, *w32 = nullptr, *w32b = nullptr;
  const int cheb_deg = o.reserved[2] > 0 ? o.reserved[2] : 8;
  const bool cheb = o.precond == XF_PRECOND_CHEB;
  if (cheb && (cheb_deg < 2 || cheb_deg > 12 || cheb_deg % 2))
    return xf_fail(ctx, XF_ERR_ARG, "xf_solve: XF_PRECOND_CHEB degree (opts.reserved[2]) must be even, 2 to 12");
  if (cheb && (!mixed || op->kind != XF_OP_LAPLACE || !xf_cg_poly_supported(g) || !xf_cg_pqb_supported(g)))
    return xf_fail(ctx, XF_ERR_UNSUPPORTED,
                   "xf_solve: XF_PRECOND_CHEB needs mixed precision and a uniform Laplace grid without boundary rows "
                   "(n2 n3 a multiple of 4, n3 even)");
  if (!mixed) {
    r = B.get<double>(n); p = B.get<double>(n); q = B.get<double>(n);
    if (!r || !p || !q) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: cannot allocate CG vectors");
  } else {
    e32 = B.get<float>(n); r32 = B.get<float>(n); p32 = B.get<float>(n); q32 = B.get<float>(n);
    if (!e32 || !r32 || !p32 || !q32) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: cannot allocate CG vectors");
    if (op->kind == XF_OP_LAPLACE && xf_cg_pq_supported(g)) {
      p32b = B.get<float>(n);
      if (!p32b) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: cannot allocate CG vectors");
    }
    if (cheb && (!(z32 = B.get<float>(n)) || !(r32b = B.get<float>(n)) || (cheb_deg >= 4 && !(w32 = B.get<float>(n))) ||
                 (cheb_deg >= 6 && !(w32b = B.get<float>(n)))))
      return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: cannot allocate CG vectors");
  }
  double* tmp = B.get<double>(n, false);
  if (!tmp) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: cannot allocate residual");
  for (int attempt = 0; attempt < 3; attempt++) {
    k_reset_state<<<1, 1, 0, ctx->stream>>>(S, o.rtol * o.rtol, 0.0, o.maxit - total_it, o.replace_every, mixed ? 1 : 0);
    k_dot_ctl<double><<<rb, RED_THREADS, 0, ctx->stream>>>(b, b, g->smask, n, S, SL_B, CTL_NONE, 0);
    std::function<void(int)> iter;
    int chunk = o.check_every > 0 ? o.check_every : 16;
    const bool lap = op->kind == XF_OP_LAPLACE;
    if (!mixed) {
      MvReq<double> m0;
      m0.x = x; m0.y = r; m0.s = b; m0.sign = -1; m0.neg = 1; m0.zero_inactive = 1; m0.dot_self = 1; m0.slot = SL_A;
      m0.ctl = CTL_CG_INIT;
      xf_mv64(op, m0);
      XF_CUDA(ctx, cudaMemcpyAsync(p, r, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      iter = [=](int) {
        if (lap) {
          xf_cg_q64(op, p, q);
        } else {
          MvReq<double> m1;
          m1.x = p; m1.y = q; m1.w = p; m1.zero_inactive = 1; m1.slot = SL_A; m1.ctl = CTL_CG_ALPHA;
          xf_mv64(op, m1);
        }
        k_cg_xr<double><<<xb64, RED_THREADS, 0, ctx->stream>>>(x, r, p, q, n, S);
        k_cg_p<double><<<eb, 256, 0, ctx->stream>>>(p, r, n, S, 0);
      };
    } else if (cheb) {
      // Polynomially preconditioned mixed CG.  The kernels of an iteration:
      // K0 z = p(A) r with (r, z) and beta (both stencil levels in one pass),
      // K1 p' = z + beta p inside the stencil with q = A p', (p', q), alpha,
      // K2 e += alpha p', r -= alpha q with (r, r) for the stop test.  K2 and
      // the next K0 run as one fused launch (the update applied to each
      // plane as it streams in, the residual alternating between two
      // buffers), so a graph chunk of `replace_every` iterations is K0, then
      // K1 + fused K2/K0 per iteration, and a last K1 + K2 with the FP64 fold
      // and the true-residual replacement into the first buffer; the next
      // chunk's K0 continues the direction from the replaced residual.
      // Degree 2 m >= 4 (8 is the default) splits K0 into m passes, one per
      // quadratic factor of p: w = p_m(A) r (fused with K2 as above), m - 2
      // passes w <- p_k(A) w, and z = p_1(A) w with (r, z).  XF_POLYR=0 runs
      // K2 and K0 as separate launches.
      chunk = o.replace_every;
      float *e = e32, *r = r32, *pa = p32, *q = q32, *z = z32;
      float *pb = p32b, *rb = r32b, *w = w32, *wb = w32b;
      const bool fused = !(getenv("XF_POLYR") && getenv("XF_POLYR")[0] == '0');
      const int nf = cheb_deg / 2;
      const double lmax = 4.0 * (g->ucx + g->ucy + g->ucz);   // Gershgorin bound of the uniform Laplace rows
      const double ratio = o.reserved[1] > 0 ? (double)o.reserved[1] : nf > 2 ? 250.0 : nf > 1 ? 120.0 : 30.0;
      float coeffs[3], f[6][3];
      if (nf > 1) {
        if (!xf_cheb_factors(lmax, ratio, cheb_deg, f))
          return xf_fail(ctx, XF_ERR_ARG, "xf_solve: no real quadratic factors of the degree-%d polynomial (ratio %g)",
                         cheb_deg, ratio);
      } else {
        xf_cheb2_coeffs(lmax, ratio, coeffs);
      }
      // passes after the first: w <- p_k(A) w for k = m-1 .. 2 (ping-pong), then z = p_1(A) w
      auto rest = [=](float* rres) {
        float *src = w, *dst = wb;
        for (int k = nf - 2; k >= 1; k--) {
          xf_cg_poly_first_launch(op, src, dst, f[k], nullptr, nullptr, nullptr, nullptr, nullptr);
          std::swap(src, dst);
        }
        xf_cg_poly_second_launch(op, src, rres, z, f[0]);
      };
      XF_CUDA(ctx, cudaMemsetAsync(e, 0, n * 4, ctx->stream));
      XF_CUDA(ctx, cudaMemsetAsync(pa, 0, n * 4, ctx->stream));
      XF_CUDA(ctx, cudaMemsetAsync(pb, 0, n * 4, ctx->stream));
      XF_CUDA(ctx, cudaMemsetAsync(z, 0, n * 4, ctx->stream));
      xf_cg_res64(op, x, b, r, SL_A, CTL_CG_INIT);
      const int last = chunk - 1;
      iter = [=](int c) {
        // the residual before this iteration's update (fused: buffer c & 1)
        float* rc = fused && (c & 1) ? rb : r;
        if (!fused || c == 0) {
          if (nf > 1) {
            xf_cg_poly_first_launch(op, rc, w, f[nf - 1], nullptr, nullptr, nullptr, nullptr, nullptr);
            rest(rc);
          } else {
            xf_cg_poly_launch(op, rc, z, coeffs);
          }
        }
        xf_cg_pqb_launch(op, z, pa, pb, q, CTL_PCG_ALPHA_FLIP);
        if (fused && c < last) {
          float* rn = (c & 1) ? r : rb;
          if (nf > 1) {
            xf_cg_poly_first_launch(op, rc, w, f[nf - 1], q, pa, pb, e, rn);
            rest(rn);
          } else {
            xf_cg_polyr_launch(op, rc, rn, q, pa, pb, e, z, coeffs);
          }
        } else {
          k_cg_xr<float><<<xb32, RED_THREADS, 0, ctx->stream>>>(e, rc, pa, q, n, S, pb, CTL_PCG_RR);
        }
        if (c == last) {
          k_fold<<<eb, 256, 0, ctx->stream>>>(x, e, n, S, 2);
          xf_cg_res64(op, x, b, r, SL_C, CTL_PCG_REPL);
        }
      };
    } else if (lap && p32b && !(getenv("XF_PQ_FUSE") && getenv("XF_PQ_FUSE")[0] == '0')) {
      // Two kernels per iteration: K1 forms p' = r + beta p inside the
      // stencil (q = A p', (p', q), alpha; p ping-pongs between p32 and a
      // second buffer), K2 updates e and r with (r, r) and beta.  One graph
      // chunk = `replace_every` iterations; its last iteration folds the FP32
      // correction into x and replaces r by the true FP64 residual, whose
      // beta the next K1 uses.
      chunk = o.replace_every;
      float *e = e32, *r = r32, *pa = p32, *q = q32;
      float* pb = p32b;
      XF_CUDA(ctx, cudaMemsetAsync(e, 0, n * 4, ctx->stream));
      XF_CUDA(ctx, cudaMemsetAsync(pa, 0, n * 4, ctx->stream));
      XF_CUDA(ctx, cudaMemsetAsync(pb, 0, n * 4, ctx->stream));
      xf_cg_res64(op, x, b, r, SL_A, CTL_CG_INIT);
      const int last = chunk - 1;
      iter = [=](int c) {
        xf_cg_pq32(op, r, pa, pb, q);
        k_cg_xr<float><<<xb32, RED_THREADS, 0, ctx->stream>>>(e, r, pa, q, n, S, pb);
        if (c == last) {
          k_fold<<<eb, 256, 0, ctx->stream>>>(x, e, n, S, 2);
          xf_cg_res64(op, x, b, r, SL_C, CTL_MIXED_REPL);
        }
      };
    } else {
      // One graph chunk = `replace_every` iterations; its last iteration folds
      // the FP32 correction into x and replaces r by the true FP64 residual.
      chunk = o.replace_every;
      float *e = e32, *r = r32, *p = p32, *q = q32;
      XF_CUDA(ctx, cudaMemsetAsync(e, 0, n * 4, ctx->stream));
      MvReq<double> m0;
      m0.x = x; m0.y32 = r; m0.s = b; m0.sign = -1; m0.neg = 1; m0.zero_inactive = 1; m0.dot_self = 1; m0.slot = SL_A;
      m0.ctl = CTL_CG_INIT;
      xf_mv64(op, m0);
      XF_CUDA(ctx, cudaMemcpyAsync(p, r, n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
      const int last = chunk - 1;
      iter = [=](int c) {
        if (lap) {
          xf_cg_q32(op, p, q);
        } else {
          MvReq<float> m1;
          m1.x = p; m1.y = q; m1.w = p; m1.zero_inactive = 1; m1.slot = SL_A; m1.ctl = CTL_CG_ALPHA;
          xf_mv32(op, m1);
        }
        k_cg_xr<float><<<xb32, RED_THREADS, 0, ctx->stream>>>(e, r, p, q, n, S);
        if (c == last) {
          k_fold<<<eb, 256, 0, ctx->stream>>>(x, e, n, S, 2);
          if (lap) {
            xf_cg_res64(op, x, b, r, SL_C, CTL_MIXED_REPL);
          } else {
            MvReq<double> m2;
            m2.x = x; m2.y32 = r; m2.s = b; m2.sign = -1; m2.neg = 1; m2.zero_inactive = 1; m2.dot_self = 1;
            m2.slot = SL_C; m2.ctl = CTL_MIXED_REPL;
            xf_mv64(op, m2);
          }
        }
        k_cg_p<float><<<eb, 256, 0, ctx->stream>>>(p, r, n, S, c == last ? 1 : 0);
      };
    }
    XF_CUDA(ctx, cudaGetLastError());
    int rc = run_loop(ctx, iter, chunk, o.maxit - total_it, &hs);
    if (rc) return rc;
    total_it += (int)hs.it;
    total_repl += (int)hs.repl;
    hs.kernels += 3 + (mixed ? 1 : 0) + 2;
    if (mixed) {
      // fold any correction left behind by an early stop (no-op otherwise)
      k_fold<<<eb, 256, 0, ctx->stream>>>(x, e32, n, S, 0);
    }
    int r2 = true_residual(op, x, b, tmp, &rel, nullptr);
    if (r2) return r2;
    // The recursive residual can drift from the true one: restart from the
    // current iterate until the true residual meets the tolerance.
    if (hs.status != XF_OK || rel <= o.rtol || total_it >= o.maxit) break;
  }
  st->status = (int)hs.status;
  if (st->status == XF_OK && rel > o.rtol) st->status = total_it >= o.maxit ? XF_MAXIT : XF_STALL;
  st->iterations = total_it;
  st->replacements = total_repl;
  st->reserved[0] = (double)hs.kernels;
  st->rel_resid = rel;
  st->abs_resid = rel;
  return XF_OK;
}

static int solve_reference(xf_op* op, const xf_solve_opts& o, xf_vec* xv, const xf_vec* bv, xf_solve_stats* st) {
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  DevScratch* S = ctx->scratch;
  const int64_t n = g->ncell;
  const uint8_t* m = g->smask;
  double* x = (double*)xv->data;
  const double* b = (const double*)bv->data;
  const bool exact = o.exact != 0;
  Bufs B(ctx);
  const int rb = red_blocks(ctx, n), eb = grid_blocks(ctx, n, 256);
  std::function<void(int)> iter;
  bool even_chunks = false;   // the iteration alternates buffers by parity
  HostState hs = {0, 0, 0, 0, 0};
  double eps = o.atol;
  if (o.method == XF_CG_REFERENCE) {
    if (eps <= 0) eps = 1e-5;   // XSLAE.cpp:64
    k_reset_state<<<1, 1, 0, ctx->stream>>>(S, 0.0, eps, o.maxit, 1, 0);
    // xk_1 = copy(x) (whole box); rk_1 = A(xk_1) - b; (rk_1, rk_1)
    double* xk_1 = B.get<double>(n, false);
    double* rk = B.get<double>(n);
    if (!xk_1 || !rk) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    XF_CUDA(ctx, cudaMemcpyAsync(xk_1, x, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    MvReq<double> q0;
    q0.x = xk_1; q0.y = rk; q0.s = b; q0.sign = -1; q0.dot_self = 1; q0.exact = exact; q0.slot = SL_A; q0.ctl = CTL_RCG_INIT;
    xf_mv64(op, q0);
    // tauk = (rk_1,rk_1) / (A rk_1, rk_1)
    MvReq<double> q1;
    q1.x = rk; q1.w = rk; q1.exact = exact; q1.slot = SL_A; q1.ctl = CTL_RCG_TAU0;
    xf_mv64(op, q1);
    // xk = xk_1 - tauk*rk_1 (x already equals xk_1 on every cell)
    k_axmy_dev<<<eb, 256, 0, ctx->stream>>>(x, xk_1, rk, m, n, S, D_TAUK);
    // rk = A(xk) - b
    MvReq<double> q2;
    q2.x = x; q2.y = rk; q2.s = b; q2.sign = -1; q2.dot_self = 1; q2.exact = exact; q2.slot = SL_A; q2.ctl = CTL_RCG_RES0;
    xf_mv64(op, q2);
    iter = [=](int) {
      MvReq<double> a;
      a.x = rk; a.w = rk; a.exact = exact; a.slot = SL_A; a.ctl = CTL_RCG_TAU;
      xf_mv64(op, a);
      k_rcg_update<<<eb, 256, 0, ctx->stream>>>(x, xk_1, rk, m, n, S);
      MvReq<double> c;
      c.x = x; c.y = rk; c.s = b; c.sign = -1; c.dot_self = 1; c.exact = exact; c.slot = SL_A; c.ctl = CTL_RCG_RES;
      xf_mv64(op, c);
    };
  } else if (o.method == XF_BICGSTAB) {
    if (eps <= 0) eps = 1e-5;   // XSLAE.cpp:669
    k_reset_state<<<1, 1, 0, ctx->stream>>>(S, 0.0, eps, o.maxit, 1, 0);
    double *Rn = B.get<double>(n), *sRn = B.get<double>(n), *Pn = B.get<double>(n), *Pn1 = B.get<double>(n);
    double *Vn = B.get<double>(n), *Sn = B.get<double>(n), *Tn = B.get<double>(n);
    if (!Rn || !sRn || !Pn || !Pn1 || !Vn || !Sn || !Tn) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    // Rn = b - A(Un)
    MvReq<double> q0;
    q0.x = x; q0.y = Rn; q0.s = b; q0.sign = -1; q0.neg = 1; q0.exact = exact;
    xf_mv64(op, q0);
    XF_CUDA(ctx, cudaMemcpyAsync(sRn, Rn, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    k_bcgs_end<true><<<rb, RED_THREADS, 0, ctx->stream>>>(x, Rn, Pn, Pn1, Sn, Tn, m, n, S, 0, CTL_BCGS_NORM0);
    // Jacobi (XF_PRECOND_JACOBI; Laplace and advection-diffusion operators): right
    // preconditioning by the inverse row diagonals, so A sees dinv p and
    // dinv s, x moves along them, and the residual stays b - A x.  It evens
    // out rows of very different scales (semi-sums of 1/2, normal differences
    // of 1/h, Actual rows of 1/tau and more).
    const double* dinv = nullptr;
    double *Ph = nullptr, *Sh = nullptr;
    if (o.precond == XF_PRECOND_JACOBI) {
      int js = xf_op_jacobi(op, &dinv);
      if (js) return js;
      Ph = B.get<double>(n);
      Sh = B.get<double>(n);
      if (!Ph || !Sh) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    } else if (o.precond != XF_PRECOND_NONE) {
      return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: BiCGStab takes XF_PRECOND_JACOBI or none");
    }
    // the previous direction and the new one alternate between Pn and Pn1 with
    // the iteration's parity (chunks of an even number of iterations)
    even_chunks = true;
    iter = [=](int it) {
      double* Pold = (it & 1) ? Pn1 : Pn;
      double* Pnew = (it & 1) ? Pn : Pn1;
      k_dot_ctl<double><<<rb, RED_THREADS, 0, ctx->stream>>>(sRn, Rn, m, n, S, SL_A, CTL_BCGS_PN1, 1);
      if (exact) k_bcgs_p<true><<<eb, 256, 0, ctx->stream>>>(Pnew, Rn, Pold, Vn, m, n, S, dinv, Ph);
      else k_bcgs_p<false><<<eb, 256, 0, ctx->stream>>>(Pnew, Rn, Pold, Vn, m, n, S, dinv, Ph);
      MvReq<double> a;
      a.x = dinv ? Ph : Pnew; a.y = Vn; a.w = sRn; a.exact = exact; a.slot = SL_A; a.ctl = CTL_BCGS_AN;
      xf_mv64(op, a);
      if (exact) k_bcgs_s<true><<<eb, 256, 0, ctx->stream>>>(Sn, Rn, Vn, m, n, S, dinv, Sh);
      else k_bcgs_s<false><<<eb, 256, 0, ctx->stream>>>(Sn, Rn, Vn, m, n, S, dinv, Sh);
      MvReq<double> c;
      c.x = dinv ? Sh : Sn; c.y = Tn; c.w = Sn; c.dot_self = 1; c.exact = exact; c.slot = SL_A; c.ctl = CTL_BCGS_WN;
      xf_mv64(op, c);
      if (exact) k_bcgs_end<true><<<rb, RED_THREADS, 0, ctx->stream>>>(x, Rn, nullptr, Pnew, Sn, Tn, m, n, S, 1,
                                                                        CTL_BCGS_END, Ph, Sh);
      else k_bcgs_end<false><<<rb, RED_THREADS, 0, ctx->stream>>>(x, Rn, nullptr, Pnew, Sn, Tn, m, n, S, 1,
                                                                  CTL_BCGS_END, Ph, Sh);
    };
  } else if (o.method == XF_MINRES) {
    if (eps <= 0) eps = 1e-7;   // XSLAE.cpp:358
    k_reset_state<<<1, 1, 0, ctx->stream>>>(S, 0.0, eps, o.maxit, 1, 0);
    double *rk = B.get<double>(n), *Ark = B.get<double>(n);
    if (!rk || !Ark) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    MvReq<double> q0;
    q0.x = x; q0.y = rk; q0.s = b; q0.sign = -1; q0.dot_self = 1; q0.exact = exact; q0.slot = SL_A; q0.ctl = CTL_MR_INIT;
    xf_mv64(op, q0);
    iter = [=](int) {
      MvReq<double> a;
      a.x = rk; a.y = Ark; a.w = rk; a.dot_self = 1; a.exact = exact; a.slot = SL_A; a.ctl = CTL_MR_ALFA;
      xf_mv64(op, a);
      k_mr_x<<<eb, 256, 0, ctx->stream>>>(x, rk, m, n, S);
      MvReq<double> c;
      c.x = x; c.y = rk; c.s = b; c.sign = -1; c.dot_self = 1; c.exact = exact; c.slot = SL_A; c.ctl = CTL_MR_RES;
      xf_mv64(op, c);
    };
  } else if (o.method == XF_BICG) {
    // A^T exists for packed operators only (T3dLaplaceOperator::operator~
    // throws, XOperator.h:302).
    if (op->kind != XF_OP_PACK)
      return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: BiCG needs a packed operator (xf_pack_create) for A^T");
    if (eps <= 0) eps = 1e-8;   // XSLAE.cpp:166
    k_reset_state<<<1, 1, 0, ctx->stream>>>(S, 0.0, eps, o.maxit, 1, 0);
    double *rk = B.get<double>(n), *rt = B.get<double>(n), *pk = B.get<double>(n), *pt = B.get<double>(n);
    double *Ap = B.get<double>(n), *Atp = B.get<double>(n);
    if (!rk || !rt || !pk || !pt || !Ap || !Atp) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
    k_bicg_init<<<eb, 256, 0, ctx->stream>>>(x, rk, rt, pk, pt, b, m, n);
    k_dot_ctl<double><<<rb, RED_THREADS, 0, ctx->stream>>>(rk, rk, m, n, S, SL_D, CTL_BICG_INIT, 0);
    iter = [=](int) {
      k_dot_ctl<double><<<rb, RED_THREADS, 0, ctx->stream>>>(rk, rt, m, n, S, SL_B, CTL_NONE, 1);
      MvReq<double> a;
      a.x = pk; a.y = Ap; a.w = pt; a.slot = SL_A; a.ctl = CTL_BICG_ALPHA;
      xf_mv64(op, a);
      MvReq<double> t;
      t.x = pt; t.y = Atp; t.transpose = 1; t.guard = 1;
      xf_mv64(op, t);
      k_bicg_update<<<rb, RED_THREADS, 0, ctx->stream>>>(x, rk, rt, pk, Ap, Atp, m, n, S);
      k_bicg_p<<<eb, 256, 0, ctx->stream>>>(pk, pt, rk, rt, m, n, S);
    };
  } else {
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: method %d not available", o.method);
  }
  XF_CUDA(ctx, cudaGetLastError());
  int chunk = o.check_every > 0 ? o.check_every : 16;
  if (even_chunks) chunk += chunk & 1;
  int rc = run_loop(ctx, iter, chunk, o.maxit, &hs);
  if (rc) return rc;
  double* tmp = B.get<double>(n, false);
  if (!tmp) return xf_fail(ctx, XF_ERR_NOMEM, "xf_solve: allocation");
  double own = o.method == XF_BICGSTAB ? read_scalar(ctx, D_NORM) : read_scalar(ctx, D_EPSCUR);
  double rel = 0;
  int r2 = true_residual(op, x, b, tmp, &rel, nullptr);
  if (r2) return r2;
  st->status = (int)hs.status;
  st->iterations = (int)hs.it;
  st->rel_resid = rel;
  st->abs_resid = own;
  st->reserved[0] = (double)(hs.kernels + 6);
  return XF_OK;
}

// ---------------------------------------------------------------------------
// Kernel timing of one CG iteration, each kernel alone (CUDA events on the
// context stream around every launch; the solver state is reset between
// launches so no control step turns the next launch into a no-op).
extern "C" int xf_profile_cg_kernels(xf_op* op, int reps, double* ms_out) {
  if (!op || !ms_out || reps <= 0) return XF_ERR_ARG;
  xf_grid* g = op->g;
  xf_ctx* ctx = g->ctx;
  if (op->kind != XF_OP_LAPLACE) return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_profile_cg_kernels: Laplace operators only");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  DevScratch* S = ctx->scratch;
  const int64_t n = g->ncell;
  const int rb = red_blocks(ctx, n), eb = grid_blocks(ctx, n, 256);
  Bufs B(ctx);
  float *e = B.get<float>(n), *r = B.get<float>(n), *p = B.get<float>(n), *q = B.get<float>(n);
  double *x = B.get<double>(n), *b = B.get<double>(n), *p64 = B.get<double>(n), *q64 = B.get<double>(n);
  if (!e || !r || !p || !q || !x || !b || !p64 || !q64) return xf_fail(ctx, XF_ERR_NOMEM, "xf_profile_cg_kernels: allocation");
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  auto time = [&](const std::function<void()>& f) -> double {
    double tot = 0;
    for (int k = 0; k < reps + 2; k++) {
      k_reset_state<<<1, 1, 0, ctx->stream>>>(S, 0.0, 0.0, 1ll << 40, 1ll << 40, 1);
      cudaEventRecord(t0, ctx->stream);
      f();
      cudaEventRecord(t1, ctx->stream);
      cudaEventSynchronize(t1);
      float ms = 0;
      cudaEventElapsedTime(&ms, t0, t1);
      if (k >= 2) tot += ms;
    }
    return tot / reps;
  };
  ms_out[0] = time([&] { xf_cg_q32(op, p, q); });
  const int xb32 = xr_blocks<float>(ctx, n);
  ms_out[1] = time([&] { k_cg_xr<float><<<xb32, RED_THREADS, 0, ctx->stream>>>(e, r, p, q, n, S); });
  ms_out[2] = time([&] { k_cg_p<float><<<eb, 256, 0, ctx->stream>>>(p, r, n, S, 0); });
  ms_out[3] = time([&] { xf_cg_res64(op, x, b, r, SL_C, CTL_NONE); });
  ms_out[4] = time([&] { xf_cg_q64(op, p64, q64); });
  ms_out[5] = ms_out[6] = -1.0;
  if (xf_cg_pq_supported(g)) {
    float* p2 = B.get<float>(n);
    if (!p2) return xf_fail(ctx, XF_ERR_NOMEM, "xf_profile_cg_kernels: allocation");
    ms_out[5] = time([&] { xf_cg_pq32(op, r, p, p2, q); });
    if (xf_cg_pqt_supported(g)) ms_out[6] = time([&] { xf_cg_pq32_variant(op, r, p, p2, q, 1); });
  }
  ms_out[7] = ms_out[8] = ms_out[9] = ms_out[10] = ms_out[11] = -1.0;
  if (xf_cg_poly_supported(g)) {
    float coeffs[3];
    xf_cheb2_coeffs(4.0 * (g->ucx + g->ucy + g->ucz), 30.0, coeffs);
    ms_out[7] = time([&] { xf_cg_poly_launch(op, r, e, coeffs); });
    float *r2 = B.get<float>(n), *z2 = B.get<float>(n);
    if (!r2 || !z2) return xf_fail(ctx, XF_ERR_NOMEM, "xf_profile_cg_kernels: allocation");
    ms_out[8] = time([&] { xf_cg_polyr_launch(op, r, r2, q, p, p, e, z2, coeffs); });
    float f1[3], f2[3];
    if (xf_cheb4_factors(4.0 * (g->ucx + g->ucy + g->ucz), 120.0, f1, f2)) {
      ms_out[9] = time([&] { xf_cg_poly_first_launch(op, r, z2, f2, q, p, p, e, r2); });
      ms_out[10] = time([&] { xf_cg_poly_second_launch(op, z2, r2, e, f1); });
      ms_out[11] = time([&] { xf_cg_poly_first_launch(op, z2, e, f1, nullptr, nullptr, nullptr, nullptr, nullptr); });
    }
  }
  ms_out[12] = ms_out[13] = ms_out[14] = -1.0;
  if (xf_cg_poly_supported(g) && xf_tl_prolong_ay_supported(g) && (g->n1 - 2) % 4 == 0 && (g->n2 - 2) % 4 == 0 &&
      (g->n3 - 2) % 4 == 0) {
    // the learned two-level preconditioner's fine-grid passes: y = P zc with
    // A y and (y, A y); the smoother's first pass on r - omega A y; its last,
    // z = omega y + s p1(A) w into z and the direction slot with (z, r), (z, q)
    const int c2 = (g->n2 - 2) / 4 + 2, c3 = (g->n3 - 2) / 4 + 2;
    const int64_t nc = (int64_t)((g->n1 - 2) / 4 + 2) * c2 * c3;
    float *zc = B.get<float>(nc), *y = B.get<float>(n), *w = B.get<float>(n), *z2 = B.get<float>(n);
    if (!zc || !y || !w || !z2) return xf_fail(ctx, XF_ERR_NOMEM, "xf_profile_cg_kernels: allocation");
    float f1[3], f2[3];
    if (xf_cheb4_factors(4.0 * (g->ucx + g->ucy + g->ucz), 6.0, f1, f2)) {
      ms_out[12] = time([&] { xf_tl_prolong_ay(op, zc, c2, c3, y, q, SL_C); });
      ms_out[13] = time([&] {
        xf_cg_poly_tl_launch(op, true, false, r, q, w, f2, SL_C, SL_C + 1, y, 1.f, p, r, q, SL_C + 2, SL_C + 3);
      });
      ms_out[14] = time([&] {
        xf_cg_poly_tl_launch(op, false, true, w, q, e, f1, SL_C, SL_C + 1, y, 1.f, p, r, q, SL_C + 2, SL_C + 3);
      });
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" void xf_solve_opts_default(xf_solve_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->method = XF_CG;
  o->precision = XF_PREC_FP64;
  o->precond = XF_PRECOND_NONE;
  o->maxit = 100000;
  o->rtol = 1e-8;
  o->atol = 0.0;
  o->replace_every = 50;
  o->check_every = 16;
  o->exact = 0;
}

extern "C" int xf_solve(xf_op* op, const xf_solve_opts* opts, xf_vec* x, const xf_vec* b, xf_solve_stats* stats) {
  if (!op || !x || !b || !stats) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  if (x->g != op->g || b->g != op->g) return xf_fail(ctx, XF_ERR_STATE, "xf_solve: vectors of another grid");
  if (x->dtype != XF_F64 || b->dtype != XF_F64) return xf_fail(ctx, XF_ERR_STATE, "xf_solve: x and b must be FP64");
  int st;
  if ((st = xf_op_ready(op))) return st;
  xf_solve_opts o;
  if (opts) o = *opts;
  else xf_solve_opts_default(&o);
  if (o.maxit <= 0) o.maxit = 100000;
  if (o.rtol <= 0) o.rtol = 1e-8;
  if (o.replace_every <= 0) o.replace_every = 50;
  if (o.check_every <= 0) o.check_every = 16;
  memset(stats, 0, sizeof(*stats));
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  if (op->kind == XF_OP_PACK && (o.precision != XF_PREC_FP64 || (o.method == XF_CG && o.exact)))
    return xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: packed operators solve in FP64");
  if (o.method == XF_CG) st = solve_cg(op, o, x, b, stats);
  else if (o.method == XF_CG_REFERENCE || o.method == XF_BICGSTAB || o.method == XF_MINRES || o.method == XF_BICG)
    st = solve_reference(op, o, x, b, stats);
  else st = xf_fail(ctx, XF_ERR_UNSUPPORTED, "xf_solve: method %d not available", o.method);
  if (st) {
    cudaStreamSynchronize(ctx->stream);
    return st;
  }
  XF_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  XF_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  stats->ms = ms;
  return XF_OK;
}

extern "C" int xf_solve_host(xf_op* op, const xf_solve_opts* opts, double* host_x, const double* host_b,
                             xf_solve_stats* stats) {
  if (!op || !host_x || !host_b) return XF_ERR_ARG;
  xf_ctx* ctx = op->g->ctx;
  // The device boxes of x and b stay with the operator between calls (no
  // allocation, zero fill or free per solve); the copies and the solve are
  // queued on the context stream with one synchronisation at the end.
  int st;
  if (!op->host_x && (st = xf_vec_create(op->g, XF_F64, &op->host_x))) return st;
  if (!op->host_b && (st = xf_vec_create(op->g, XF_F64, &op->host_b))) return st;
  const size_t bytes = (size_t)op->g->ncell * sizeof(double);
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaMemcpyAsync(op->host_x->data, host_x, bytes, cudaMemcpyHostToDevice, ctx->stream));
  XF_CUDA(ctx, cudaMemcpyAsync(op->host_b->data, host_b, bytes, cudaMemcpyHostToDevice, ctx->stream));
  if ((st = xf_solve(op, opts, op->host_x, op->host_b, stats))) return st;
  XF_CUDA(ctx, cudaMemcpyAsync(host_x, op->host_x->data, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}
