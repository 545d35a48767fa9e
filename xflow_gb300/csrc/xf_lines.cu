// Batched tridiagonal lines: TSLAE::SolveByScalarRunning (XSLAE.cpp:416-445)
// for every grid line of an ADI sweep at once.
//
// Line (l1, l2), element m of every array sits at l1*ls1 + l2*ls2 + m*ms, so
// the lines of a box along any axis are one call (e.g. along i: ms = s1,
// ls1 = s2 over j, ls2 = 1 over k).  One thread per line runs the reference's
// recurrences in its operation order:
//     A[0] = 0, B[0] = u[0];
//     A[m] = -c[m] / (a[m] A[m-1] + b[m]),  B[m] = (f[m] - a[m] B[m-1]) / (a[m] A[m-1] + b[m]);
//     u[m] = A[m] u[m+1] + B[m],  m = M-1 .. 1  (u[0], u[M] are boundary values).
// A[m] goes to the context's workspace laid out [m][line] (coalesced across the
// threads of a warp); B[m] waits in u[m] until the back-substitution replaces
// it.  FP64 without contraction and with IEEE division: bit-identical to the
// serial reference.
#include "xf_common.cuh"

__global__ void k_thomas(int M, int nl1, int nl2, int64_t ls1, int64_t ls2, int64_t ms, double* __restrict__ u,
                         const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                         const double* __restrict__ f, double* __restrict__ Aw) {
  const int64_t nl = (int64_t)nl1 * nl2;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l >= nl) return;
  const int l1 = (int)(l / nl2), l2 = (int)(l - (int64_t)l1 * nl2);
  const int64_t base = l1 * ls1 + l2 * ls2;
  double Am1 = 0, Bm1 = u[base];
  for (int m = 1; m < M; m++) {
    const int64_t e = base + m * ms;
    const double am = a[e];
    const double den = am * Am1 + b[e];
    const double Am = (-c[e]) / den;
    const double Bm = (f[e] - am * Bm1) / den;
    Aw[(int64_t)m * nl + l] = Am;
    u[e] = Bm;
    Am1 = Am;
    Bm1 = Bm;
  }
  double un = u[base + (int64_t)M * ms];
  for (int m = M - 1; m > 0; m--) {
    const int64_t e = base + m * ms;
    un = Aw[(int64_t)m * nl + l] * un + u[e];
    u[e] = un;
  }
}

extern "C" int xf_thomas_lines(xf_ctx* ctx, int M, int nl1, int nl2, int64_t ls1, int64_t ls2, int64_t ms, double* u,
                               const double* a, const double* b, const double* c, const double* f) {
  if (!ctx || !u || !a || !b || !c || !f) return XF_ERR_ARG;
  if (M < 1 || nl1 < 0 || nl2 < 0) return xf_fail(ctx, XF_ERR_ARG, "xf_thomas_lines: M >= 1 and line counts >= 0");
  const int64_t nl = (int64_t)nl1 * nl2;
  if (nl == 0 || M == 1) return XF_OK;   // nothing between the two boundary values
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  double* Aw = (double*)xf_ctx_work(ctx, (size_t)M * nl * sizeof(double));
  if (!Aw) return xf_fail(ctx, XF_ERR_NOMEM, "xf_thomas_lines: workspace of %lld doubles", (long long)(M * nl));
  const int t = 128;
  k_thomas<<<(unsigned)((nl + t - 1) / t), t, 0, ctx->stream>>>(M, nl1, nl2, ls1, ls2, ms, u, a, b, c, f, Aw);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}
