// Immersed boundary (TImmersedBoundaryProblem, XProblem.cpp:8436-9046) and
// batched tridiagonal lines (TSLAE::SolveByScalarRunning, XSLAE.cpp:416-445).
//
// Markers live on the device as the reference's node arrays (positions 3 per
// node, node kind, next/prev neighbour, rest lengths and curvatures).  One
// thread per marker; the 7x7x7 cosine-delta weights of a marker are computed
// once per axis (7 + 7 + 7 values, the reference recomputes them per cell:
// same values) and the sums run in the reference's i -> j -> k order.
//
// Forces are gathered, not scattered: the serial reference loop
// (XProblem.cpp:8436-8547) adds, node by node, the node's own term to itself
// and its stretching/bending terms to next and prev.  At creation the host
// lists, per target node, the (source node, term) pairs in that serial order;
// the GPU then sums each target's list from zero, which reproduces the serial
// rounding exactly.  The reference's OpenMP loop races on these neighbour
// updates; the serial order is the one restated here.
//
// Spreading scatters 343 atomic FP64 adds per marker into the zeroed force
// box (contributions from different markers to one cell land in any order:
// last-bit differences against the serial loop).
//
// Thomas lines: one thread per line, the reference's recurrences and
// operation order; the forward coefficients A[m] go to a per-context
// workspace laid out [m][line] (coalesced across threads), B[m] is kept in
// u[m] until the back-substitution overwrites it.  Bit-identical to the
// serial reference (FP64, no contraction, IEEE division).
#include <math.h>

#include <vector>

#include "xf_common.cuh"

struct xf_ib {
  xf_ctx* ctx;
  int nn;
  double* pos;        // 3 per node
  double* ref;        // 3 per node
  double* vel;        // [axis][nn]
  double* force;      // [axis][nn]
  double* terms;      // [3][nn]: own, to-next, to-prev force terms of the last forces call
  double* dist0;
  double* curv0;      // 3 per node
  double* stiff;
  int32_t* kind;
  int32_t* next;
  int32_t* prev;
  int32_t* in_ptr;    // CSR over targets: nn + 1
  int32_t* in_src;    // source node * 3 + term (0 own, 1 next, 2 prev), serial order
  double params[4];
};

constexpr int IB_RANGE = 3;

// TImmersedBoundaryProblem::Index(grid, coord, type, axis, RANGE, RANGE),
// XProblem.cpp:8931-8967 (uniform grid; nend = number of nodes - 1).
__device__ __forceinline__ int ib_index(double coord, double step, int nend, int type, int axis) {
  int index = (int)floor((coord + (type != axis ? 0.5 * step : 0)) / step);
  if (index > (nend - 1) - IB_RANGE) index = (nend - 1) - IB_RANGE;
  if (index < IB_RANGE) index = IB_RANGE;
  return index;
}
// Coord(grid, index, type, axis), XProblem.cpp:8988-9006.
__device__ __forceinline__ double ib_coord(int index, double step, int type, int axis) {
  return index * step - (type != axis ? 0.5 * step : 0);
}
// Cosine delta, XProblem.cpp:9008-9032.
__device__ __forceinline__ double ib_delta(double distance, double h) {
  if (distance < 2 * h) return 1.0 / (4 * h) * (1 + cos(M_PI * distance / (2 * h)));
  return 0;
}

struct IbWeights {
  int xi, yi, zi;
  double wx[7], wy[7], wz[7];
};

__device__ __forceinline__ void ib_weights(const double* pos, int q, int n1, int n2, int n3, double h0, double h1,
                                           double h2, int axis, IbWeights& w) {
  const double px = pos[3 * q], py = pos[3 * q + 1], pz = pos[3 * q + 2];
  w.xi = ib_index(px, h0, n1 - 1, 1, axis);
  w.yi = ib_index(py, h1, n2 - 1, 2, axis);
  w.zi = ib_index(pz, h2, n3 - 1, 3, axis);
#pragma unroll
  for (int t = 0; t < 7; t++) {
    w.wx[t] = ib_delta(fabs(px - ib_coord(w.xi - IB_RANGE + t, h0, 1, axis)), h0);
    w.wy[t] = ib_delta(fabs(py - ib_coord(w.yi - IB_RANGE + t, h1, 2, axis)), h1);
    w.wz[t] = ib_delta(fabs(pz - ib_coord(w.zi - IB_RANGE + t, h2, 3, axis)), h2);
  }
}

// Interpolate, XProblem.cpp:8620-8791: node velocity = sum over the 7^3
// stencil of (u_ijk * wx * wy * wz) * h^3 (h of the interpolated axis).
__global__ void k_ib_interpolate(const double* __restrict__ vel, int n1, int n2, int n3, double h0, double h1,
                                 double h2, int axis, int nn, const double* __restrict__ pos,
                                 double* __restrict__ node_vel) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  IbWeights w;
  ib_weights(pos, q, n1, n2, n3, h0, h1, h2, axis, w);
  const double ha = axis == 1 ? h0 : axis == 2 ? h1 : h2;
  const double cb = ha * ha * ha;
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  double acc = 0;
  for (int a = 0; a < 7; a++)
    for (int b = 0; b < 7; b++) {
      const double* row = vel + (w.xi - IB_RANGE + a) * s1 + (w.yi - IB_RANGE + b) * s2 + (w.zi - IB_RANGE);
#pragma unroll
      for (int c = 0; c < 7; c++) acc += (row[c] * w.wx[a] * w.wy[b] * w.wz[c]) * cb;
    }
  node_vel[q] = acc;
}

// UpdateBoundaryPosition, XProblem.cpp:8858-8894.
__global__ void k_ib_update(int nn, int axis, double tau, const double* __restrict__ node_vel, double* pos) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  pos[3 * q + axis - 1] += node_vel[q] * tau;
}

// Node force laws, XImmersedBoundary.cpp:654-759, per node: the own term and
// the terms it adds to next and prev (ComputeBoundaryForces,
// XProblem.cpp:8436-8547).  Kinds: 0 elastic, 1 target, 2 fixed-elastic,
// 3 plain node, 4 fixed-stretching.
__global__ void k_ib_terms(int nn, int axis, const double* __restrict__ pos, const double* __restrict__ ref,
                           const int32_t* __restrict__ kind, const int32_t* __restrict__ next,
                           const int32_t* __restrict__ prev, const double* __restrict__ dist0,
                           const double* __restrict__ curv0, const double* __restrict__ node_stiff, double stiffness,
                           double kst, double kbend, double area, double* __restrict__ terms) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  const int a = axis - 1;
  double sf = 0, bf = 0, tf = 0;
  const int nx = next[q], pv = prev[q];
  const int kd = kind[q];
  if ((kd == 0 || kd == 2 || kd == 4) && nx >= 0) {
    const double DX = pos[3 * q] - pos[3 * nx], DY = pos[3 * q + 1] - pos[3 * nx + 1],
                 DZ = pos[3 * q + 2] - pos[3 * nx + 2];
    const double distance = sqrt(DX * DX + DY * DY + DZ * DZ);
    const double distance_axis = pos[3 * q + a] - pos[3 * nx + a];
    const double k = kd == 2 ? node_stiff[q] : kst;
    sf = k * (distance - dist0[q]) * distance_axis / distance;
  }
  if (kd == 0 && nx >= 0 && pv >= 0) {
    const double curv = pos[3 * nx + a] - 2 * pos[3 * q + a] + pos[3 * pv + a];
    bf = kbend * (curv0[3 * q + a] - curv);
  }
  if (kd == 1 || kd == 4) tf = stiffness * (pos[3 * q + a] - ref[3 * q + a]);
  if (kd == 2) tf = node_stiff[q] * (pos[3 * q + a] - ref[3 * q + a]);
  terms[q] = -(sf + 2 * bf + tf) * area;
  terms[nn + q] = (sf + bf) * area;
  terms[2 * nn + q] = bf * area;
}

// Each target sums its incoming terms from zero in the serial loop's order.
__global__ void k_ib_gather(int nn, const int32_t* __restrict__ in_ptr, const int32_t* __restrict__ in_src,
                            const double* __restrict__ terms, double* __restrict__ force) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  double f = 0;
  for (int e = in_ptr[q]; e < in_ptr[q + 1]; e++) {
    const int s = in_src[e];
    f += terms[(s % 3) * nn + s / 3];
  }
  force[q] = f;
}

// SpreadForce, XProblem.cpp:8550-8617 (arithmetic): f_ijk += F * wx * wy * wz
// over the 7^3 stencil of every marker; fbox is zeroed first (`force |= 0.0`).
__global__ void k_ib_spread(double* fbox, int n1, int n2, int n3, double h0, double h1, double h2, int axis, int nn,
                            const double* __restrict__ pos, const double* __restrict__ force) {
  const int q = blockIdx.x;
  if (q >= nn) return;
  __shared__ IbWeights w;
  if (threadIdx.x == 0) ib_weights(pos, q, n1, n2, n3, h0, h1, h2, axis, w);
  __syncthreads();
  const double F = force[q];
  const int64_t s1 = (int64_t)n2 * n3, s2 = n3;
  for (int t = threadIdx.x; t < 343; t += blockDim.x) {
    const int a = t / 49, b = (t / 7) % 7, c = t % 7;
    const int64_t cell = (w.xi - IB_RANGE + a) * s1 + (w.yi - IB_RANGE + b) * s2 + (w.zi - IB_RANGE + c);
    atomicAdd(fbox + cell, F * w.wx[a] * w.wy[b] * w.wz[c]);
  }
}

// ---------------------------------------------------------------------------
static int ib_check_box(const xf_ib* ib, const xf_vec* v, const double* h0, int axis, const char* who) {
  if (!ib || !v || !h0) return XF_ERR_ARG;
  if (axis < 1 || axis > 3) return xf_fail(ib->ctx, XF_ERR_ARG, "%s: axis must be 1, 2 or 3", who);
  if (v->dtype != XF_F64) return xf_fail(ib->ctx, XF_ERR_ARG, "%s: the box must be FP64", who);
  if (v->g->ctx != ib->ctx) return xf_fail(ib->ctx, XF_ERR_ARG, "%s: box and markers belong to different contexts", who);
  const xf_grid* g = v->g;
  // Index() clamps to [RANGE, nend-1-RANGE]: the 7-wide stencil needs at least
  // 2*RANGE+2 nodes per axis to stay inside the box.
  if (g->n1 < 2 * IB_RANGE + 2 || g->n2 < 2 * IB_RANGE + 2 || g->n3 < 2 * IB_RANGE + 2)
    return xf_fail(ib->ctx, XF_ERR_ARG, "%s: box smaller than the 7-point delta stencil", who);
  if (!(h0[0] > 0 && h0[1] > 0 && h0[2] > 0)) return xf_fail(ib->ctx, XF_ERR_ARG, "%s: spacings must be > 0", who);
  return XF_OK;
}

static void ib_free(xf_ib* ib) {
  void* ps[] = {ib->pos, ib->ref, ib->vel, ib->force, ib->terms, ib->dist0, ib->curv0, ib->stiff,
                ib->kind, ib->next, ib->prev, ib->in_ptr, ib->in_src};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete ib;
}

extern "C" int xf_ib_create(xf_ctx* ctx, int nn, const double* pos, const double* ref, const int32_t* kind,
                            const int32_t* next, const int32_t* prev, const double* dist0, const double* curv0,
                            const double* node_stiff, const double* params, xf_ib** out) {
  if (!ctx || !out || nn <= 0 || !pos || !ref || !kind || !next || !prev || !dist0 || !curv0 || !node_stiff || !params)
    return XF_ERR_ARG;
  *out = nullptr;
  for (int q = 0; q < nn; q++) {
    if (kind[q] < 0 || kind[q] > 4) return xf_fail(ctx, XF_ERR_ARG, "xf_ib_create: node %d has kind %d", q, kind[q]);
    if (next[q] < -1 || next[q] >= nn || prev[q] < -1 || prev[q] >= nn)
      return xf_fail(ctx, XF_ERR_ARG, "xf_ib_create: node %d has a neighbour outside [0, %d)", q, nn);
  }
  // incoming term lists in the serial loop's order (source ascending; own,
  // next, prev within one source)
  std::vector<int32_t> cnt(nn + 1, 0), src;
  for (int p = 0; p < nn; p++) {
    cnt[p + 1]++;
    if (next[p] >= 0) cnt[next[p] + 1]++;
    if (prev[p] >= 0) cnt[prev[p] + 1]++;
  }
  for (int q = 0; q < nn; q++) cnt[q + 1] += cnt[q];
  src.resize(cnt[nn]);
  std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
  for (int p = 0; p < nn; p++) {
    src[fill[p]++] = 3 * p + 0;
    if (next[p] >= 0) src[fill[next[p]]++] = 3 * p + 1;
    if (prev[p] >= 0) src[fill[prev[p]]++] = 3 * p + 2;
  }
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  xf_ib* ib = new xf_ib();
  memset(ib, 0, sizeof(*ib));
  ib->ctx = ctx;
  ib->nn = nn;
  memcpy(ib->params, params, sizeof(ib->params));
  const size_t d = sizeof(double), i4 = sizeof(int32_t);
  bool ok = cudaMalloc(&ib->pos, 3 * nn * d) == cudaSuccess && cudaMalloc(&ib->ref, 3 * nn * d) == cudaSuccess &&
            cudaMalloc(&ib->vel, 3 * nn * d) == cudaSuccess && cudaMalloc(&ib->force, 3 * nn * d) == cudaSuccess &&
            cudaMalloc(&ib->terms, 3 * nn * d) == cudaSuccess && cudaMalloc(&ib->dist0, nn * d) == cudaSuccess &&
            cudaMalloc(&ib->curv0, 3 * nn * d) == cudaSuccess && cudaMalloc(&ib->stiff, nn * d) == cudaSuccess &&
            cudaMalloc(&ib->kind, nn * i4) == cudaSuccess && cudaMalloc(&ib->next, nn * i4) == cudaSuccess &&
            cudaMalloc(&ib->prev, nn * i4) == cudaSuccess && cudaMalloc(&ib->in_ptr, (nn + 1) * i4) == cudaSuccess &&
            cudaMalloc(&ib->in_src, src.size() * i4) == cudaSuccess;
  if (!ok) {
    ib_free(ib);
    cudaGetLastError();
    return xf_fail(ctx, XF_ERR_NOMEM, "xf_ib_create: device allocation of %d markers", nn);
  }
  cudaStream_t s = ctx->stream;
  ok = cudaMemcpyAsync(ib->pos, pos, 3 * nn * d, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->ref, ref, 3 * nn * d, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemsetAsync(ib->vel, 0, 3 * nn * d, s) == cudaSuccess &&
       cudaMemsetAsync(ib->force, 0, 3 * nn * d, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->dist0, dist0, nn * d, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->curv0, curv0, 3 * nn * d, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->stiff, node_stiff, nn * d, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->kind, kind, nn * i4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->next, next, nn * i4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->prev, prev, nn * i4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->in_ptr, cnt.data(), (nn + 1) * i4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaMemcpyAsync(ib->in_src, src.data(), src.size() * i4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
       cudaStreamSynchronize(s) == cudaSuccess;
  if (!ok) {
    cudaError_t e = cudaGetLastError();
    ib_free(ib);
    return xf_fail(ctx, XF_ERR_CUDA, "xf_ib_create: upload failed (%s)", cudaGetErrorString(e));
  }
  *out = ib;
  return XF_OK;
}

extern "C" int xf_ib_destroy(xf_ib* ib) {
  if (!ib) return XF_OK;
  cudaSetDevice(ib->ctx->device);
  cudaStreamSynchronize(ib->ctx->stream);
  ib_free(ib);
  return XF_OK;
}

static double* ib_field(const xf_ib* ib, int field, size_t* count) {
  *count = 3 * (size_t)ib->nn;
  switch (field) {
    case XF_IB_POS: return ib->pos;
    case XF_IB_VEL: return ib->vel;
    case XF_IB_FORCE: return ib->force;
    default: return nullptr;
  }
}

extern "C" int xf_ib_download(const xf_ib* ib, int field, double* host) {
  if (!ib || !host) return XF_ERR_ARG;
  size_t n;
  double* p = ib_field(ib, field, &n);
  if (!p) return xf_fail(ib->ctx, XF_ERR_ARG, "xf_ib_download: unknown field %d", field);
  xf_ctx* ctx = ib->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaMemcpyAsync(host, p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

extern "C" int xf_ib_upload(xf_ib* ib, int field, const double* host) {
  if (!ib || !host) return XF_ERR_ARG;
  size_t n;
  double* p = ib_field(ib, field, &n);
  if (!p) return xf_fail(ib->ctx, XF_ERR_ARG, "xf_ib_upload: unknown field %d", field);
  xf_ctx* ctx = ib->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaMemcpyAsync(p, host, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return XF_OK;
}

static inline int ib_blocks(int n, int t) { return (n + t - 1) / t; }

extern "C" int xf_ib_interpolate(xf_ib* ib, const xf_vec* vel, const double* h0, int axis) {
  int st = ib_check_box(ib, vel, h0, axis, "xf_ib_interpolate");
  if (st) return st;
  xf_ctx* ctx = ib->ctx;
  const xf_grid* g = vel->g;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  k_ib_interpolate<<<ib_blocks(ib->nn, 128), 128, 0, ctx->stream>>>(
      (const double*)vel->data, g->n1, g->n2, g->n3, h0[0], h0[1], h0[2], axis, ib->nn, ib->pos,
      ib->vel + (size_t)(axis - 1) * ib->nn);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_ib_update_position(xf_ib* ib, int axis, double tau) {
  if (!ib) return XF_ERR_ARG;
  if (axis < 1 || axis > 3) return xf_fail(ib->ctx, XF_ERR_ARG, "xf_ib_update_position: axis must be 1, 2 or 3");
  xf_ctx* ctx = ib->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  k_ib_update<<<ib_blocks(ib->nn, 256), 256, 0, ctx->stream>>>(ib->nn, axis, tau,
                                                               ib->vel + (size_t)(axis - 1) * ib->nn, ib->pos);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_ib_compute_forces(xf_ib* ib, int axis) {
  if (!ib) return XF_ERR_ARG;
  if (axis < 1 || axis > 3) return xf_fail(ib->ctx, XF_ERR_ARG, "xf_ib_compute_forces: axis must be 1, 2 or 3");
  xf_ctx* ctx = ib->ctx;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int nb = ib_blocks(ib->nn, 256);
  k_ib_terms<<<nb, 256, 0, ctx->stream>>>(ib->nn, axis, ib->pos, ib->ref, ib->kind, ib->next, ib->prev, ib->dist0,
                                          ib->curv0, ib->stiff, ib->params[0], ib->params[1], ib->params[2],
                                          ib->params[3], ib->terms);
  k_ib_gather<<<nb, 256, 0, ctx->stream>>>(ib->nn, ib->in_ptr, ib->in_src, ib->terms,
                                           ib->force + (size_t)(axis - 1) * ib->nn);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}

extern "C" int xf_ib_spread(xf_ib* ib, xf_vec* force, const double* h0, int axis) {
  int st = ib_check_box(ib, force, h0, axis, "xf_ib_spread");
  if (st) return st;
  xf_ctx* ctx = ib->ctx;
  const xf_grid* g = force->g;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  XF_CUDA(ctx, cudaMemsetAsync(force->data, 0, g->ncell * sizeof(double), ctx->stream));
  k_ib_spread<<<ib->nn, 128, 0, ctx->stream>>>((double*)force->data, g->n1, g->n2, g->n3, h0[0], h0[1], h0[2], axis,
                                                ib->nn, ib->pos, ib->force + (size_t)(axis - 1) * ib->nn);
  XF_CUDA(ctx, cudaGetLastError());
  return XF_OK;
}
