// Voxelisation of a closed triangle surface into the point-code box: every
// point (x[i], y[j], z[k]) inside the surface gets a given code (the
// immersed-body configuration masks its icosphere Fictive this way; the
// reference has no voxeliser and uses the STL vertices only as immersed
// boundary markers, XImmersedBoundary.cpp:1560-1570).
//
// One warp per ray along x at (y[j], z[k]).  A triangle is crossed when the
// ray's (y, z) lies in its projection onto the (y, z) plane.  Points on a
// projected edge follow the top-left rule of rasterisation: with the
// triangle's projection traversed counter-clockwise, an edge counts when it
// runs downwards in z, or horizontally in +y.  Two triangles sharing an edge
// traverse it in opposite directions, so exactly one of them counts it.  Each
// edge function is computed from the edge's endpoints in lexicographic order
// and negated for the other direction, so both triangles see exactly opposite
// values.  Triangles whose projection has zero area are skipped (the ray
// grazes them).  Crossing abscissae are sorted; a point is inside when an odd
// number of them lie below its x.  Products and sums are rounded one by one
// (no fused multiply-add), so the CPU restatement gets the same bits.
#include <stdint.h>

#include <vector>

#include "xf_common.cuh"

namespace {

constexpr int VX_MAXC = 128;   // surface crossings per ray

struct P2 {
  double u, v;
};

// Edge function of the directed edge a -> b at p: > 0 left of the edge.
__device__ __forceinline__ double edge_fn(P2 a, P2 b, P2 p) {
  const bool fwd = a.u < b.u || (a.u == b.u && a.v < b.v);
  const P2 s = fwd ? a : b, t = fwd ? b : a;
  const double du = __dsub_rn(t.u, s.u), dv = __dsub_rn(t.v, s.v);
  const double e = __dsub_rn(__dmul_rn(du, __dsub_rn(p.v, s.v)), __dmul_rn(dv, __dsub_rn(p.u, s.u)));
  return fwd ? e : -e;
}

// Whether p on the directed edge a -> b (counter-clockwise traversal) counts.
__device__ __forceinline__ bool top_left(P2 a, P2 b) {
  const double du = __dsub_rn(b.u, a.u), dv = __dsub_rn(b.v, a.v);
  return dv < 0.0 || (dv == 0.0 && du > 0.0);
}

// Conservative (y, z) bounding box of each triangle in FP32, rounded outwards:
// the ray test below rejects on it before the exact FP64 edge functions.
__global__ void k_tri_boxes(const double* __restrict__ V, const int32_t* __restrict__ F, long long nf,
                            float4* __restrict__ box) {
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
    const int32_t ia = F[3 * f], ib = F[3 * f + 1], ic = F[3 * f + 2];
    const double ya = V[3 * ia + 1], yb = V[3 * ib + 1], yc = V[3 * ic + 1];
    const double za = V[3 * ia + 2], zb = V[3 * ib + 2], zc = V[3 * ic + 2];
    box[f] = make_float4(__double2float_rd(fmin(ya, fmin(yb, yc))), __double2float_ru(fmax(ya, fmax(yb, yc))),
                         __double2float_rd(fmin(za, fmin(zb, zc))), __double2float_ru(fmax(za, fmax(zb, zc))));
  }
}

// One warp per ray: the lanes take the triangles in turn, the hits are
// compacted into the warp's list by ballot, lane 0 sorts it, and the lanes
// share the sweep along x.
constexpr int VX_WARPS = 4;
__global__ void __launch_bounds__(32 * VX_WARPS) k_voxelize(int n1, int n2, int n3, const double* __restrict__ xn,
                                                           const double* __restrict__ yn, const double* __restrict__ zn,
                                                           const double* __restrict__ V, const int32_t* __restrict__ F,
                                                           const float4* __restrict__ box, long long nf,
                                                           int32_t inside_code, int32_t* __restrict__ codes,
                                                           int* __restrict__ err) {
  __shared__ double xs_all[VX_WARPS][VX_MAXC];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long ray = blockIdx.x * (long long)VX_WARPS + warp;
  if (ray >= (long long)n2 * n3) return;   // the whole warp
  double* xs = xs_all[warp];
  const int j = (int)(ray / n3), k = (int)(ray - (long long)j * n3);
  const P2 p = {yn[j], zn[k]};
  const float pu_lo = __double2float_rd(p.u), pu_hi = __double2float_ru(p.u);
  const float pv_lo = __double2float_rd(p.v), pv_hi = __double2float_ru(p.v);
  int nc = 0;
  for (long long f0 = 0; f0 < nf; f0 += 32) {
    const long long f = f0 + lane;
    bool hit = false;
    double x = 0.0;
    if (f < nf) {
      const float4 bx = box[f];
      if (pu_hi >= bx.x && pu_lo <= bx.y && pv_hi >= bx.z && pv_lo <= bx.w) {
        const int32_t ia = F[3 * f], ib = F[3 * f + 1], ic = F[3 * f + 2];
        const P2 a = {V[3 * ia + 1], V[3 * ia + 2]}, b = {V[3 * ib + 1], V[3 * ib + 2]};
        const P2 c = {V[3 * ic + 1], V[3 * ic + 2]};
        const double area = edge_fn(a, b, c);
        if (area != 0.0) {
          // counter-clockwise traversal a -> b2 -> c2
          const P2 b2 = area > 0 ? b : c, c2 = area > 0 ? c : b;
          const double e0 = edge_fn(a, b2, p), e1 = edge_fn(b2, c2, p), e2 = edge_fn(c2, a, p);
          hit = (e0 > 0.0 || (e0 == 0.0 && top_left(a, b2))) && (e1 > 0.0 || (e1 == 0.0 && top_left(b2, c2))) &&
                (e2 > 0.0 || (e2 == 0.0 && top_left(c2, a)));
          if (hit) {   // barycentric x: weights e1 (opposite a), e2 (opposite b2), e0 (opposite c2)
            const double xa = V[3 * ia], xb = area > 0 ? V[3 * ib] : V[3 * ic], xc = area > 0 ? V[3 * ic] : V[3 * ib];
            const double num = __dadd_rn(__dadd_rn(__dmul_rn(e1, xa), __dmul_rn(e2, xb)), __dmul_rn(e0, xc));
            x = __ddiv_rn(num, __dadd_rn(__dadd_rn(e1, e2), e0));
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (hit) {
      const int pos = nc + __popc(m & ((1u << lane) - 1u));
      if (pos < VX_MAXC) xs[pos] = x;
    }
    nc += __popc(m);
  }
  if (nc > VX_MAXC) {
    if (lane == 0) atomicExch(err, 1);
    return;
  }
  __syncwarp();
  if (lane == 0)
    for (int q = 1; q < nc; q++) {   // insertion sort: a handful of crossings per ray
      const double v = xs[q];
      int r = q - 1;
      while (r >= 0 && xs[r] > v) {
        xs[r + 1] = xs[r];
        r--;
      }
      xs[r + 1] = v;
    }
  __syncwarp();
  for (int i = lane; i < n1; i += 32) {
    const double xi = xn[i];
    int c = 0;
    while (c < nc && xs[c] < xi) c++;
    if (c & 1) codes[((long long)i * n2 + j) * n3 + k] = inside_code;
  }
}

}  // namespace

extern "C" int xf_voxelize_mesh(xf_ctx* ctx, int n1, int n2, int n3, const double* x_nodes, const double* y_nodes,
                                const double* z_nodes, const double* vertices, long long nvert, const int32_t* faces,
                                long long nface, int32_t inside_code, int32_t* codes) {
  if (!ctx || n1 < 1 || n2 < 1 || n3 < 1 || !x_nodes || !y_nodes || !z_nodes || !codes || nvert < 0 || nface < 0 ||
      (nface > 0 && (!vertices || !faces)))
    return XF_ERR_ARG;
  for (long long f = 0; f < 3 * nface; f++)
    if (faces[f] < 0 || faces[f] >= nvert)
      return xf_fail(ctx, XF_ERR_ARG, "xf_voxelize_mesh: face %lld names vertex %d of %lld", f / 3, faces[f], nvert);
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t nb = (size_t)n1 * n2 * n3;
  std::vector<void*> bufs;
  auto get = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes ? bytes : 16, ctx->stream) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  double *dx = (double*)get(n1 * 8), *dy = (double*)get(n2 * 8), *dz = (double*)get(n3 * 8);
  double* dv = (double*)get((size_t)nvert * 24);
  int32_t* df = (int32_t*)get((size_t)nface * 12);
  int32_t* dc = (int32_t*)get(nb * 4);
  int* derr = (int*)get(sizeof(int));
  float4* dbox = (float4*)get((size_t)nface * sizeof(float4));
  int st = XF_OK, herr = 0;
  cudaError_t e = cudaSuccess;
  if (!dx || !dy || !dz || !dv || !df || !dc || !derr || !dbox) {
    st = xf_fail(ctx, XF_ERR_NOMEM, "xf_voxelize_mesh: device allocation");
  } else {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x_nodes, n1 * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y_nodes, n2 * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z_nodes, n3 * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && nvert) e = cudaMemcpyAsync(dv, vertices, nvert * 24, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && nface) e = cudaMemcpyAsync(df, faces, nface * 12, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, codes, nb * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(derr, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess && nface) {
      k_tri_boxes<<<grid_blocks(ctx, nface, 256), 256, 0, ctx->stream>>>(dv, df, nface, dbox);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      const long long rays = (long long)n2 * n3;
      k_voxelize<<<(unsigned)((rays + VX_WARPS - 1) / VX_WARPS), 32 * VX_WARPS, 0, ctx->stream>>>(
          n1, n2, n3, dx, dy, dz, dv, df, dbox, nface, inside_code, dc, derr);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = xf_fail(ctx, XF_ERR_CUDA, "xf_voxelize_mesh: %s", cudaGetErrorString(e));
    else if (herr) st = xf_fail(ctx, XF_ERR_ARG, "xf_voxelize_mesh: a ray crosses the surface more than %d times", VX_MAXC);
    else if ((e = cudaMemcpy(codes, dc, nb * 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
      st = xf_fail(ctx, XF_ERR_CUDA, "xf_voxelize_mesh: %s", cudaGetErrorString(e));
  }
  for (void* p : bufs) cudaFreeAsync(p, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return st;
}
