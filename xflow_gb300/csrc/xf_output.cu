// Field output: the VTK legacy ASCII volume the time loop writes
// (TVPProblem::SolveBySplitting, XProblem.cpp:6132-6345) and NPY files in the
// format of the reference's cnpy::npy_save (cnpy.h:66-112, 206-233).
//
// The VTK text is produced on the device: for each section a length pass
// (node averages formatted, lengths summed per block), one scan of the block
// sums, and a write pass (lengths again, a block scan, characters stored at
// their offsets); the host streams each section's bytes to the file through
// two pinned staging buffers.  Numbers are printed as C's "%f" prints them:
// the exact binary value rounded to 6 decimals, ties to even, "-" for any
// negative value (also -0.0 and values that round to zero), "inf" / "nan".
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "xf_common.cuh"

namespace {

constexpr int OUT_THREADS = 256;

// Character sink: counts always, stores when p is set.
struct Emit {
  char* p;
  int n;
  __device__ __forceinline__ void c(char ch) {
    if (p) p[n] = ch;
    n++;
  }
  __device__ __forceinline__ void s(const char* t) {
    while (*t) c(*t++);
  }
};

// Digits of v, most significant first, into d (at most 20); returns the count.
__device__ __forceinline__ int u64_digits(uint64_t v, char* d) {
  char t[20];
  int n = 0;
  do {
    t[n++] = (char)('0' + (int)(v % 10));
    v /= 10;
  } while (v);
  for (int q = 0; q < n; q++) d[q] = t[n - 1 - q];
  return n;
}

// Digits of a little-endian base-2^32 integer (destroyed), most significant
// first into d (at most 330); returns the count.
__device__ __noinline__ int big_digits(uint32_t* limb, int nl, char* d) {
  char t[333];
  int n = 0;
  while (nl > 0 && limb[nl - 1] == 0) nl--;
  while (nl > 0) {
    uint64_t rem = 0;
    for (int q = nl - 1; q >= 0; q--) {
      const uint64_t cur = (rem << 32) | limb[q];
      limb[q] = (uint32_t)(cur / 1000000000u);
      rem = cur % 1000000000u;
    }
    while (nl > 0 && limb[nl - 1] == 0) nl--;
    uint32_t r = (uint32_t)rem;
    for (int q = 0; q < 9; q++) {
      t[n++] = (char)('0' + r % 10);
      r /= 10;
    }
  }
  while (n > 1 && t[n - 1] == '0') n--;
  if (n == 0) t[n++] = '0';
  for (int q = 0; q < n; q++) d[q] = t[n - 1 - q];
  return n;
}

// "%f" of x into e.
__device__ void fmt_f6(double x, Emit& e) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const bool neg = (bits >> 63) != 0;
  const int ex = (int)((bits >> 52) & 0x7ff);
  const uint64_t frac = bits & ((1ull << 52) - 1);
  if (neg) e.c('-');
  if (ex == 0x7ff) {
    e.s(frac ? "nan" : "inf");
    return;
  }
  const uint64_t m = ex ? (frac | (1ull << 52)) : frac;
  const int e2 = ex ? ex - 1075 : -1074;   // x = m * 2^e2
  char d[333];
  int nd;
  // N = round-half-even(m * 10^6 * 2^e2), printed with the point 6 digits from the right
  if (e2 < 0) {
    const int s = -e2;
    const uint64_t Ml = m * 1000000ull, Mh = __umul64hi(m, 1000000ull);   // m 10^6 < 2^73
    uint64_t qlo = 0, qhi = 0;
    if (s < 74) {
      bool up;
      if (s < 64) {
        qlo = (Ml >> s) | (Mh << (64 - s));
        qhi = Mh >> s;
        const uint64_t rem = Ml & ((1ull << s) - 1), half = 1ull << (s - 1);
        up = rem > half || (rem == half && (qlo & 1));
      } else if (s == 64) {
        qlo = Mh;
        const uint64_t half = 1ull << 63;
        up = Ml > half || (Ml == half && (qlo & 1));
      } else {   // 65..73
        qlo = Mh >> (s - 64);
        const uint64_t rh = Mh & ((1ull << (s - 64)) - 1), hh = 1ull << (s - 65);
        up = rh > hh || (rh == hh && Ml > 0) || (rh == hh && Ml == 0 && (qlo & 1));
      }
      if (up && ++qlo == 0) qhi++;
    }
    if (qhi == 0) {
      nd = u64_digits(qlo, d);
    } else {
      uint32_t limb[4] = {(uint32_t)qlo, (uint32_t)(qlo >> 32), (uint32_t)qhi, (uint32_t)(qhi >> 32)};
      nd = big_digits(limb, 4, d);
    }
  } else {
    if (e2 < 11 && (m << e2) <= 18446744073709ull) {
      nd = u64_digits((m << e2) * 1000000ull, d);
    } else {
      uint32_t limb[36];
      const int w = e2 >> 5, b = e2 & 31;
      for (int q = 0; q < 36; q++) limb[q] = 0;
      // m << b spans at most three limbs
      const uint64_t lo = m << b;
      const uint64_t hi = b ? (m >> (64 - b)) : 0;
      limb[w] = (uint32_t)lo;
      limb[w + 1] = (uint32_t)(lo >> 32);
      limb[w + 2] = (uint32_t)hi;
      int nl = w + 3;
      uint64_t carry = 0;
      for (int q = 0; q < nl; q++) {
        const uint64_t t = (uint64_t)limb[q] * 1000000ull + carry;
        limb[q] = (uint32_t)t;
        carry = t >> 32;
      }
      if (carry) limb[nl++] = (uint32_t)carry;
      nd = big_digits(limb, nl, d);
    }
  }
  if (nd <= 6) {
    e.c('0');
    e.c('.');
    for (int q = nd; q < 6; q++) e.c('0');
    for (int q = 0; q < nd; q++) e.c(d[q]);
  } else {
    for (int q = 0; q < nd - 6; q++) e.c(d[q]);
    e.c('.');
    for (int q = nd - 6; q < nd; q++) e.c(d[q]);
  }
}

enum { SEC_POINTS = 0, SEC_VELOCITY, SEC_PRESSURE, SEC_DENSITY, SEC_CONC, SEC_VIS, SEC_LIST };

struct VtkArgs {
  int N, L, M;                        // the node grid's EndIndex per axis (box (N+1) x (L+1) x (M+1))
  int64_t npts;                       // (N-1)(L-1)(M-1)
  const double *x, *y, *z;            // node coordinates
  const uint8_t* node_code;           // node box codes
  const double *u, *v, *w;            // staggered boxes
  const uint8_t* code8;               // the section's mask (pressure box)
  const double* f8;                   // the section's field (pressure box)
  const double* list;                 // SEC_LIST: values
};

// Node average of an 8-cell pressure-box field (XProblem.cpp:6199-6236):
// masked count of non-Fictive cells, unmasked sum in the reference's order.
__device__ __forceinline__ double avg8(const uint8_t* __restrict__ code, const double* __restrict__ f, int i, int j,
                                       int k, int64_t s1, int64_t s2) {
  const int64_t c = i * s1 + j * s2 + k;
  if (code[c] == 0) return 0.0;
  const int64_t o1 = c + s1, o2 = c + s1 + s2, o3 = c + s1 + 1, o4 = c + s1 + s2 + 1, o5 = c, o6 = c + s2,
                o7 = c + 1, o8 = c + s2 + 1;
  const int avr = (int)(code[o1] != 0) + (int)(code[o2] != 0) + (int)(code[o3] != 0) + (int)(code[o4] != 0) +
                  (int)(code[o5] != 0) + (int)(code[o6] != 0) + (int)(code[o7] != 0) + (int)(code[o8] != 0);
  return (f[o1] + f[o2] + f[o3] + f[o4] + f[o5] + f[o6] + f[o7] + f[o8]) / avr;
}

template <int SEC>
__device__ __forceinline__ void record(const VtkArgs& a, int64_t q, Emit& e) {
  if (SEC == SEC_LIST) {
    fmt_f6(a.list[q], e);
    e.c('\n');
    return;
  }
  const int64_t ni = a.N - 1, nj = a.L - 1;
  const int i = 1 + (int)(q % ni), j = 1 + (int)((q / ni) % nj), k = 1 + (int)(q / (ni * nj));
  if (SEC == SEC_POINTS) {   // "%f  %f  %f\n"
    fmt_f6(a.x[i], e);
    e.c(' '); e.c(' ');
    fmt_f6(a.y[j], e);
    e.c(' '); e.c(' ');
    fmt_f6(a.z[k], e);
    e.c('\n');
  } else if (SEC == SEC_VELOCITY) {   // "%f " "%f " "%f\n "
    const int nb2 = a.L + 1, nb3 = a.M + 1;   // node box; P box is one larger on every axis
    double uu = 0, vv = 0, ww = 0;
    if (a.node_code[((int64_t)i * nb2 + j) * nb3 + k] != 0) {
      const int64_t us1 = (int64_t)(nb2 + 1) * (nb3 + 1), us2 = nb3 + 1;       // u: (N+1) x (L+2) x (M+2)
      const int64_t vs1 = (int64_t)nb2 * (nb3 + 1), vs2 = nb3 + 1;             // v: (N+2) x (L+1) x (M+2)
      const int64_t ws1 = (int64_t)(nb2 + 1) * nb3, ws2 = nb3;                 // w: (N+2) x (L+2) x (M+1)
      const int64_t cu = i * us1 + j * us2 + k, cv = i * vs1 + j * vs2 + k, cw = i * ws1 + j * ws2 + k;
      uu = (a.u[cu] + a.u[cu + us2] + a.u[cu + 1] + a.u[cu + us2 + 1]) / 4;
      vv = (a.v[cv] + a.v[cv + vs1] + a.v[cv + 1] + a.v[cv + vs1 + 1]) / 4;
      ww = (a.w[cw] + a.w[cw + ws1] + a.w[cw + ws2] + a.w[cw + ws1 + ws2]) / 4;
    }
    fmt_f6(uu, e);
    e.c(' ');
    fmt_f6(vv, e);
    e.c(' ');
    fmt_f6(ww, e);
    e.c('\n');
    e.c(' ');
  } else {
    const int64_t ps2 = a.M + 2, ps1 = (int64_t)(a.L + 2) * ps2;
    fmt_f6(avg8(a.code8, a.f8, i, j, k, ps1, ps2), e);
    e.c('\n');
    if (SEC == SEC_PRESSURE) e.c(' ');   // "%f\n " for pressure, "%f\n" for the others
  }
}

template <int SEC>
__global__ void __launch_bounds__(OUT_THREADS) k_vtk_len(VtkArgs a, int64_t* __restrict__ block_sum) {
  __shared__ int64_t sh[OUT_THREADS / 32];
  const int64_t q = (int64_t)blockIdx.x * OUT_THREADS + threadIdx.x;
  int len = 0;
  if (q < a.npts) {
    Emit e{nullptr, 0};
    record<SEC>(a, q, e);
    len = e.n;
  }
  int64_t v = len;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < OUT_THREADS / 32; w++) t += sh[w];
    block_sum[blockIdx.x] = t;
  }
}

// Exclusive scan of n block sums in place (one block); total at [n].
__global__ void __launch_bounds__(1024) k_vtk_scan(int64_t* __restrict__ s, int64_t n) {
  __shared__ int64_t sh[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < n; b0 += 1024) {
    const int64_t t = b0 + threadIdx.x;
    const int64_t v = t < n ? s[t] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int64_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    if (t < n) s[t] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) s[n] = carry;
}

template <int SEC>
__global__ void __launch_bounds__(OUT_THREADS) k_vtk_write(VtkArgs a, const int64_t* __restrict__ block_off,
                                                           char* __restrict__ out) {
  __shared__ int sh[OUT_THREADS / 32];
  const int64_t q = (int64_t)blockIdx.x * OUT_THREADS + threadIdx.x;
  int len = 0;
  if (q < a.npts) {
    Emit e{nullptr, 0};
    record<SEC>(a, q, e);
    len = e.n;
  }
  // exclusive offset of this record within the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = len;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; w++) before += sh[w];
  if (q < a.npts) {
    Emit e{out + block_off[blockIdx.x] + before + incl - len, 0};
    record<SEC>(a, q, e);
  }
}

// Pinned double-buffered device -> file stream.
struct Streamer {
  xf_ctx* ctx;
  FILE* f;
  char* pin[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  size_t cap = 0;
  int64_t written = 0;
  int err = XF_OK;
  int init(size_t chunk) {
    cap = chunk;
    for (int b = 0; b < 2; b++) {
      if (cudaHostAlloc(&pin[b], cap, cudaHostAllocDefault) != cudaSuccess ||
          cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return xf_fail(ctx, XF_ERR_NOMEM, "VTK output: pinned staging buffers");
      }
    }
    return XF_OK;
  }
  ~Streamer() {
    for (int b = 0; b < 2; b++) {
      if (pin[b]) cudaFreeHost(pin[b]);
      if (ev[b]) cudaEventDestroy(ev[b]);
    }
  }
  int host(const char* s, size_t n) {
    if (fwrite(s, 1, n, f) != n) return xf_fail(ctx, XF_ERR_ARG, "VTK output: write failed");
    written += (int64_t)n;
    return XF_OK;
  }
  int device(const char* d, int64_t n) {
    const int64_t nchunk = (n + (int64_t)cap - 1) / (int64_t)cap;
    for (int64_t c = 0; c <= nchunk; c++) {
      if (c < nchunk) {
        const int b = (int)(c & 1);
        const size_t len = (size_t)((c + 1) * (int64_t)cap > n ? n - c * (int64_t)cap : (int64_t)cap);
        XF_CUDA(ctx, cudaMemcpyAsync(pin[b], d + c * (int64_t)cap, len, cudaMemcpyDeviceToHost, ctx->stream));
        XF_CUDA(ctx, cudaEventRecord(ev[b], ctx->stream));
      }
      if (c > 0) {   // write the previous chunk while this one copies
        const int b = (int)((c - 1) & 1);
        XF_CUDA(ctx, cudaEventSynchronize(ev[b]));
        const size_t len = (size_t)(c * (int64_t)cap > n ? n - (c - 1) * (int64_t)cap : (int64_t)cap);
        int st;
        if ((st = host(pin[b], len))) return st;
      }
    }
    return XF_OK;
  }
};

// Formats one section on the device into ctx work space and streams it.
template <int SEC>
int vtk_section(xf_ctx* ctx, const VtkArgs& a, Streamer& out) {
  const int64_t nblk = (a.npts + OUT_THREADS - 1) / OUT_THREADS;
  if (nblk == 0) return XF_OK;
  int64_t* sums = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&sums, (nblk + 1) * sizeof(int64_t), ctx->stream));
  k_vtk_len<SEC><<<(unsigned)nblk, OUT_THREADS, 0, ctx->stream>>>(a, sums);
  k_vtk_scan<<<1, 1024, 0, ctx->stream>>>(sums, nblk);
  int64_t total = 0;
  XF_CUDA(ctx, cudaMemcpyAsync(&total, sums + nblk, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* text = (char*)xf_ctx_work(ctx, (size_t)total);
  if (!text) {
    cudaFreeAsync(sums, ctx->stream);
    return xf_fail(ctx, XF_ERR_NOMEM, "VTK output: %lld bytes of text", (long long)total);
  }
  k_vtk_write<SEC><<<(unsigned)nblk, OUT_THREADS, 0, ctx->stream>>>(a, sums, text);
  XF_CUDA(ctx, cudaGetLastError());
  XF_CUDA(ctx, cudaFreeAsync(sums, ctx->stream));
  return out.device(text, total);
}

bool f64_box(const xf_vec* v, int n1, int n2, int n3) {
  return v && v->dtype == XF_F64 && v->g->n1 == n1 && v->g->n2 == n2 && v->g->n3 == n3;
}

}  // namespace

extern "C" int xf_vtk_write(const char* path, const xf_grid* nodes, const double* x, const double* y,
                            const double* z, const xf_vec* u, const xf_vec* v, const xf_vec* w, const xf_vec* p,
                            const xf_vec* density, const xf_vec* conc, const xf_vec* vis, int64_t* bytes) {
  if (!path || !nodes || !x || !y || !z) return XF_ERR_ARG;
  xf_ctx* ctx = nodes->ctx;
  const int N = nodes->n1 - 1, L = nodes->n2 - 1, M = nodes->n3 - 1;
  if (N < 2 || L < 2 || M < 2) return xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: the node box needs 3 nodes per axis");
  if (!f64_box(u, N + 1, L + 2, M + 2) || !f64_box(v, N + 2, L + 1, M + 2) || !f64_box(w, N + 2, L + 2, M + 1))
    return xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: u, v, w must be FP64 staggered boxes of the %dx%dx%d pressure box",
                   N + 2, L + 2, M + 2);
  const xf_vec* sc[4] = {p, density, conc, vis};
  for (const xf_vec* s : sc)
    if (!f64_box(s, N + 2, L + 2, M + 2))
      return xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: p, density, conc and vis must be FP64 pressure boxes");
  const int64_t npts = (int64_t)(N - 1) * (L - 1) * (M - 1);
  if (npts > INT32_MAX) return xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: more points than the format's %%d holds");
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  FILE* f = fopen(path, "wb");
  if (!f) return xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: cannot open %s", path);
  int st = XF_OK;
  double* dxyz = nullptr;
  {
    Streamer out;
    out.ctx = ctx;
    out.f = f;
    VtkArgs a;
    memset(&a, 0, sizeof(a));
    a.N = N; a.L = L; a.M = M; a.npts = npts;
    a.node_code = nodes->code;
    a.u = (const double*)u->data; a.v = (const double*)v->data; a.w = (const double*)w->data;
    char hdr[512];
    auto fail_cuda = [&](cudaError_t e) { return xf_fail(ctx, XF_ERR_CUDA, "xf_vtk_write: %s", cudaGetErrorString(e)); };
    cudaError_t ce = cudaMallocAsync(&dxyz, (size_t)(N + 1 + L + 1 + M + 1) * sizeof(double), ctx->stream);
    if (ce != cudaSuccess) { st = fail_cuda(ce); goto done; }
    cudaMemcpyAsync(dxyz, x, (N + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dxyz + N + 1, y, (L + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    ce = cudaMemcpyAsync(dxyz + N + 1 + L + 1, z, (M + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (ce != cudaSuccess) { st = fail_cuda(ce); goto done; }
    a.x = dxyz; a.y = dxyz + N + 1; a.z = dxyz + N + 1 + L + 1;
    if ((st = out.init((size_t)64 << 20))) goto done;
    snprintf(hdr, sizeof(hdr),
             "# vtk DataFile Version 3.0\nFlow\nASCII\n\nDATASET STRUCTURED_GRID\nDIMENSIONS %d %d %d\nPOINTS %d double\n",
             N - 1, L - 1, M - 1, (int)npts);
    if ((st = out.host(hdr, strlen(hdr))) || (st = vtk_section<SEC_POINTS>(ctx, a, out))) goto done;
    snprintf(hdr, sizeof(hdr), "POINT_DATA %d\n\nVECTORS Velocity double\n", (int)npts);
    if ((st = out.host(hdr, strlen(hdr))) || (st = vtk_section<SEC_VELOCITY>(ctx, a, out))) goto done;
    {
      // pressure (its own mask), density (its own), concentration and viscosity (both the concentration mask)
      const char* heads[4] = {"\nSCALARS Pressure float\nLOOKUP_TABLE default\n",
                              "\nSCALARS Density float\nLOOKUP_TABLE default\n",
                              "\nSCALARS Concentration float\nLOOKUP_TABLE default\n",
                              "\nSCALARS Viscosity float\nLOOKUP_TABLE default\n"};
      const xf_vec* masks[4] = {p, density, conc, conc};
      for (int s = 0; s < 4 && st == XF_OK; s++) {
        a.code8 = masks[s]->g->code;
        a.f8 = (const double*)sc[s]->data;
        if ((st = out.host(heads[s], strlen(heads[s])))) break;
        st = s == 0 ? vtk_section<SEC_PRESSURE>(ctx, a, out) : vtk_section<SEC_DENSITY>(ctx, a, out);
      }
    }
  done:
    if (bytes) *bytes = out.written;
  }
  if (dxyz) cudaFreeAsync(dxyz, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if (fclose(f) != 0 && st == XF_OK) st = xf_fail(ctx, XF_ERR_ARG, "xf_vtk_write: close failed");
  return st;
}

extern "C" int xf_format_fixed6(xf_ctx* ctx, const double* values, int64_t n, char* out, int64_t capacity,
                                int64_t* length) {
  if (!ctx || (!values && n > 0) || !length || n < 0) return XF_ERR_ARG;
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  *length = 0;
  if (n == 0) return XF_OK;
  VtkArgs a;
  memset(&a, 0, sizeof(a));
  a.npts = n;
  double* dv = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&dv, n * sizeof(double), ctx->stream));
  XF_CUDA(ctx, cudaMemcpyAsync(dv, values, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  a.list = dv;
  const int64_t nblk = (n + OUT_THREADS - 1) / OUT_THREADS;
  int64_t* sums = nullptr;
  XF_CUDA(ctx, cudaMallocAsync(&sums, (nblk + 1) * sizeof(int64_t), ctx->stream));
  k_vtk_len<SEC_LIST><<<(unsigned)nblk, OUT_THREADS, 0, ctx->stream>>>(a, sums);
  k_vtk_scan<<<1, 1024, 0, ctx->stream>>>(sums, nblk);
  int64_t total = 0;
  XF_CUDA(ctx, cudaMemcpyAsync(&total, sums + nblk, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *length = total;
  int st = XF_OK;
  if (out && total <= capacity) {
    char* text = (char*)xf_ctx_work(ctx, (size_t)total);
    if (!text) {
      st = xf_fail(ctx, XF_ERR_NOMEM, "xf_format_fixed6: work space");
    } else {
      k_vtk_write<SEC_LIST><<<(unsigned)nblk, OUT_THREADS, 0, ctx->stream>>>(a, sums, text);
      cudaMemcpyAsync(out, text, (size_t)total, cudaMemcpyDeviceToHost, ctx->stream);
    }
  } else if (out) {
    st = xf_fail(ctx, XF_ERR_ARG, "xf_format_fixed6: %lld bytes needed", (long long)total);
  }
  cudaFreeAsync(sums, ctx->stream);
  cudaFreeAsync(dv, ctx->stream);
  XF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return st;
}

// NPY version 1.0 header exactly as cnpy::create_npy_header builds it
// (cnpy.h:206-233): the dict text, space padding so that 10 + its length is a
// multiple of 16 (a full 16 when it already is), the last pad a newline.
static std::string npy_header(const char* descr, const int64_t* shape, int nd) {
  std::string d = "{'descr': '";
  d += descr;
  d += "', 'fortran_order': False, 'shape': (";
  for (int q = 0; q < nd; q++) {
    if (q) d += ", ";
    d += std::to_string((long long)shape[q]);
  }
  if (nd == 1) d += ",";
  d += "), }";
  const size_t rem = 16 - (10 + d.size()) % 16;
  d.append(rem, ' ');
  d.back() = '\n';
  std::string h;
  h += (char)0x93;
  h += "NUMPY";
  h += (char)1;
  h += (char)0;
  h += (char)(d.size() & 0xff);
  h += (char)((d.size() >> 8) & 0xff);
  return h + d;
}

extern "C" int xf_npy_write(const char* path, const xf_vec* vec) {
  if (!path || !vec) return XF_ERR_ARG;
  const xf_grid* g = vec->g;
  xf_ctx* ctx = g->ctx;
  const int64_t shape[3] = {g->n1, g->n2, g->n3};
  const size_t esz = vec->dtype == XF_F64 ? 8 : 4;
  const std::string h = npy_header(vec->dtype == XF_F64 ? "<f8" : "<f4", shape, 3);
  XF_CUDA(ctx, cudaSetDevice(ctx->device));
  FILE* f = fopen(path, "wb");
  if (!f) return xf_fail(ctx, XF_ERR_ARG, "xf_npy_write: cannot open %s", path);
  int st = XF_OK;
  {
    Streamer out;
    out.ctx = ctx;
    out.f = f;
    if (!(st = out.init((size_t)32 << 20)) && !(st = out.host(h.data(), h.size())))
      st = out.device((const char*)vec->data, g->ncell * (int64_t)esz);
  }
  if (fclose(f) != 0 && st == XF_OK) st = xf_fail(ctx, XF_ERR_ARG, "xf_npy_write: close failed");
  return st;
}
