// Allocation-free residual norm: r = b - A x and ||r||_2 with the stored FP64
// blocks, for callers that may not allocate device memory.
//
// Scratch is one FP64 partial sum per CTA of the residual launch, held in the
// file-scope device array g_noalloc_partial (kNoAllocMaxPartials entries,
// 512 KiB).  Its address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made for
// a context on that device; later calls reuse the cached pointer.  The first
// call per device may load this library's module on that device, so make it
// before any stream capture that is to contain the entry point.  The cached
// address belongs to the device's primary context: it assumes that context
// lives for the whole process (a host program that calls cudaDeviceReset or
// otherwise tears the primary context down must not call this entry point
// afterwards).  Like the other entry points, a call leaves the calling
// thread's current device set to the context's device.
//
// Nothing in the scratch has to start at zero: each call writes the partial
// sum of every CTA it launches before its second kernel reads exactly those
// entries.  Two calls whose kernels overlap in time on the same device (two
// streams, or two contexts on one device) share the scratch and race: order
// them on one stream or with events.
//
// Included into dg_solver.cu after its other entry points; it reads the
// context (dg_ctx) and helpers defined there and changes none of them.
#pragma once

#include <mutex>

namespace {

// CTAs of one residual launch = ceil(nele / elements per CTA); 65536 partial
// sums cover 524288 tetrahedra (8 per CTA) or 1048576 triangles (16 per CTA)
constexpr int kNoAllocMaxPartials = 65536;
constexpr int kNoAllocMaxDevices = 64;

}  // namespace

static __device__ __align__(256) double g_noalloc_partial[kNoAllocMaxPartials];

namespace dg {

// r = b - A x with the FP64 stored blocks, one thread per (element, row), the
// same per-thread summation order as residual_kernel (own block, then the
// faces in order); partial[blockIdx.x] = sum of r^2 over the CTA's rows in a
// fixed order (warp tree, then warps in order).
template <int N, int F, int EPB>
__global__ void __launch_bounds__(EPB* N) residual_sumsq_kernel(const double* __restrict__ blk,
                                                                const int* __restrict__ nbe,
                                                                const double* __restrict__ x,
                                                                const double* __restrict__ b,
                                                                double* __restrict__ r, int64_t B,
                                                                double* __restrict__ partial) {
  constexpr int NW = (EPB * N + 31) / 32;
  __shared__ double xs[EPB][F + 1][N];
  __shared__ int nbs[EPB][F];
  __shared__ double red[NW];
  const int le = threadIdx.x / N, m = threadIdx.x % N;
  const int64_t e = (int64_t)blockIdx.x * EPB + le;
  const bool valid = e < B;
  if (valid && m < F) nbs[le][m] = nbe[e * F + m];
  __syncthreads();
  if (valid) {
    xs[le][0][m] = x[e * N + m];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      int nb = nbs[le][f];
      xs[le][1 + f][m] = nb >= 0 ? x[(int64_t)nb * N + m] : 0.0;
    }
  }
  __syncthreads();
  double q = 0.0;
  if (valid) {
    const double* A = blk + (size_t)e * (F + 1) * N * N;
    double acc = 0.0;
#pragma unroll
    for (int n = 0; n < N; ++n) acc += A[n * N + m] * xs[le][0][n];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (nbs[le][f] >= 0) {
        const double* Af = A + (size_t)(1 + f) * N * N;
#pragma unroll
        for (int n = 0; n < N; ++n) acc += Af[n * N + m] * xs[le][1 + f][n];
      }
    }
    const double res = (b ? b[e * N + m] : 0.0) - acc;
    if (r) r[e * N + m] = res;
    q = res * res;
  }
  q = warp_sum(q);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = q;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// *out = sqrt(sum_i partial[i]) for i < n, one CTA, fixed summation order
__global__ void __launch_bounds__(1024) sumsq_finish_kernel(const double* __restrict__ partial, int n,
                                                            double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  s = warp_sum(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[w];
    *out = sqrt(t);
  }
}

}  // namespace dg

namespace {

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// device address of g_noalloc_partial on the context's device (current)
int noalloc_scratch(dg_ctx* c, double** out) {
  if (c->dev < 0 || c->dev >= kNoAllocMaxDevices)
    return fail(c, DG_ERR_ARG, "dg_residual_norm_noalloc: device ordinal " + std::to_string(c->dev) +
                                   " beyond the " + std::to_string(kNoAllocMaxDevices) + " supported");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[c->dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
    if (e != cudaSuccess || !p)
      return fail(c, DG_ERR_CUDA,
                  std::string("dg_residual_norm_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_ptr[c->dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[c->dev];
  return DG_OK;
}

// Usable partial sums: kNoAllocMaxPartials, or fewer when DG_NOALLOC_MAX_PARTIALS
// holds a smaller positive number (a test hook that can only tighten the
// limit, so the rejection path can be exercised on small meshes).
int64_t noalloc_limit() {
  int64_t lim = kNoAllocMaxPartials;
  const char* v = std::getenv("DG_NOALLOC_MAX_PARTIALS");
  if (v && v[0]) {
    const long long t = std::atoll(v);
    if (t > 0 && t < lim) lim = t;
  }
  return lim;
}

template <int D>
int launch_residual_norm_noalloc(dg_ctx* c, const double* x, const double* b, double* r, double* norm_out,
                                 cudaStream_t st) {
  using E = Elem<D>;
  const int64_t g = ((int64_t)c->B + E::EPB - 1) / E::EPB;
  const int64_t lim = noalloc_limit();
  if (g > lim)
    return fail(c, DG_ERR_ARG,
                "dg_residual_norm_noalloc: " + std::to_string(c->B) + " elements need " + std::to_string(g) +
                    " partial sums; the static scratch holds " + std::to_string(lim) +
                    " (at most " + std::to_string(lim * E::EPB) + " elements)");
  double* partial = nullptr;
  int rc = noalloc_scratch(c, &partial);
  if (rc) return rc;
  if (g) residual_sumsq_kernel<E::N, E::F, E::EPB><<<(unsigned)g, E::EPB * E::N, 0, st>>>(
      c->d_blk, c->d_nbe, x, b, r, c->B, partial);
  sumsq_finish_kernel<<<1, 1024, 0, st>>>(partial, (int)g, norm_out);
  bump(2);
  CKL(c);
  return DG_OK;
}

}  // namespace

// r = b - A x (r may be NULL: norm only; b NULL means b = 0) and
// *norm_out = ||r||_2, both on the device, without allocating: the scratch is
// the static g_noalloc_partial above.
extern "C" int dg_residual_norm_noalloc(dg_ctx* c, const double* x, const double* b, double* r, double* norm_out,
                                        void* stream) {
  if (!c || !x || !norm_out) return set_thread_error(DG_ERR_ARG, "dg_residual_norm_noalloc: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_residual_norm_noalloc: operator not built");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  return c->D == 3 ? launch_residual_norm_noalloc<3>(c, x, b, r, norm_out, st)
                   : launch_residual_norm_noalloc<2>(c, x, b, r, norm_out, st);
}
