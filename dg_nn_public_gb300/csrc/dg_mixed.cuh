// Mixed-precision solve: FP64 iterative refinement around an FP32 inner
// solver.  Included into dg_solver.cu (same translation unit: it uses the
// context and the launch helpers defined there).
//
//   outer (FP64):  r = b - A x;  stop when ||r|| <= tol
//   inner (FP32):  solve A d = r / ||r|| with right-preconditioned flexible
//                  GMRES(m): z_j = M v_j, w = A z_j, classical Gram-Schmidt
//                  (one pass by default, CGS2 optional; FP64 partial sums),
//                  Hessenberg least squares in FP64 on the host; stops when
//                  the Hessenberg residual estimate falls below the inner
//                  target (checked every `chunk` steps)
//   x += ||r|| * d  (FP64)
//
// M is the reference's DG->CG SFC V-cycle in reduced precision: FP32 copies
// of the operator blocks (FGMRES apply) and of the SFC level values, BF16
// copies of the blocks and smoother matrices for the preconditioner's
// smoothing steps, the damped block inverse w A_ee^-1 as smoother (the
// three-sweep Jacobi map as an option) and an exact dense inverse on the
// first SFC level small enough.

namespace {

struct Lev32 {
  int n = 0;
  const int* rowptr = nullptr;   // shared with the FP64 level
  const int* col = nullptr;
  const int* up = nullptr;
  float* val = nullptr;
  float* diag = nullptr;
  float* e = nullptr;
  float* e2 = nullptr;
  float* r = nullptr;
  float* rr = nullptr;
};

struct Mixed {
  bool built = false;
  float* blk = nullptr;
  float* W = nullptr;
  // BF16 copies read by the preconditioner's smoothing / residual kernels
  __nv_bfloat16* blk16 = nullptr;
  __nv_bfloat16* W16 = nullptr;
  // shared-face copies (own blocks, then one block per interior face; 3D
  // bulk-copy kernels): sf = in use for this build; has5 = the five-blocks
  // per element copies above are current (plain kernels, batched solve)
  float* sblk32 = nullptr;
  __nv_bfloat16* sblk16 = nullptr;
  bool sf = false, has5 = false;
  // scaled face blocks S_ef = W_e A_ef (BF16, chunked, four per element) and
  // c = W b of the current preconditioner application; sc = in use
  __nv_bfloat16* scblk16 = nullptr;
  float* chat = nullptr;
  bool sc = false;
  std::vector<Lev32> lev;
  float *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *t5 = nullptr, *t6 = nullptr;
  float *cg1 = nullptr;
  float* r1 = nullptr;   // (nele, ncorner) element P1 restriction scratch
  float *V = nullptr, *Z = nullptr;
  int vcap = 0;
  double* H = nullptr;
  std::vector<cudaGraphExec_t> graphs;   // one per (chunk start) of the inner Arnoldi loop
  // exact coarse solve: dense inverse of SFC level dense_l (-1 = none)
  int dense_l = -1;
  float* dense_inv = nullptr;
  int g_m = 0, g_chunk = 0;
  const float* g_vptr = nullptr;
  // device-side convergence test of the inner FGMRES (givens_check_kernel,
  // with dg_ctx::cond_graph):
  // gv = [cs (m) | sn (m) | g (m+1) | threshold], kdone = first step count
  // whose least-squares residual is below the threshold (0 = none yet);
  // g_kern[chunk][step] = kernels of that step in the chunk's graph; cond =
  // chunk graphs skip the steps after convergence (conditional nodes)
  double* gv = nullptr;
  int* kdone = nullptr;
  // operator-build scratch kept with the context: FP64 smoother blocks and
  // the Gauss-Jordan augmented matrix of the dense coarse level
  double* winv = nullptr;
  double* gj = nullptr;
  // damping factors of the smoothing steps (device copy of
  // dg_ctx::mixed_wscale, read by the smoothing kernels)
  float* d_ws = nullptr;
  size_t gj_cap = 0;
  std::vector<double> gv_host;
  std::vector<std::vector<int>> g_kern;
  std::vector<bool> g_cond;
  bool cond = true;
  // Gram-Schmidt partial sums: one float4 of the vectors per thread,
  // nblk4 = ceil(nonods / 4 / 256) blocks, KMAXV sums per block
  double* part = nullptr;
  int nblk4 = 0;
  // arrival counters of the fused Gram-Schmidt kernels (the last CTA of a
  // launch reduces the partial sums and resets its counter): [0, 32) one per
  // grid row of the dots, [32] the update's norm
  unsigned* gs_cnt = nullptr;
  int* nzflag = nullptr;   // bnonzero_kernel flag of the solve's starting x
  // batched (multi-RHS) solve state (dg_batched.cuh)
  void* batch = nullptr;
  // cluster V-cycle (dg_vcycle_cluster.cuh): CTAs per cluster (0 = the
  // launch chain) and dynamic shared memory per CTA, set per mixed build
  int vc_cs = 0;
  size_t vc_smem = 0;
  // per level: rows per CTA slice, shared-memory word offsets of the slice
  // vectors and of the image's row offsets / diagonal / entries
  std::vector<int> vc_ch, vc_off, vc_rpo, vc_dgo, vc_eno;
  int vc_vwords = 0, vc_iwords = 0;   // words of slice vectors / of one CTA's image
  int32_t* vc_img = nullptr;          // the images of all CTAs
  size_t vc_img_cap = 0;
};

void destroy_batch(void* batch);   // dg_batched.cuh

__global__ void f64_to_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n, double scale) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)(a[k] * scale);
}

// Launch on st, as a programmatic dependent launch when c->use_pdl (the
// kernel's launch overlaps the tail of the preceding kernel; its
// pdl_wait_then_trigger() keeps the data order).  Used for the chain of
// kernels of one inner Arnoldi step.
template <typename... KArgs, typename... Args>
int launch_k(dg_ctx* c, void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
             Args... args) {
  if (grid == 0) return DG_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c->use_pdl ? 1 : 0;
  CK(c, cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
  bump();
  return DG_OK;
}

template <typename... KArgs, typename... Args>
int launch_k2(dg_ctx* c, void (*kern)(KArgs...), dim3 grid, unsigned block, size_t smem, cudaStream_t st,
              Args... args) {
  if (grid.x == 0 || grid.y == 0) return DG_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c->use_pdl ? 1 : 0;
  CK(c, cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
  bump();
  return DG_OK;
}

// e = Ainv r for a small dense level matrix: one warp per row.  The row of
// the fixed inverse is read into registers (float4, up to 20 per lane, i.e.
// n <= 2560 without a second pass) before the programmatic-launch wait, so
// the 21.5 MB read overlaps the previous kernel; after the wait the CTA
// stages r in shared memory (n floats of dynamic shared memory).  With
// rr_src, r is formed there as the pair sums of the finer level's residual
// (r[k] = rr_src[2k] + rr_src[2k+1], zero pad at n_src: the SFC restriction,
// lev_restrict_kernel), so the restriction needs no launch of its own.
__global__ void dense_matvec_kernel(const float* __restrict__ Ainv, const float* __restrict__ r,
                                    float* __restrict__ e, int n, const float* __restrict__ rr_src, int n_src) {
  extern __shared__ __align__(16) float dense_rs[];
  constexpr int PRE = 20;
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  const bool vec = (n & 3) == 0;   // rows 16-byte aligned
  const int n4 = vec ? n / 4 : 0;
  const float* ar = Ainv + (size_t)(row < n ? row : 0) * n;
  float4 a[PRE];
  if (vec) {
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int k4 = lane + 32 * q;
      a[q] = (row < n && k4 < n4) ? reinterpret_cast<const float4*>(ar)[k4] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  } else {
    // scalar loads of columns lane + 32 q, packed four to a register quad
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int k = lane + 128 * q;
      a[q].x = (row < n && k < n) ? ar[k] : 0.0f;
      a[q].y = (row < n && k + 32 < n) ? ar[k + 32] : 0.0f;
      a[q].z = (row < n && k + 64 < n) ? ar[k + 64] : 0.0f;
      a[q].w = (row < n && k + 96 < n) ? ar[k + 96] : 0.0f;
    }
  }
  pdl_wait_then_trigger();
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    dense_rs[k] = rr_src ? rr_src[2 * k] + (2 * k + 1 < n_src ? rr_src[2 * k + 1] : 0.0f) : r[k];
  __syncthreads();
  if (row >= n) return;
  const float* rs = dense_rs;
  float s = 0.0f;
  if (vec) {
    const float4* rs4 = reinterpret_cast<const float4*>(rs);
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int k4 = lane + 32 * q;
      if (k4 < n4) {
        const float4 rv = rs4[k4];
        float t = a[q].x * rv.x;
        t = __fmaf_rn(a[q].y, rv.y, t);
        t = __fmaf_rn(a[q].z, rv.z, t);
        t = __fmaf_rn(a[q].w, rv.w, t);
        s += t;
      }
    }
    for (int k4 = lane + 32 * PRE; k4 < n4; k4 += 32) {
      const float4 av = reinterpret_cast<const float4*>(ar)[k4], rv = rs4[k4];
      float t = av.x * rv.x;
      t = __fmaf_rn(av.y, rv.y, t);
      t = __fmaf_rn(av.z, rv.z, t);
      t = __fmaf_rn(av.w, rv.w, t);
      s += t;
    }
  } else {
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int k = lane + 128 * q;
      if (k < n) s = __fmaf_rn(a[q].x, rs[k], s);
      if (k + 32 < n) s = __fmaf_rn(a[q].y, rs[k + 32], s);
      if (k + 64 < n) s = __fmaf_rn(a[q].z, rs[k + 64], s);
      if (k + 96 < n) s = __fmaf_rn(a[q].w, rs[k + 96], s);
    }
    for (int k = lane + 128 * PRE; k < n; k += 32) s = __fmaf_rn(ar[k], rs[k], s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) e[row] = s;
}

// SFC-level Jacobi sweep (lev_jacobi_kernel, FP32, LPR lanes per row) whose
// input iterate is formed on the fly from the neighbouring level, so that
// the transfer between levels needs no launch of its own:
//   MODE 1 (restriction in): e_in[j] = ea[2j] + ea[2j+1] and
//     r[i] = eb[2i] + eb[2i+1] (zero pad at n_src; lev_restrict_kernel),
//     r is stored for the level's later sweeps;
//   MODE 2 (prolongation in): e_in[j] = ea[j] + eb[up[j]]
//     (lev_prolong_kernel), r read as given.
// Then rr = r - A e_in, e_out = e_in + rr / diag * w, rr_out = rr (if set):
// the same operations as the transfer launch followed by the sweep.
template <int MODE>
__global__ void lev_jacobi_x_kernel(const int* __restrict__ rowptr, const int* __restrict__ col,
                                    const float* __restrict__ val, const float* __restrict__ diag,
                                    const float* __restrict__ ea, const float* __restrict__ eb,
                                    const int* __restrict__ up, int n_src, float* __restrict__ r,
                                    float* __restrict__ e_out, float* __restrict__ rr_out, int n, float w) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / LPR, lane = t % LPR;
  constexpr int PRE = 4;
  int k0 = 0, k1 = 0;
  int cpre[PRE];
  float vpre[PRE];
  if (i < n) {
    k0 = rowptr[i] + lane;
    k1 = rowptr[i + 1];
  }
#pragma unroll
  for (int q = 0; q < PRE; ++q) {
    const int k = k0 + q * LPR;
    cpre[q] = k < k1 ? col[k] : 0;
    vpre[q] = k < k1 ? val[k] : 0.0f;
  }
  pdl_wait_then_trigger();
  auto ein = [&](int j) -> float {
    if (MODE == 1) return ea[2 * j] + (2 * j + 1 < n_src ? ea[2 * j + 1] : 0.0f);
    return ea[j] + eb[up[j]];
  };
  float s = 0.0f;
  if (i < n) {
#pragma unroll
    for (int q = 0; q < PRE; ++q)
      if (k0 + q * LPR < k1) s = __fmaf_rn(vpre[q], ein(cpre[q]), s);
    for (int k = k0 + PRE * LPR; k < k1; k += LPR) s = __fmaf_rn(val[k], ein(col[k]), s);
  }
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
  if (i >= n || lane != 0) return;
  float ri;
  if (MODE == 1) {
    ri = eb[2 * i] + (2 * i + 1 < n_src ? eb[2 * i + 1] : 0.0f);
    r[i] = ri;
  } else {
    ri = r[i];
  }
  const float rr = ri - s;
  e_out[i] = __fmaf_rn(rr / diag[i], w, ein(i));
  if (rr_out) rr_out[i] = rr;
}

// ---------------------------------------------------------------------------
// BF16 blocks of P3 tetrahedra (20x20) in a chunked layout for wide loads:
// the block's columns 0-7, 8-15 and 16-19 form three chunks, each stored as
// [row m][column within the chunk] (8, 8 and 4 wide).  Row m of a block is
// then two 16-byte loads and one 8-byte load instead of twenty 2-byte ones,
// which is what keeps enough bytes in flight to stream the blocks at HBM
// rate.  Chunk offsets (in elements): 0, 160, 320; a block is 400 elements
// (800 bytes), so every block and chunk starts on a 16-byte boundary.
constexpr int kC20Off1 = 160, kC20Off2 = 320;

// destination index of entry (row m, column n) of a block in that layout
__host__ __device__ __forceinline__ int chunk20_index(int m, int n) {
  return n < 8 ? m * 8 + n : (n < 16 ? kC20Off1 + m * 8 + (n - 8) : kC20Off2 + m * 4 + (n - 16));
}

// a: nblock column-major FP64 (or FP32) blocks [blk][n][m] -> chunked BF16 blocks
template <typename ST>
__global__ void convert_f64_bf16_chunk20_kernel(const ST* __restrict__ a, __nv_bfloat16* __restrict__ b,
                                                int64_t nblock) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nblock * 400) return;
  const int64_t blk = k / 400;
  const int rem = (int)(k - blk * 400);
  const int n = rem / 20, m = rem % 20;
  b[blk * 400 + chunk20_index(m, n)] = __float2bfloat16_rn((float)a[k]);
}

struct Row20 {
  uint4 a, b;
  uint2 c;
};

__device__ __forceinline__ Row20 load_row20(const __nv_bfloat16* __restrict__ blk, int m) {
  Row20 q;
  q.a = __ldg(reinterpret_cast<const uint4*>(blk) + m);
  q.b = __ldg(reinterpret_cast<const uint4*>(blk + kC20Off1) + m);
  q.c = __ldg(reinterpret_cast<const uint2*>(blk + kC20Off2) + m);
  return q;
}

__device__ __forceinline__ Row20 zero_row20() {
  Row20 q;
  q.a = make_uint4(0u, 0u, 0u, 0u);
  q.b = q.a;
  q.c = make_uint2(0u, 0u);
  return q;
}

// the two BF16 values of a 32-bit word (low half = lower column), exactly
__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// acc + sum_n row[n] * v[n], n = 0..19 in order (one FMA chain)
__device__ __forceinline__ float dot_row20(const Row20& q, const float* v, float acc) {
  const uint32_t w[10] = {q.a.x, q.a.y, q.a.z, q.a.w, q.b.x, q.b.y, q.b.z, q.b.w, q.c.x, q.c.y};
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    acc = fmaf(bf_lo(w[i]), v[2 * i], acc);
    acc = fmaf(bf_hi(w[i]), v[2 * i + 1], acc);
  }
  return acc;
}

// residual_kernel<20, 4, EPB, bf16, float, float> on the chunked layout
// (same flags, same per-thread summation order, so the same results): the
// block rows (and the smoother row) are loaded into registers before the
// CTA waits for its x gather, so all of an element's loads are in flight
// together.
template <int EPB>
__global__ void __launch_bounds__(EPB * 20) residual_bf16c20_kernel(
    const __nv_bfloat16* __restrict__ blk, const __nv_bfloat16* __restrict__ W, const int* __restrict__ nbe,
    const float* __restrict__ x, const float* __restrict__ b, float* __restrict__ r, float* __restrict__ x_out,
    int64_t B, int flags, const float* __restrict__ P, float* __restrict__ r1, const float* __restrict__ wsp) {
  const float wscale = wsp ? *wsp : 1.0f;
  constexpr int N = 20, F = 4;
  __shared__ float xs[EPB][F + 1][N];
  __shared__ float rs[EPB][N];
  __shared__ float Ps[N * F];   // P converted once per CTA, not per use
  __shared__ int nbs[EPB][F];
  const int le = threadIdx.x / N, m = threadIdx.x % N;
  const int64_t e = (int64_t)blockIdx.x * EPB + le;
  const bool valid = e < B;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  if (valid && m < F) nbs[le][m] = nbe[e * F + m];
  if (flags & RF_RESTRICT)
    for (int i = threadIdx.x; i < N * F; i += EPB * N) Ps[i] = (float)P[i];
  __syncthreads();
  Row20 q[F + 1];
  Row20 wq = zero_row20();
  const __nv_bfloat16* A = blk + (size_t)e * (F + 1) * N * N;
  if (valid && !zerox) {
    q[0] = load_row20(A, m);
#pragma unroll
    for (int f = 0; f < F; ++f) q[1 + f] = nbs[le][f] >= 0 ? load_row20(A + (1 + f) * N * N, m) : zero_row20();
  }
  if (valid && smooth) wq = load_row20(W + (size_t)e * N * N, m);
  if (valid && !zerox) {
    xs[le][0][m] = x[e * N + m];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const int nb = nbs[le][f];
      xs[le][1 + f][m] = nb >= 0 ? x[(int64_t)nb * N + m] : 0.0f;
    }
  }
  __syncthreads();
  float acc = 0.0f;
  if (valid && !zerox) {
    acc = dot_row20(q[0], xs[le][0], acc);
#pragma unroll
    for (int f = 0; f < F; ++f)
      if (nbs[le][f] >= 0) acc = dot_row20(q[1 + f], xs[le][1 + f], acc);
  }
  float res = 0.0f;
  if (valid) {
    res = (b ? b[e * N + m] : 0.0f) - acc;
    if (r) r[e * N + m] = (flags & RF_NEG) ? -res : res;
  }
  if (flags & RF_RESTRICT) {
    rs[le][m] = res;
    __syncthreads();
    constexpr int NC = F;
    if (valid && m < NC) {
      float s = 0.0f;
#pragma unroll
      for (int n = 0; n < N; ++n) s += Ps[n * NC + m] * rs[le][n];
      r1[e * NC + m] = s;
    }
  }
  if (smooth) {
    rs[le][m] = res;
    __syncthreads();
    if (valid) x_out[e * N + m] = (zerox ? 0.0f : xs[le][0][m]) + wscale * dot_row20(wq, rs[le], 0.0f);
  }
}

// ---------------------------------------------------------------------------
// FP32 blocks of P3 tetrahedra in the matching chunked layout: five chunks
// of four columns, each [row m][column within the chunk], so row m of a
// block is five 16-byte loads (chunk c at byte 320 c + 16 m).
__host__ __device__ __forceinline__ int chunk20f_index(int m, int n) { return (n >> 2) * 80 + m * 4 + (n & 3); }

template <typename ST>
__global__ void convert_f64_f32_chunk20_kernel(const ST* __restrict__ a, float* __restrict__ b, int64_t nblock) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nblock * 400) return;
  const int64_t blk = k / 400;
  const int rem = (int)(k - blk * 400);
  const int n = rem / 20, m = rem % 20;
  b[blk * 400 + chunk20f_index(m, n)] = (float)a[k];
}

struct Row20f {
  float4 c[5];
};

// one block row in shared memory, per storage type, and its dot product with
// v[0..19] as one FMA chain in column order (the order of residual_kernel)
template <typename MT>
struct Chunk20;

template <>
struct Chunk20<__nv_bfloat16> {
  using Row = Row20;
  static constexpr int BlockBytes = 800;
  static __device__ __forceinline__ Row lds(const unsigned char* blk, int m) {
    Row q;
    q.a = *reinterpret_cast<const uint4*>(blk + 16 * m);
    q.b = *reinterpret_cast<const uint4*>(blk + 2 * kC20Off1 + 16 * m);
    q.c = *reinterpret_cast<const uint2*>(blk + 2 * kC20Off2 + 8 * m);
    return q;
  }
  static __device__ __forceinline__ float dot(const Row& q, const float* v, float acc) {
    return dot_row20(q, v, acc);
  }
  // acc + sum_n blk[n][m] * v[n], n = 0..19 in order: row m of the
  // transposed block (column m of the stored one), same FMA order as dot
  static __device__ __forceinline__ float dot_col(const unsigned char* blk, int m, const float* v, float acc) {
    const int base = m < 8 ? 2 * m : (m < 16 ? 2 * kC20Off1 + 2 * (m - 8) : 2 * kC20Off2 + 2 * (m - 16));
    const int step = m < 16 ? 16 : 8;
    const unsigned char* p = blk + base;
#pragma unroll
    for (int n = 0; n < 20; ++n) {
      const uint32_t h = *reinterpret_cast<const unsigned short*>(p + n * step);
      acc = fmaf(__uint_as_float(h << 16), v[n], acc);
    }
    return acc;
  }
};

template <>
struct Chunk20<float> {
  using Row = Row20f;
  static constexpr int BlockBytes = 1600;
  static __device__ __forceinline__ Row lds(const unsigned char* blk, int m) {
    Row q;
#pragma unroll
    for (int c = 0; c < 5; ++c) q.c[c] = *reinterpret_cast<const float4*>(blk + 320 * c + 16 * m);
    return q;
  }
  static __device__ __forceinline__ float dot(const Row& q, const float* v, float acc) {
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      acc = fmaf(q.c[c].x, v[4 * c], acc);
      acc = fmaf(q.c[c].y, v[4 * c + 1], acc);
      acc = fmaf(q.c[c].z, v[4 * c + 2], acc);
      acc = fmaf(q.c[c].w, v[4 * c + 3], acc);
    }
    return acc;
  }
  static __device__ __forceinline__ float dot_col(const unsigned char* blk, int m, const float* v, float acc) {
    const float* p = reinterpret_cast<const float*>(blk + 320 * (m >> 2) + 4 * (m & 3));
#pragma unroll
    for (int n = 0; n < 20; ++n) acc = fmaf(p[4 * n], v[n], acc);
    return acc;
  }
};

// ---------------------------------------------------------------------------
// Shared face blocks.  The SIP operator is symmetric (A_{e,nb} = A_{nb,e}^T
// to rounding; the face penalty uses the face's own area from either side),
// so the reduced-precision copies store each interior face once: an array of
// B own blocks followed by one block per interior face, that face's block of
// its lower-numbered element (rows of that element, columns of the
// neighbour).  fref5[e][0] = 2 e (own block), fref5[e][1 + f] = 2 (B + id) for
// a face e owns, 2 (B + id) + 1 for a face its neighbour owns (read
// transposed), -1 on the boundary.  The FP32 apply and the BF16 steps then
// stream (B + #interior faces) blocks instead of 5 B.
//
// dst block i <- src block (idx[i]), converted into the chunked layout
template <typename MT>
__global__ void convert_gather_chunk20_kernel(const double* __restrict__ a, const int* __restrict__ idx,
                                              MT* __restrict__ b, int64_t nblock) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nblock * 400) return;
  const int64_t blk = k / 400;
  const int rem = (int)(k - blk * 400);
  const int n = rem / 20, m = rem % 20;
  const float v = (float)a[(int64_t)idx[blk] * 400 + rem];
  if constexpr (std::is_same<MT, float>::value)
    b[blk * 400 + chunk20f_index(m, n)] = v;
  else
    b[blk * 400 + chunk20_index(m, n)] = __float2bfloat16_rn(v);
}

// ---------------------------------------------------------------------------
// The residual / smoothing step of residual_kernel<20, 4, ., MT, float,
// float> as a persistent kernel that streams the blocks with the Tensor
// Memory Accelerator: MINB CTAs per SM walk the element groups
// g = blockIdx.x, blockIdx.x + gridDim.x, ...; a group's EPB elements are
// consecutive, so their blocks (EPB * 5 blocks) and, with WITH_W, their
// smoother matrices are two contiguous bulk copies (cp.async.bulk,
// completion on an mbarrier) into a ring of S shared-memory stages.  While
// group k is computed, groups k+1 .. k+S-1 are in flight, and the x / b
// gathers of group k+1 (ordinary loads, from L2) are issued before group k's
// wait, so neither the block stream nor the gathers stall on a per-CTA round
// trip.  Same arithmetic in the same order as residual_kernel, so the same
// results.  Every mbarrier wait is bounded: on time-out the kernel sets
// *err = 3, waits (bounded) for its own copies in flight and returns.
template <typename MT, int EPB, bool WITH_W>
struct TmaGroup {
  static constexpr int BlockBytes = Chunk20<MT>::BlockBytes;
  static constexpr int ABytes = EPB * 5 * BlockBytes;
  static constexpr int WBytes = WITH_W ? EPB * BlockBytes : 0;
  static constexpr int StageBytes = ABytes + WBytes;
};
constexpr uint32_t kTmaSpinLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  uint64_t state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state)
               : "r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  (void)state;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; false on time-out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kTmaSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// L2 policy "evict first" for data read once per pass (the block stream), so
// that it does not push the vectors and the SFC level matrices out of L2
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ void bulk_copy_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                   uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

template <typename MT, int EPB, int S, int MINB, bool WITH_W, bool SF>
__global__ void __launch_bounds__(EPB * 20, MINB) residual_tma_kernel(
    const MT* __restrict__ blk, const MT* __restrict__ W, const int* __restrict__ nbe, const float* __restrict__ x,
    const float* __restrict__ b, float* __restrict__ r, float* __restrict__ x_out, int64_t B, int flags,
    const float* __restrict__ P, float* __restrict__ r1, int* __restrict__ err, const int* __restrict__ fref5,
    const float* __restrict__ wsp, float* __restrict__ c_out) {
  const float wscale = wsp ? *wsp : 1.0f;
  constexpr int N = 20, F = 4;
  using G = TmaGroup<MT, EPB, WITH_W>;
  using C = Chunk20<MT>;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  __shared__ __align__(8) uint64_t bar[S];
  __shared__ float xs[EPB][F + 1][N];
  __shared__ float rs[EPB][N];
  __shared__ float Ps[N][F];
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int le = tid / N, m = tid % N;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = WITH_W && (flags & RF_SMOOTH);
  const bool restrict_ = flags & RF_RESTRICT;
  const int64_t ngroups = (B + EPB - 1) / EPB;
  const int64_t stride = gridDim.x;
  for (int t = tid; t < N * F; t += EPB * N) Ps[t / F][t % F] = P ? (float)P[t] : 0.0f;
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const uint64_t pol = l2_evict_first_policy();
  const bool hint = flags & RF_STREAM_HINT;
  const int lane = tid & 31;
  // Shared-face mode, stage layout: the group's own blocks in slots
  // 0 .. ne-1 (one copy), the face blocks the group's elements own from slot
  // EPB on (their ids are consecutive: one copy), then one slot per face
  // block owned by a neighbour (one copy each, read transposed).  For face
  // (le, f) = lane 4 le + f: fslot[stage][lane] = its slot, bit lane of
  // tmask[stage] = read transposed.
  __shared__ uint32_t tmask[S];
  __shared__ unsigned char fslot[S][32];
  static_assert(!SF || 4 * EPB <= 32, "one lane per face of a group");
  // warp 0, shared-face mode: fref5 entry of face (lane / 4, lane % 4) of
  // the next group to be issued (loaded one group ahead)
  int fr_a = -1;
  auto load_fr = [&](int64_t k) {
    fr_a = -1;
    const int64_t g = blockIdx.x + k * stride;
    if (!SF || zerox || g >= ngroups) return;
    const int64_t e0 = g * EPB;
    const int nf4 = 4 * (int)((B - e0) < EPB ? (B - e0) : EPB);
    if (lane < nf4) fr_a = fref5[(e0 + lane / 4) * 5 + 1 + (lane & 3)];
  };
  // copies of the CTA's k-th group go to stage k % S, phase parity (k / S) & 1;
  // called by all of warp 0 (the group test is uniform across the warp)
  auto issue = [&](int64_t k) {
    const int64_t g = blockIdx.x + k * stride;
    if (g >= ngroups) return;
    const int64_t e0 = g * EPB;
    const uint32_t ne = (uint32_t)((B - e0) < EPB ? (B - e0) : EPB);
    const uint32_t bw = smooth ? ne * (uint32_t)G::BlockBytes : 0u;
    unsigned char* sp = tma_smem + (size_t)(k % S) * G::StageBytes;
    uint64_t* br = &bar[k % S];
    if constexpr (SF) {
      constexpr uint32_t BB = G::BlockBytes;
      const bool owned = fr_a >= 0 && !(fr_a & 1), trans = fr_a >= 0 && (fr_a & 1);
      const uint32_t bi = (uint32_t)fr_a >> 1;   // block index in the shared array
      const uint32_t mo = __ballot_sync(0xffffffffu, owned);
      const uint32_t mt = __ballot_sync(0xffffffffu, trans);
      const uint32_t bi0 = __reduce_min_sync(0xffffffffu, owned ? bi : 0xffffffffu);
      const uint32_t no = __popc(mo), nt = __popc(mt);
      uint32_t slot = owned ? EPB + (bi - bi0) : EPB + no + __popc(mt & ((1u << lane) - 1u));
      if (fr_a >= 0 && slot >= 5u * EPB) {   // face table not in owner order: report, stay in the stage
        atomicExch(err, 5);
        slot = 0;
      }
      fslot[k % S][lane] = (unsigned char)(fr_a >= 0 ? slot : 0u);
      if (lane == 0) {
        tmask[k % S] = mt;
        const uint32_t bo = zerox ? 0u : ne * BB;
        mbar_expect_tx(br, bo + (no + nt) * BB + bw);
        // own blocks, transposed reads and smoother matrices are their last
        // use in this pass (evict first); a face block read as stored is read
        // again, transposed, by the neighbour shortly after, so it stays in L2
        if (hint) {
          if (bo) bulk_copy_g2s_hint(sp, blk + e0 * 400, bo, br, pol);
          if (bw) bulk_copy_g2s_hint(sp + G::ABytes, W + e0 * 400, bw, br, pol);
        } else {
          if (bo) bulk_copy_g2s(sp, blk + e0 * 400, bo, br);
          if (bw) bulk_copy_g2s(sp + G::ABytes, W + e0 * 400, bw, br);
        }
        if (no) bulk_copy_g2s(sp + (size_t)EPB * BB, blk + (int64_t)bi0 * 400, no * BB, br);
      }
      __syncwarp();
      if (trans) {
        const MT* src = blk + (int64_t)bi * 400;
        unsigned char* dst = sp + (size_t)slot * BB;
        if (hint) bulk_copy_g2s_hint(dst, src, BB, br, pol);
        else bulk_copy_g2s(dst, src, BB, br);
      }
    } else if (lane == 0) {
      const uint32_t ba = zerox ? 0u : ne * 5u * G::BlockBytes;
      mbar_expect_tx(br, ba + bw);
      if (hint) {
        if (ba) bulk_copy_g2s_hint(sp, blk + e0 * 2000, ba, br, pol);
        if (bw) bulk_copy_g2s_hint(sp + G::ABytes, W + e0 * 400, bw, br, pol);
      } else {
        if (ba) bulk_copy_g2s(sp, blk + e0 * 2000, ba, br);
        if (bw) bulk_copy_g2s(sp + G::ABytes, W + e0 * 400, bw, br);
      }
    }
  };
  if (tid < 32) {
    for (int k = 0; k < S; ++k) {
      load_fr(k);
      issue(k);
    }
    load_fr(S);
  }
  // register prefetch of the gathers of the next group
  auto load_nb = [&](int64_t g) {
    const int64_t e = g * EPB + le;
    return (g < ngroups && e < B) ? reinterpret_cast<const int4*>(nbe)[e] : make_int4(-1, -1, -1, -1);
  };
  int4 nb_cur = load_nb(blockIdx.x);
  // blocks, smoother matrices and neighbour table are fixed during a solve:
  // the copies above may run ahead of the preceding kernel; x and b may not
  pdl_wait_then_trigger();
  float x_own = 0.0f, x_nb[F] = {0.0f, 0.0f, 0.0f, 0.0f}, b_cur = 0.0f;
  auto load_x = [&](int64_t g, const int4& nb) {
    const int64_t e = g * EPB + le;
    const bool ok = g < ngroups && e < B;
    x_own = (ok && !zerox) ? x[e * N + m] : 0.0f;
    const int nbv[F] = {nb.x, nb.y, nb.z, nb.w};
#pragma unroll
    for (int f = 0; f < F; ++f) x_nb[f] = (ok && !zerox && nbv[f] >= 0) ? x[(int64_t)nbv[f] * N + m] : 0.0f;
    b_cur = (ok && b) ? b[e * N + m] : 0.0f;
  };
  load_x(blockIdx.x, nb_cur);
  int4 nb_next = load_nb(blockIdx.x + stride);
  int64_t k = 0;
  for (int64_t g = blockIdx.x; g < ngroups; g += stride, ++k) {
    const int64_t e = g * EPB + le;
    const bool valid = e < B;
    const int nbv[F] = {nb_cur.x, nb_cur.y, nb_cur.z, nb_cur.w};
    xs[le][0][m] = x_own;
#pragma unroll
    for (int f = 0; f < F; ++f) xs[le][1 + f][m] = x_nb[f];
    const float bb = b_cur;
    // gathers of the next group, in flight during this group's work
    nb_cur = nb_next;
    load_x(g + stride, nb_cur);
    nb_next = load_nb(g + 2 * stride);
    const int s = (int)(k % S);
    if (!mbar_wait_bounded(&bar[s], (uint32_t)((k / S) & 1))) {
      atomicExch(err, 3);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    const unsigned char* sp = tma_smem + (size_t)s * G::StageBytes;
    float acc = 0.0f;
    if (valid && !zerox) {
      const unsigned char* Ae = sp + (size_t)le * (SF ? 1 : 5) * G::BlockBytes;
      const uint32_t tm = SF ? tmask[s] >> (4 * le) : 0u;
      acc = C::dot(C::lds(Ae, m), xs[le][0], acc);
#pragma unroll
      for (int f = 0; f < F; ++f)
        if (nbv[f] >= 0) {
          const unsigned char* Af =
              SF ? sp + (size_t)fslot[s][4 * le + f] * G::BlockBytes : Ae + (1 + f) * G::BlockBytes;
          if (SF && ((tm >> f) & 1u))
            acc = C::dot_col(Af, m, xs[le][1 + f], acc);
          else
            acc = C::dot(C::lds(Af, m), xs[le][1 + f], acc);
        }
    }
    float res = 0.0f;
    if (valid) {
      res = bb - acc;
      if (r) r[e * N + m] = (flags & RF_NEG) ? -res : res;
    }
    if (restrict_ || smooth) {
      rs[le][m] = res;
      __syncthreads();
      if (restrict_ && valid && m < F) {
        float t = 0.0f;
#pragma unroll
        for (int n = 0; n < N; ++n) t += Ps[n][m] * rs[le][n];
        r1[e * F + m] = t;
      }
      if (smooth && valid) {
        const float wr = C::dot(C::lds(sp + G::ABytes + (size_t)le * G::BlockBytes, m), rs[le], 0.0f);
        x_out[e * N + m] = (zerox ? 0.0f : xs[le][0][m]) + wscale * wr;
        if (c_out) c_out[e * N + m] = wr;   // W_e res, kept for the scaled-face steps
      }
    }
    __syncthreads();   // stage s and xs / rs free again
    if (tid < 32) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(k + S);
      if (SF) load_fr(k + S + 1);
    }
  }
  if (abort_flag && tid == 0) {
    // drain this CTA's copies still in flight (groups k .. k+S-1), bounded
    for (int64_t j = k; j < k + S; ++j) {
      if (blockIdx.x + j * stride >= ngroups) break;
      (void)mbar_wait_bounded(&bar[j % S], (uint32_t)((j / S) & 1));
    }
  }
}

// sf: shared-face block array (blk = own blocks + one block per interior
// face, addressed through c->d_fref5); otherwise five blocks per element
template <typename MT, int EPB, int S, int MINB, bool WITH_W>
int launch_tma(dg_ctx* c, const MT* blk, const MT* W, const float* x, const float* b, float* r, float* x_out,
               int flags, float* r1, cudaStream_t st, bool sf, const float* wscale = nullptr,
               float* c_out = nullptr) {
  if (c->l2_hint) flags |= RF_STREAM_HINT;
  const int64_t ngroups = (c->B + EPB - 1) / EPB;
  const unsigned g = (unsigned)std::min<int64_t>(ngroups, (int64_t)c->nsm * MINB);
  const size_t smem = (size_t)S * TmaGroup<MT, EPB, WITH_W>::StageBytes;
  if (sf)
    return launch_k(c, residual_tma_kernel<MT, EPB, S, MINB, WITH_W, true>, g, EPB * 20, smem, st, blk, W,
                    (const int*)c->d_nbe, x, b, r, x_out, (int64_t)c->B, flags, (const float*)c->d_P32, r1,
                    (int*)c->d_err, (const int*)c->d_fref5, wscale, c_out);
  return launch_k(c, residual_tma_kernel<MT, EPB, S, MINB, WITH_W, false>, g, EPB * 20, smem, st, blk, W,
                  (const int*)c->d_nbe, x, b, r, x_out, (int64_t)c->B, flags, (const float*)c->d_P32, r1,
                  (int*)c->d_err, (const int*)nullptr, wscale, c_out);
}

template <typename MT, int EPB, int S, int MINB, bool WITH_W>
int set_tma_smem(dg_ctx* c) {
  const int bytes = S * TmaGroup<MT, EPB, WITH_W>::StageBytes;
  CK(c, cudaFuncSetAttribute(residual_tma_kernel<MT, EPB, S, MINB, WITH_W, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  CK(c, cudaFuncSetAttribute(residual_tma_kernel<MT, EPB, S, MINB, WITH_W, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  return DG_OK;
}

// BF16 preconditioner step (3D) through the bulk-copy kernel.  Launch shapes
// (elements per group, stages, CTAs per SM); c2 sweep: (8,5,1) 49.3 us,
// (8,3,1) 49.2, (8,2,2) 41.2, (4,2,4) 41.3, (4,2,5) 41.6, (4,1,8) 41.5,
// (6,2,3) 40.7 -- several CTAs per SM hide the per-group round trip that
// one CTA per SM cannot.
constexpr int kTmaVariants = 3;

int launch_bf16_tma(dg_ctx* c, Mixed& M, const float* x, const float* b, float* r, float* x_out, int flags,
                    cudaStream_t st, const float* ws = nullptr, float* c_out = nullptr) {
  const __nv_bfloat16* A = M.sf ? M.sblk16 : M.blk16;
  switch (c->tma_variant) {
    case 1:
      return launch_tma<__nv_bfloat16, 8, 2, 2, true>(c, A, M.W16, x, b, r, x_out, flags, M.r1, st, M.sf, ws, c_out);
    case 2:
      return launch_tma<__nv_bfloat16, 4, 2, 4, true>(c, A, M.W16, x, b, r, x_out, flags, M.r1, st, M.sf, ws, c_out);
    default:
      return launch_tma<__nv_bfloat16, 6, 2, 3, true>(c, A, M.W16, x, b, r, x_out, flags, M.r1, st, M.sf, ws, c_out);
  }
}

// ---------------------------------------------------------------------------
// Smoothing on scaled face blocks.  With W_e = w A_ee^-1 the damped block
// Jacobi step x' = x + s W_e (b - A x) is, element by element,
//   x'_e = x_e + s (c_e - w x_e - sum_f S_ef x_nb(f)),
// c_e = W_e b_e and S_ef = W_e A_ef: the self block becomes w I.  A step then
// streams the four face blocks of an element (BF16, chunked layout, 3,200
// bytes) instead of its five blocks and its smoother matrix (4,800 bytes).
// c is formed by the zero-start step of each preconditioner application
// (c_out of residual_tma_kernel) and serves every later step on the same
// right-hand side.  The same persistent bulk-copy ring as
// residual_tma_kernel: MINB CTAs per SM, groups of EPB consecutive elements,
// S stages; blocks are copied before the programmatic-launch wait (they are
// fixed during a solve), x and c gathered after it.
constexpr int kScVariants = 4;

// S_ef = W_e A_ef for the four faces of every element, in FP32 from the FP32
// smoother matrices (column-major, W(m, n) at [n * 20 + m]) and the FP64
// blocks, rounded once to BF16 in the chunked layout: one CTA of 400 threads
// per element, thread (m, n) forms entry (m, n) of each face block as one
// FMA chain over k.
__global__ void __launch_bounds__(400) scaled_faces_kernel(const float* __restrict__ W,
                                                           const double* __restrict__ blk,
                                                           __nv_bfloat16* __restrict__ out, int64_t B) {
  constexpr int N = 20, F = 4;
  __shared__ float Ws[N * N];
  __shared__ float As[F][N * N];
  const int64_t e = blockIdx.x;
  const int t = threadIdx.x;
  Ws[t] = W[e * N * N + t];
#pragma unroll
  for (int f = 0; f < F; ++f) As[f][t] = (float)blk[(e * (F + 1) + 1 + f) * N * N + t];
  __syncthreads();
  const int m = t % N, n = t / N;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) acc = fmaf(Ws[k * N + m], As[f][n * N + k], acc);
    out[(e * F + f) * N * N + chunk20_index(m, n)] = __float2bfloat16_rn(acc);
  }
}

template <int EPB, int S, int MINB>
__global__ void __launch_bounds__(EPB * 20, MINB) smooth_scaled_tma_kernel(
    const __nv_bfloat16* __restrict__ sblk, const int* __restrict__ nbe, const float* __restrict__ x,
    const float* __restrict__ cv, float* __restrict__ x_out, int64_t B, float w, const float* __restrict__ wsp,
    int* __restrict__ err, int flags) {
  constexpr int N = 20, F = 4, BB = Chunk20<__nv_bfloat16>::BlockBytes;
  constexpr uint32_t GroupBytes = EPB * F * BB;
  using C = Chunk20<__nv_bfloat16>;
  const float wscale = wsp ? *wsp : 1.0f;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  __shared__ __align__(8) uint64_t bar[S];
  __shared__ float xs[EPB][F][N];
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int le = tid / N, m = tid % N;
  const int64_t ngroups = (B + EPB - 1) / EPB;
  const int64_t stride = gridDim.x;
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const uint64_t pol = l2_evict_first_policy();
  const bool hint = flags & RF_STREAM_HINT;
  auto issue = [&](int64_t k) {   // thread 0: group k of this CTA -> stage k % S
    const int64_t g = blockIdx.x + k * stride;
    if (g >= ngroups) return;
    const int64_t e0 = g * EPB;
    const uint32_t ne = (uint32_t)((B - e0) < EPB ? (B - e0) : EPB);
    unsigned char* sp = tma_smem + (size_t)(k % S) * GroupBytes;
    uint64_t* br = &bar[k % S];
    mbar_expect_tx(br, ne * F * BB);
    if (hint) bulk_copy_g2s_hint(sp, sblk + e0 * F * 400, ne * F * BB, br, pol);
    else bulk_copy_g2s(sp, sblk + e0 * F * 400, ne * F * BB, br);
  };
  if (tid == 0)
    for (int k = 0; k < S; ++k) issue(k);
  auto load_nb = [&](int64_t g) {
    const int64_t e = g * EPB + le;
    return (g < ngroups && e < B) ? reinterpret_cast<const int4*>(nbe)[e] : make_int4(-1, -1, -1, -1);
  };
  int4 nb_cur = load_nb(blockIdx.x);
  pdl_wait_then_trigger();
  float x_own = 0.0f, c_own = 0.0f, x_nb[F] = {0.0f, 0.0f, 0.0f, 0.0f};
  auto load_x = [&](int64_t g, const int4& nb) {
    const int64_t e = g * EPB + le;
    const bool ok = g < ngroups && e < B;
    x_own = ok ? x[e * N + m] : 0.0f;
    c_own = ok ? cv[e * N + m] : 0.0f;
    const int nbv[F] = {nb.x, nb.y, nb.z, nb.w};
#pragma unroll
    for (int f = 0; f < F; ++f) x_nb[f] = (ok && nbv[f] >= 0) ? x[(int64_t)nbv[f] * N + m] : 0.0f;
  };
  load_x(blockIdx.x, nb_cur);
  int4 nb_next = load_nb(blockIdx.x + stride);
  int64_t k = 0;
  for (int64_t g = blockIdx.x; g < ngroups; g += stride, ++k) {
    const int64_t e = g * EPB + le;
    const bool valid = e < B;
    const int nbv[F] = {nb_cur.x, nb_cur.y, nb_cur.z, nb_cur.w};
#pragma unroll
    for (int f = 0; f < F; ++f) xs[le][f][m] = x_nb[f];
    const float xo = x_own, co = c_own;
    nb_cur = nb_next;
    load_x(g + stride, nb_cur);
    nb_next = load_nb(g + 2 * stride);
    const int s = (int)(k % S);
    if (!mbar_wait_bounded(&bar[s], (uint32_t)((k / S) & 1))) {
      atomicExch(err, 3);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    if (valid) {
      const unsigned char* Se = tma_smem + (size_t)s * GroupBytes + (size_t)le * F * BB;
      float acc = 0.0f;
#pragma unroll
      for (int f = 0; f < F; ++f)
        if (nbv[f] >= 0) acc = C::dot(C::lds(Se + f * BB, m), xs[le][f], acc);
      x_out[e * N + m] = xo + wscale * (co - fmaf(w, xo, acc));
    }
    __syncthreads();   // stage s and xs free again
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(k + S);
    }
  }
  if (abort_flag && tid == 0) {
    for (int64_t j = k; j < k + S; ++j) {
      if (blockIdx.x + j * stride >= ngroups) break;
      (void)mbar_wait_bounded(&bar[j % S], (uint32_t)((j / S) & 1));
    }
  }
}

template <int EPB, int S, int MINB>
int launch_scaled_shape(dg_ctx* c, const __nv_bfloat16* sblk, const float* x, const float* cv, float* x_out,
                        cudaStream_t st, const float* ws) {
  const int64_t ngroups = (c->B + EPB - 1) / EPB;
  const unsigned g = (unsigned)std::min<int64_t>(ngroups, (int64_t)c->nsm * MINB);
  const size_t smem = (size_t)S * EPB * 4 * Chunk20<__nv_bfloat16>::BlockBytes;
  return launch_k(c, smooth_scaled_tma_kernel<EPB, S, MINB>, g, EPB * 20, smem, st, sblk, (const int*)c->d_nbe, x,
                  cv, x_out, (int64_t)c->B, (float)c->mixed_smooth_w, ws, (int*)c->d_err,
                  c->l2_hint ? (int)RF_STREAM_HINT : 0);
}

template <int EPB, int S, int MINB>
int set_scaled_smem(dg_ctx* c) {
  CK(c, cudaFuncSetAttribute(smooth_scaled_tma_kernel<EPB, S, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             S * EPB * 4 * Chunk20<__nv_bfloat16>::BlockBytes));
  return DG_OK;
}

// launch shapes (elements per group, stages, CTAs per SM) of the scaled-face
// smoothing kernel, picked by autotune_mixed
int launch_scaled(dg_ctx* c, const __nv_bfloat16* sblk, const float* x, const float* cv, float* x_out,
                  cudaStream_t st, const float* ws) {
  switch (c->sc_variant) {
    case 1: return launch_scaled_shape<8, 2, 3>(c, sblk, x, cv, x_out, st, ws);
    case 2: return launch_scaled_shape<4, 2, 6>(c, sblk, x, cv, x_out, st, ws);
    case 3: return launch_scaled_shape<6, 3, 3>(c, sblk, x, cv, x_out, st, ws);
    default: return launch_scaled_shape<6, 2, 4>(c, sblk, x, cv, x_out, st, ws);
  }
}

int set_scaled_smem_all(dg_ctx* c) {
  int rc;
  if ((rc = set_scaled_smem<6, 2, 4>(c)) || (rc = set_scaled_smem<8, 2, 3>(c)) || (rc = set_scaled_smem<4, 2, 6>(c)) ||
      (rc = set_scaled_smem<6, 3, 3>(c)))
    return rc;
  return DG_OK;
}

// Gauss-Jordan inversion on the GPU (FP64, no pivoting: the coarse SFC level
// matrix is a Galerkin product of an SPD operator, so every pivot is
// positive; a non-positive pivot sets *err = 4).  G is the augmented n x 2n
// matrix [A | I], row-major; step k eliminates column k from every row.
// fcol[i] = G[i][k] and prow[j] = G[k][j] / G[k][k] are taken first so that
// the update reads no element it writes.
__global__ void gj_prep_kernel(const double* __restrict__ G, int n, int k, double* __restrict__ fcol,
                               double* __restrict__ prow, int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double piv = G[(size_t)k * 2 * n + k];
  if (t == 0 && !(piv > 0.0)) atomicExch(err, 4);
  if (t < n) fcol[t] = G[(size_t)t * 2 * n + k];
  const int j = k + t;
  if (j < 2 * n) prow[j] = G[(size_t)k * 2 * n + j] / piv;
}

__global__ void gj_update_kernel(double* __restrict__ G, int n, int k, const double* __restrict__ fcol,
                                 const double* __restrict__ prow) {
  const int j = k + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= 2 * n) return;
  double* row = G + (size_t)i * 2 * n;
  row[j] = (i == k) ? prow[j] : row[j] - fcol[i] * prow[j];
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inverse of the dense coarse level in FP32 (the
// inverse is applied in FP32; the level matrix is symmetric positive
// definite, so no pivoting).  G = [A | I] is n x 2n row-major.  Block step
// over the rows and columns P = [k0, k0 + b):
//   C = G[:, P] (copy; D = C[P, :]), Dinv = D^-1 (one CTA),
//   G[P, :] = Dinv G[P, :],  G[i, :] -= C[i, :] G[P, :] for i not in P.
// Columns left of k0 are already unit columns and the right half is still
// zero beyond n + k0 + b in the rows of P, so a step touches the columns
// [k0, n + k0 + b) only: n^3 FMAs in all, in n / b steps of four launches
// instead of 2 n launches of the one-pivot form.
constexpr int kGjB = 32;

__global__ void gjb_copy_kernel(const float* __restrict__ G, int n, int k0, int b, float* __restrict__ C) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * b) return;
  const int i = t / b, q = t % b;
  C[t] = G[(size_t)i * 2 * n + k0 + q];
}

// Dinv = D^-1 for D = C[k0 .. k0+b, :] (b <= kGjB), one CTA of 256 threads
__global__ void __launch_bounds__(256) gjb_dinv_kernel(const float* __restrict__ C, int k0, int b,
                                                       float* __restrict__ Dinv, int* __restrict__ err) {
  __shared__ float S[kGjB][2 * kGjB + 1];
  __shared__ float f[kGjB];
  for (int t = threadIdx.x; t < b * 2 * b; t += blockDim.x) {
    const int r = t / (2 * b), j = t % (2 * b);
    S[r][j] = j < b ? C[(size_t)(k0 + r) * b + j] : (j - b == r ? 1.0f : 0.0f);
  }
  __syncthreads();
  for (int p = 0; p < b; ++p) {
    const float piv = S[p][p];
    if (!(piv > 0.0f)) {   // uniform
      if (threadIdx.x == 0) atomicExch(err, 4);
      return;
    }
    if (threadIdx.x < b) f[threadIdx.x] = S[threadIdx.x][p];
    __syncthreads();
    const float rp = 1.0f / piv;
    for (int j = threadIdx.x; j < 2 * b; j += blockDim.x) S[p][j] *= rp;
    __syncthreads();
    for (int t = threadIdx.x; t < b * 2 * b; t += blockDim.x) {
      const int r = t / (2 * b), j = t % (2 * b);
      if (r != p) S[r][j] = fmaf(-f[r], S[p][j], S[r][j]);
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) Dinv[t] = S[t / b][b + t % b];
}

// G[P, j] = sum_q Dinv[r][q] G[k0 + q][j] for the columns j in [k0, n + k0 + b);
// one thread per column (reads its b entries, then writes them)
__global__ void __launch_bounds__(128) gjb_rows_kernel(float* __restrict__ G, int n, int k0, int b,
                                                       const float* __restrict__ Dinv) {
  __shared__ float Ds[kGjB * kGjB];
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) Ds[t] = Dinv[t];
  __syncthreads();
  const int j = k0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= min(2 * n, n + k0 + b)) return;
  float g[kGjB];
#pragma unroll
  for (int q = 0; q < kGjB; ++q) g[q] = q < b ? G[(size_t)(k0 + q) * 2 * n + j] : 0.0f;
  for (int r = 0; r < b; ++r) {
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < kGjB; ++q) s = fmaf(Ds[r * b + (q < b ? q : 0)], g[q], s);
    G[(size_t)(k0 + r) * 2 * n + j] = s;
  }
}

// G[i, j] -= sum_q C[i][q] G[k0 + q][j] for rows i not in P and columns j in
// [k0 + b, n + k0 + b); G[i, P] = 0.  64 x 64 tiles, 256 threads of 4 x 4.
__global__ void __launch_bounds__(256) gjb_update_kernel(float* __restrict__ G, int n, int k0, int b,
                                                         const float* __restrict__ C) {
  __shared__ float Cs[64][kGjB + 1];
  __shared__ __align__(16) float Rs[kGjB][64];
  const int i0 = blockIdx.y * 64, j0 = k0 + b + blockIdx.x * 64;
  const int jend = min(2 * n, n + k0 + b);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int t = threadIdx.x; t < 64 * kGjB; t += 256) {
    const int r = t / kGjB, q = t % kGjB;
    Cs[r][q] = (i0 + r < n && q < b) ? C[(size_t)(i0 + r) * b + q] : 0.0f;
  }
  for (int t = threadIdx.x; t < kGjB * 64; t += 256) {
    const int q = t / 64, c = t % 64;
    Rs[q][c] = (q < b && j0 + c < jend) ? G[(size_t)(k0 + q) * 2 * n + j0 + c] : 0.0f;
  }
  __syncthreads();
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0f;
#pragma unroll 8
  for (int q = 0; q < kGjB; ++q) {
    const float4 rv = *reinterpret_cast<const float4*>(&Rs[q][4 * tx]);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float cv = Cs[4 * ty + u][q];
      acc[u][0] = fmaf(cv, rv.x, acc[u][0]);
      acc[u][1] = fmaf(cv, rv.y, acc[u][1]);
      acc[u][2] = fmaf(cv, rv.z, acc[u][2]);
      acc[u][3] = fmaf(cv, rv.w, acc[u][3]);
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = i0 + 4 * ty + u;
    if (i >= n || (i >= k0 && i < k0 + b)) continue;
    float* row = G + (size_t)i * 2 * n;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + 4 * tx + v;
      if (j < jend) row[j] -= acc[u][v];
    }
    if (blockIdx.x == 0)   // the block's own columns become zero
      for (int q = tx; q < b; q += 16) row[k0 + q] = 0.0f;
  }
}

// inv (n x n FP32) = right half of the FP32 G
__global__ void gjb_extract_kernel(const float* __restrict__ G, int n, float* __restrict__ inv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int64_t i = t / n, j = t % n;
  inv[t] = G[i * 2 * n + n + j];
}

// inv (n x n FP32) = right half of G
__global__ void gj_extract_kernel(const double* __restrict__ G, int n, float* __restrict__ inv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int64_t i = t / n, j = t % n;
  inv[t] = (float)G[i * 2 * n + n + j];
}


__global__ void zero_f32_kernel(float* __restrict__ a, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] = 0.0f;
}

// x += alpha * d (FP64 += FP32)
__global__ void axpy_f32_to_f64_kernel(double* __restrict__ x, const float* __restrict__ d, int64_t n,
                                       double alpha) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) x[k] += alpha * (double)d[k];
}

Mixed& mixed_of(dg_ctx* c) {
  if (!c->mixed_state) c->mixed_state = new Mixed();
  return *static_cast<Mixed*>(c->mixed_state);
}

void destroy_mixed(dg_ctx* c) {
  if (!c->mixed_state) return;
  Mixed* M = static_cast<Mixed*>(c->mixed_state);
  for (auto& g : M->graphs)
    if (g) cudaGraphExecDestroy(g);
  destroy_batch(M->batch);   // host-side state only: device buffers are context allocations
  delete M;
  c->mixed_state = nullptr;
}

template <int D>
int launch_residual32(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags,
                      cudaStream_t st, const float* ws = nullptr) {
  using E = Elem<D>;
  Mixed& M = mixed_of(c);
  if (D == 3 && c->f32_tma) {   // chunked FP32 copy, bulk-copy kernel
    const float* A = M.sf ? M.sblk32 : M.blk;
    if (flags & RF_SMOOTH)
      return launch_tma<float, 4, 2, 2, true>(c, A, M.W, x, b, r, x_out, flags, M.r1, st, M.sf, ws);
    return launch_tma<float, 4, 2, 3, false>(c, A, M.W, x, b, r, x_out, flags, M.r1, st, M.sf);
  }
  unsigned g = nblk(c->B, E::EPB);
  if (g)
    residual_kernel<E::N, E::F, E::EPB, float, float, float><<<g, E::EPB * E::N, 0, st>>>(
        M.blk, M.W, c->d_nbe, x, b, r, x_out, c->B, flags, c->T.P, M.r1, ws);
  bump();
  CKL(c);
  return DG_OK;
}

int residual32(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags, cudaStream_t st,
               const float* ws = nullptr) {
  return c->D == 3 ? launch_residual32<3>(c, x, b, r, x_out, flags, st, ws)
                   : launch_residual32<2>(c, x, b, r, x_out, flags, st, ws);
}

// residual / smoothing with the BF16 block copies (FP32 vectors and sums)
template <int D>
int launch_residual16(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags,
                      cudaStream_t st, const float* ws = nullptr) {
  using E = Elem<D>;
  Mixed& M = mixed_of(c);
  unsigned g = nblk(c->B, E::EPB);
  if (g)
    residual_kernel<E::N, E::F, E::EPB, __nv_bfloat16, float, float><<<g, E::EPB * E::N, 0, st>>>(
        M.blk16, M.W16, c->d_nbe, x, b, r, x_out, c->B, flags, c->T.P, M.r1, ws);
  bump();
  CKL(c);
  return DG_OK;
}

// residual in the preconditioner: BF16 blocks when enabled, FP32 otherwise
// *ws (device memory, so that captured graphs follow a rebuilt schedule;
// nullptr = 1) scales the smoother's correction of this step,
// x_out = x + ws W_e res: with W_e = w A_ee^-1 the step is damped by ws * w
int residual_pc(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags, cudaStream_t st,
                const float* ws = nullptr) {
  if (c->precond_bf16) {
    if (c->D == 3 && c->bf16_tma) {
      Mixed& M = mixed_of(c);
      return launch_bf16_tma(c, M, x, b, r, x_out, flags, st, ws);
    }
    if (c->D == 3) {
      Mixed& M = mixed_of(c);
      unsigned g = nblk(c->B, 8);
      if (g)
        residual_bf16c20_kernel<8><<<g, 8 * 20, 0, st>>>(M.blk16, M.W16, c->d_nbe, x, b, r, x_out, c->B, flags,
                                                          c->d_P32, M.r1, ws);
      bump();
      CKL(c);
      return DG_OK;
    }
    return launch_residual16<2>(c, x, b, r, x_out, flags, st, ws);
  }
  return residual32(c, x, b, r, x_out, flags, st, ws);
}

// P1 -> P3 prolongation of the coarse correction (mixed path, 3D):
// x[e][n] += sum_c P[n][c] (w_ec ecg[pos(p1cg[e][c])]).  8 elements per CTA;
// the 4 corner values of an element are formed once (threads m < 4) instead
// of by each of its 20 node threads.  Same products and summation order as
// prolong_cg_kernel.  The corner indices are fixed data, read before the
// programmatic-launch wait.
__global__ void __launch_bounds__(160) prolong_cg32_kernel(float* __restrict__ x, const float* __restrict__ ecg,
                                                           const int* __restrict__ pos, const int* __restrict__ p1cg,
                                                           const float* __restrict__ wdg,
                                                           const float* __restrict__ P, int64_t B) {
  __shared__ float vc[8][4];
  const int le = threadIdx.x / 20, n = threadIdx.x % 20;
  const int64_t e = (int64_t)blockIdx.x * 8 + le;
  const bool valid = e < B;
  int vp = 0;
  float w = 0.0f;
  if (valid && n < 4) {
    vp = pos[p1cg[e * 4 + n]];
    w = (float)wdg[e * 4 + n];
  }
  float p[4];
#pragma unroll
  for (int c2 = 0; c2 < 4; ++c2) p[c2] = (float)P[n * 4 + c2];
  pdl_wait_then_trigger();
  if (valid && n < 4) vc[le][n] = w * ecg[vp];
  __syncthreads();
  if (!valid) return;
  float v = 0.0f;
#pragma unroll
  for (int c2 = 0; c2 < 4; ++c2) v += p[c2] * vc[le][c2];
  x[e * 20 + n] += v;
}

// vertex gather of the element P1 restrictions (mixed path): one warp per
// vertex, lanes over the vertex's DG copies, shuffle-reduced
// With e_out, also the first Jacobi sweep of SFC level 0 from a zero guess
// (lev_jacobi_kernel with e_in = NULL: rr = r, e_out = fma(rr / diag, w, 0),
// rr_out = rr if set), so that sweep needs no launch of its own.
__global__ void gather_cg32_kernel(const float* __restrict__ r1, const int* __restrict__ gptr,
                                   const int* __restrict__ gent, const float* __restrict__ wdg,
                                   const int* __restrict__ pos, float* __restrict__ out, int ncg,
                                   const float* __restrict__ diag0, float* __restrict__ e_out,
                                   float* __restrict__ rr_out, float w) {
  const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  int k0 = 0, k1 = 0;
  if (i < ncg) {
    k0 = gptr[i];
    k1 = gptr[i + 1];
  }
  pdl_wait_then_trigger();
  if (i >= ncg) return;
  float acc = 0.0f;
  for (int k = k0 + lane; k < k1; k += 32) {
    const int ent = gent[k];
    acc = __fmaf_rn((float)wdg[ent], r1[ent], acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane != 0) return;
  const int p = pos[i];
  out[p] = acc;
  if (e_out) {
    const float rr = acc - 0.0f;
    e_out[p] = __fmaf_rn(rr / diag0[p], w, 0.0f);
    if (rr_out) rr_out[p] = rr;
  }
}

template <int D>
int launch_transfer32(dg_ctx* c, const float* r, float* cg_out, float* x_add, const float* e_sfc,
                      cudaStream_t st) {
  using E = Elem<D>;
  if (r) {
    restrict_cg_kernel<E::N, E::NC, float><<<nblk(c->ncg, 128), 128, 0, st>>>(
        r, c->T.P, c->d_gptr, c->d_gent, c->d_wdg, c->d_pos, cg_out, (int)c->ncg);
    bump();
  } else {
    int rc;
    if (D == 3)
      rc = launch_k(c, prolong_cg32_kernel, nblk(c->B, 8), 160, 0, st, x_add, e_sfc, (const int*)c->d_pos,
                    (const int*)c->d_p1cg, (const float*)c->d_wdg32, (const float*)c->d_P32, (int64_t)c->B);
    else
      rc = launch_k(c, prolong_cg_kernel<E::N, E::NC, float>, nblk(c->B * E::N, 256), 256, 0, st, x_add, e_sfc,
                    (const int*)c->d_pos, (const int*)c->d_p1cg, (const double*)c->d_wdg, (const double*)c->T.P,
                    (const int*)nullptr, 0, (int64_t)c->B, 1);
    if (rc) return rc;
  }
  CKL(c);
  return DG_OK;
}

int transfer32(dg_ctx* c, const float* r, float* cg_out, float* x_add, const float* e_sfc, cudaStream_t st) {
  return c->D == 3 ? launch_transfer32<3>(c, r, cg_out, x_add, e_sfc, st)
                   : launch_transfer32<2>(c, r, cg_out, x_add, e_sfc, st);
}

#include "dg_vcycle_cluster.cuh"

// Picks the cluster size of the V-cycle legs for this mixed build and
// lays out their shared memory: the request (dg_ctx::vc32_cluster), limited
// to kVcMaxLev levels above the dense level, to what fits in kVcSmemMax
// bytes per CTA and to what the device can schedule.  Per CTA: the slice
// vectors of every level above the dense one (4 x rows per CTA words each),
// then the matrix image of its rows (row offsets, diagonal, entries as
// (owner << 20 | slice index of the column, value bits)), built here from
// the device's FP32 level matrices and uploaded once per build.
int setup_vcycle_cluster(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  M.vc_cs = 0;
  M.vc_smem = 0;
  const int lc = M.dense_l;
  if (c->vc32_cluster == 0 || lc < 1 || lc > kVcMaxLev) return DG_OK;
  // the FP32 level matrices as the chain's kernels read them
  std::vector<std::vector<int>> rp(lc), cl(lc);
  std::vector<std::vector<float>> vl(lc), dg(lc);
  for (int l = 0; l < lc; ++l) {
    const Lev32& L = M.lev[l];
    rp[l].resize(L.n + 1);
    CK(c, cudaMemcpyAsync(rp[l].data(), L.rowptr, sizeof(int) * (L.n + 1), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    const int nnz = rp[l][L.n];
    cl[l].resize(nnz);
    vl[l].resize(nnz);
    dg[l].resize(L.n);
    CK(c, cudaMemcpyAsync(cl[l].data(), L.col, sizeof(int) * nnz, cudaMemcpyDeviceToHost, st));
    CK(c, cudaMemcpyAsync(vl[l].data(), L.val, sizeof(float) * nnz, cudaMemcpyDeviceToHost, st));
    CK(c, cudaMemcpyAsync(dg[l].data(), L.diag, sizeof(float) * L.n, cudaMemcpyDeviceToHost, st));
  }
  CK(c, cudaStreamSynchronize(st));
  auto pad = [](int64_t x, int64_t m) { return (x + m - 1) / m * m; };
  for (int cs : {16, 8}) {
    if (c->vc32_cluster > 0 && cs != c->vc32_cluster) continue;
    std::vector<int> ch(lc + 1), off(lc, 0), rpo(lc), dgo(lc), eno(lc);
    int64_t vwords = 0, iwords = 0;
    bool fits = true;
    for (int l = 0; l <= lc; ++l) ch[l] = (int)((M.lev[l].n + cs - 1) / cs);
    for (int l = 0; l < lc; ++l) {
      if (ch[l] >= (1 << kVcLocalBits)) fits = false;
      off[l] = (int)vwords;
      vwords += 4 * (int64_t)ch[l];
      int64_t maxnnz = 0;
      for (int r = 0; r < cs; ++r) {
        const int s0 = std::min(M.lev[l].n, r * ch[l]), s1 = std::min(M.lev[l].n, s0 + ch[l]);
        maxnnz = std::max<int64_t>(maxnnz, rp[l][s1] - rp[l][s0]);
      }
      rpo[l] = (int)iwords;
      iwords += pad(ch[l] + 1, 2);
      dgo[l] = (int)iwords;
      iwords += pad(ch[l], 2);
      eno[l] = (int)iwords;
      iwords += 2 * maxnnz;
    }
    vwords = pad(vwords, 4);
    iwords = pad(iwords, 4);
    if (!fits || (vwords + iwords) * 4 > kVcSmemMax) continue;
    const size_t smem = (size_t)(vwords + iwords) * 4;
    bool ok = true;
    for (auto k : {vcycle_down_kernel, vcycle_up_kernel}) {
      // the same limit for every context of the process (the attribute is
      // per kernel); each launch asks for its own size
      ok = ok && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kVcSmemMax) == cudaSuccess;
      if (cs > 8) ok = ok && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    }
    int ncl = 0;
    if (ok) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(kVcThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      ok = cudaOccupancyMaxActiveClusters(&ncl, vcycle_down_kernel, &cfg) == cudaSuccess && ncl >= 1;
    }
    cudaGetLastError();
    if (!ok) continue;
    // the images of all CTAs, one after another
    std::vector<int32_t> img((size_t)cs * iwords, 0);
    for (int r = 0; r < cs; ++r) {
      int32_t* I = img.data() + (size_t)r * iwords;
      for (int l = 0; l < lc; ++l) {
        const int n = M.lev[l].n;
        const int s0 = std::min(n, r * ch[l]), s1 = std::min(n, s0 + ch[l]);
        const int kb = rp[l][s0];
        for (int i = s0; i <= s1; ++i) I[rpo[l] + (i - s0)] = rp[l][i] - kb;
        for (int i = s0; i < s1; ++i) std::memcpy(&I[dgo[l] + (i - s0)], &dg[l][i], 4);
        for (int k = kb; k < rp[l][s1]; ++k) {
          const int col = cl[l][k];
          const int o = col / ch[l], loc = col - o * ch[l];
          I[eno[l] + 2 * (k - kb)] = (o << kVcLocalBits) | loc;
          std::memcpy(&I[eno[l] + 2 * (k - kb) + 1], &vl[l][k], 4);
        }
      }
    }
    if (M.vc_img_cap < img.size()) {
      int rc;
      if ((rc = dalloc(c, &M.vc_img, img.size()))) return rc;
      M.vc_img_cap = img.size();
    }
    CK(c, cudaMemcpyAsync(M.vc_img, img.data(), sizeof(int32_t) * img.size(), cudaMemcpyHostToDevice, st));
    CK(c, cudaStreamSynchronize(st));
    M.vc_cs = cs;
    M.vc_smem = smem;
    M.vc_ch = ch;
    M.vc_off = off;
    M.vc_rpo = rpo;
    M.vc_dgo = dgo;
    M.vc_eno = eno;
    M.vc_vwords = (int)vwords;
    M.vc_iwords = (int)iwords;
    break;
  }
  if (c->verbose)
    std::fprintf(stderr, "[mixed] V-cycle legs: %s (cluster %d, %zu B shared per CTA)\n",
                 M.vc_cs ? "cluster launches" : "launch chain", M.vc_cs, M.vc_smem);
  return DG_OK;
}

int launch_vc(dg_ctx* c, void (*kern)(const VcParams), const VcParams& p, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(M.vc_cs);
  cfg.blockDim = dim3(kVcThreads);
  cfg.dynamicSmemBytes = M.vc_smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = M.vc_cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c->use_pdl ? 2 : 1;
  CK(c, cudaLaunchKernelEx(&cfg, kern, p));
  bump();
  return DG_OK;
}

// The FP32 V-cycle with the dense coarse level as three launches: the
// cluster down leg (the vertex gather of M.r1 included), the dense mat-vec,
// the cluster up leg.  Same operations and result buffer (M.lev[0].e) as
// gather_cg32_kernel + vcycle32.
int vcycle32_cluster(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  const int lc = M.dense_l;
  VcParams p = {};
  const int V = M.vc_vwords;
  for (int l = 0; l <= lc; ++l) {
    const Lev32& L = M.lev[l];
    const int ch = M.vc_ch[l];
    const bool sl = l < lc;
    p.lev[l] = VcLevel{L.up, L.e, L.r, L.n, ch, sl ? M.vc_off[l] : 0, sl ? V + M.vc_rpo[l] : 0,
                       sl ? V + M.vc_dgo[l] : 0, sl ? V + M.vc_eno[l] : 0, 1.0f / (float)ch};
  }
  p.lc = lc;
  p.npre = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.pre_smooth_its;
  p.npost = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.post_smooth_its;
  p.w = (float)c->cfg.jac_wei;
  p.img = reinterpret_cast<const int4*>(M.vc_img);
  p.img_words = M.vc_iwords;
  p.img_off = V;
  p.r1 = M.r1;
  p.gptr = c->d_gptr;
  p.gent = c->d_gent;
  p.wdg = c->d_wdg32;
  p.pos = c->d_pos;
  p.ncg = (int)c->ncg;
  int rc;
  if ((rc = launch_vc(c, vcycle_down_kernel, p, st))) return rc;
  {
    Lev32& L = M.lev[lc];
    if ((rc = launch_k(c, dense_matvec_kernel, nblk(L.n, 8), 256, sizeof(float) * L.n, st, (const float*)M.dense_inv,
                       (const float*)L.r, L.e, L.n, (const float*)nullptr, 0)))
      return rc;
  }
  if ((rc = launch_vc(c, vcycle_up_kernel, p, st))) return rc;
  CKL(c);
  return DG_OK;
}

// The FP32 V-cycle with the dense coarse level (dense_l >= 1) as a launch
// chain in which no transfer between levels has a launch of its own: the
// vertex gather also runs level 0's first sweep (zero guess), each coarser
// level's first sweep restricts its input on the fly (lev_jacobi_x_kernel
// mode 1), the dense mat-vec restricts its right-hand side on the fly, and
// each level's first post-sweep adds the prolonged coarse correction on the
// fly (mode 2).  Same operations, buffers and e / e2 swaps as
// gather_cg32_kernel + vcycle32; c2: 11 launches instead of 17.
int vcycle32_fused(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  const int lc = M.dense_l;
  const float w = (float)c->cfg.jac_wei;
  const int TB = 128;
  const int npre = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.pre_smooth_its;
  const int npost = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.post_smooth_its;
  int rc;
  {
    Lev32& L = M.lev[0];
    if ((rc = launch_k(c, gather_cg32_kernel, nblk(c->ncg, 8), 256, 0, st, (const float*)M.r1,
                       (const int*)c->d_gptr, (const int*)c->d_gent, (const float*)c->d_wdg32, (const int*)c->d_pos,
                       L.r, (int)c->ncg, (const float*)L.diag, L.e2, npre == 0 ? L.rr : (float*)nullptr, w)))
      return rc;
    std::swap(L.e, L.e2);
  }
  for (int l = 0; l < lc; ++l) {
    Lev32& L = M.lev[l];
    const unsigned gj = nblk((int64_t)L.n * LPR, TB);
    for (int it = l == 0 ? 1 : 0; it <= npre; ++it) {
      float* keep = it == npre ? L.rr : nullptr;
      if (it == 0) {
        const Lev32& P = M.lev[l - 1];
        rc = launch_k(c, lev_jacobi_x_kernel<1>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                      (const float*)L.val, (const float*)L.diag, (const float*)P.e, (const float*)P.rr,
                      (const int*)nullptr, P.n, L.r, L.e2, keep, L.n, w);
      } else {
        rc = launch_k(c, lev_jacobi_kernel<float>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                      (const float*)L.val, (const float*)L.diag, (const float*)L.e, (const float*)L.r, L.e2, keep,
                      L.n, (double)c->cfg.jac_wei);
      }
      if (rc) return rc;
      std::swap(L.e, L.e2);
    }
  }
  {
    Lev32& L = M.lev[lc];
    const Lev32& P = M.lev[lc - 1];
    if ((rc = launch_k(c, dense_matvec_kernel, nblk(L.n, 8), 256, sizeof(float) * L.n, st, (const float*)M.dense_inv,
                       (const float*)nullptr, L.e, L.n, (const float*)P.rr, P.n)))
      return rc;
  }
  for (int l = lc - 1; l >= 0; --l) {
    Lev32& L = M.lev[l];
    const float* enext = M.lev[l + 1].e;
    const unsigned gj = nblk((int64_t)L.n * LPR, TB);
    if (npost == 0) {
      if ((rc = launch_k(c, lev_prolong_kernel<float>, nblk(L.n, TB), TB, 0, st, L.e, enext, (const int*)L.up, L.n)))
        return rc;
      continue;
    }
    for (int it = 0; it < npost; ++it) {
      if (it == 0)
        rc = launch_k(c, lev_jacobi_x_kernel<2>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                      (const float*)L.val, (const float*)L.diag, (const float*)L.e, enext, (const int*)L.up, 0, L.r,
                      L.e2, (float*)nullptr, L.n, w);
      else
        rc = launch_k(c, lev_jacobi_kernel<float>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                      (const float*)L.val, (const float*)L.diag, (const float*)L.e, (const float*)L.r, L.e2,
                      (float*)nullptr, L.n, (double)c->cfg.jac_wei);
      if (rc) return rc;
      std::swap(L.e, L.e2);
    }
  }
  CKL(c);
  return DG_OK;
}

// FP32 SFC V-cycle (same schedule as vcycle() down to the coarse level,
// where the mixed preconditioner solves exactly with the dense inverse);
// result in M.lev[0].e
int vcycle32(dg_ctx* c, const float* r_sfc, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  const int nl = (int)M.lev.size();
  const int top = nl - 1;
  const double w = c->cfg.jac_wei;
  const int TB = 128;
  if (M.dense_l >= 0) {
    // kernels only (no copy / memset nodes), so that the whole chain can be
    // linked by programmatic dependent launches: the residual arrives in
    // lev[0].r (gathered there directly when r_sfc is lev[0].r) and level 0
    // starts from a zero guess (e_in = NULL in its first sweep)
    const int lc = M.dense_l;
    const int npre = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.pre_smooth_its;
    const int npost = c->mixed_lev_sweeps >= 0 ? c->mixed_lev_sweeps : c->cfg.post_smooth_its;
    int rc;
    if (r_sfc != M.lev[0].r)
      CK(c, cudaMemcpyAsync(M.lev[0].r, r_sfc, sizeof(float) * M.lev[0].n, cudaMemcpyDeviceToDevice, st));
    for (int l = 0; l < lc; ++l) {
      Lev32& L = M.lev[l];
      const unsigned gj = nblk((int64_t)L.n * LPR, TB);
      for (int it = 0; it < npre; ++it) {
        const float* ein = (l == 0 && it == 0) ? nullptr : L.e;
        if ((rc = launch_k(c, lev_jacobi_kernel<float>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                           (const float*)L.val, (const float*)L.diag, ein, (const float*)L.r, L.e2,
                           (float*)nullptr, L.n, w)))
          return rc;
        std::swap(L.e, L.e2);
      }
      const float* ein = (l == 0 && npre == 0) ? nullptr : L.e;
      if ((rc = launch_k(c, lev_jacobi_kernel<float>, gj, TB, 0, st, (const int*)L.rowptr, (const int*)L.col,
                         (const float*)L.val, (const float*)L.diag, ein, (const float*)L.r, L.e2, L.rr, L.n, w)))
        return rc;
      std::swap(L.e, L.e2);
      Lev32& Nx = M.lev[l + 1];
      if ((rc = launch_k(c, lev_restrict_kernel<float>, nblk(Nx.n, TB), TB, 0, st, (const float*)L.rr,
                         (const float*)L.e, Nx.r, Nx.e, L.n, Nx.n)))
        return rc;
    }
    {
      Lev32& L = M.lev[lc];
      if ((rc = launch_k(c, dense_matvec_kernel, nblk(L.n, 8), 256, sizeof(float) * L.n, st, (const float*)M.dense_inv,
                         (const float*)L.r, L.e, L.n, (const float*)nullptr, 0)))
        return rc;
    }
    for (int l = lc - 1; l >= 0; --l) {
      Lev32& L = M.lev[l];
      if ((rc = launch_k(c, lev_prolong_kernel<float>, nblk(L.n, TB), TB, 0, st, L.e, (const float*)M.lev[l + 1].e,
                         (const int*)L.up, L.n)))
        return rc;
      for (int it = 0; it < npost; ++it) {
        if ((rc = launch_k(c, lev_jacobi_kernel<float>, nblk((int64_t)L.n * LPR, TB), TB, 0, st,
                           (const int*)L.rowptr, (const int*)L.col, (const float*)L.val, (const float*)L.diag,
                           (const float*)L.e, (const float*)L.r, L.e2, (float*)nullptr, L.n, w)))
          return rc;
        std::swap(L.e, L.e2);
      }
    }
    CKL(c);
    return DG_OK;
  }
  const int l0 = tail_start(c, c->tail_max32);
  CK(c, cudaMemcpyAsync(M.lev[0].r, r_sfc, sizeof(float) * M.lev[0].n, cudaMemcpyDeviceToDevice, st));
  CK(c, cudaMemsetAsync(M.lev[0].e, 0, sizeof(float) * M.lev[0].n, st));
  for (int l = 0; l < std::min(l0, top); ++l) {
    Lev32& L = M.lev[l];
    for (int it = 0; it < c->cfg.pre_smooth_its; ++it) {
      lev_jacobi_kernel<float><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e,
                                                                           L.r, L.e2, nullptr, L.n, w);
      bump();
      std::swap(L.e, L.e2);
    }
    lev_jacobi_kernel<float><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e,
                                                                         L.r, L.e2, L.rr, L.n, w);
    bump();
    std::swap(L.e, L.e2);
    Lev32& Nx = M.lev[l + 1];
    lev_restrict_kernel<float><<<nblk(Nx.n, TB), TB, 0, st>>>(L.rr, L.e, Nx.r, Nx.e, L.n, Nx.n);
    bump();
  }
  if (M.lev[top].n != 1) return fail(c, DG_ERR_STATE, "coarsest SFC level must hold one node");
  if (l0 < top) {
    TailParams<float> tp;
    tp.l0 = l0;
    tp.top = top;
    tp.pre = c->cfg.pre_smooth_its;
    tp.post = c->cfg.post_smooth_its;
    tp.w = w;
    for (int l = 0; l < nl; ++l) {
      const Lev32& L = M.lev[l];
      tp.lev[l] = TLevel<float>{L.rowptr, L.col, L.val, L.diag, L.up, L.e, L.e2, L.r, L.rr, L.n};
    }
    vcycle_tail_kernel<float><<<1, 1024, 0, st>>>(tp);
    bump();
  } else {
    Lev32& L = M.lev[top];
    lev_coarse_kernel<float><<<1, 32, 0, st>>>(L.val, L.r, L.e);
    bump();
  }
  for (int l = std::min(l0, top) - 1; l >= 0; --l) {
    Lev32& L = M.lev[l];
    lev_prolong_kernel<float><<<nblk(L.n, TB), TB, 0, st>>>(L.e, M.lev[l + 1].e, L.up, L.n);
    bump();
    for (int it = 0; it < c->cfg.post_smooth_its; ++it) {
      lev_jacobi_kernel<float><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e,
                                                                           L.r, L.e2, nullptr, L.n, w);
      bump();
      std::swap(L.e, L.e2);
    }
  }
  CKL(c);
  return DG_OK;
}

// Damping of a degree-deg Chebyshev smoother for A_ee^-1 A on [beta / ratio,
// beta], beta = cheb_margin * lmax: the polynomial's roots, smallest factor
// first, 1 / (mid + hw cos(pi (2k + 1) / (2 deg))), stored as factors of
// the smoother matrices' own damping w
void cheb_factors(const dg_ctx* c, double lmax, int deg, double ratio, float* out) {
  const double beta = c->cheb_margin * lmax, alpha = beta / ratio;
  const double mid = 0.5 * (beta + alpha), hw = 0.5 * (beta - alpha);
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < deg; ++k) {
    const double om = 1.0 / (mid + hw * std::cos(pi * (2 * k + 1) / (2.0 * deg)));
    out[k] = (float)(om / c->mixed_smooth_w);
  }
}

// DG-level smoothing steps of the mixed preconditioner (pre and post each):
// DG_MIXED_SWEEPS when set, else kMixedChebSteps with the damped block
// inverse (a Chebyshev polynomial of that degree), else the configured V(s,s)
int mixed_steps(const dg_ctx* c) {
  if (c->mixed_sweeps >= 0) return c->mixed_sweeps;
  return c->mixed_smoother == 1 ? kMixedChebSteps : c->cfg.pre_smooth_its;
}

// one smoothing step of the preconditioner with x != 0: x_out = x + s W (b -
// A x), s = *ws.  On the scaled face blocks, rhs is c = W b (formed by the
// zero-start step); otherwise it is b.
int smooth_step(dg_ctx* c, const float* x, const float* rhs, float* x_out, cudaStream_t st, const float* ws) {
  Mixed& M = mixed_of(c);
  if (M.sc) return launch_scaled(c, M.scblk16, x, rhs, x_out, st, ws);
  return residual_pc(c, x, rhs, nullptr, x_out, RF_SMOOTH, st, ws);
}

// z = M32^{-1} r (FP32, same schedule as precond()); scratch t3, t4, t5
int precond32(dg_ctx* c, const float* r, float* z, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  const int nsm = mixed_steps(c);
  float* cur = M.t3;
  float* other = M.t4;
  // per-step damping: pre-smoothing steps k = 0, 1, ... use ws[k], the
  // post-smoothing steps the same factors in reverse order
  auto ws = [&](int k) -> const float* {
    return ((nsm >= 2 && nsm <= kMaxSmoothSteps) || c->omegas_set) && k < kMaxSmoothSteps ? M.d_ws + k : nullptr;
  };
  // scaled-face steps: the zero-start step also keeps c = W r, which every
  // later step reads in place of r
  const float* rs = M.sc ? M.chat : r;
  if (nsm > 0) {
    if (M.sc) {
      if ((rc = launch_bf16_tma(c, M, nullptr, r, nullptr, cur, RF_ZEROX | RF_SMOOTH, st, ws(0), M.chat))) return rc;
    } else if ((rc = residual_pc(c, nullptr, r, nullptr, cur, RF_ZEROX | RF_SMOOTH, st, ws(0)))) {
      return rc;
    }
    for (int it = 1; it < nsm; ++it) {
      if ((rc = smooth_step(c, cur, rs, other, st, ws(it)))) return rc;
      std::swap(cur, other);
    }
  } else {
    CK(c, cudaMemsetAsync(cur, 0, sizeof(float) * c->nonods, st));
  }
  if ((rc = residual_pc(c, cur, r, nullptr, nullptr, RF_RESTRICT, st))) return rc;   // -> M.r1
  if (M.vc_cs > 0) {
    if ((rc = vcycle32_cluster(c, st))) return rc;   // gather included
  } else if (M.dense_l > 0 && c->vc32_fused) {
    if ((rc = vcycle32_fused(c, st))) return rc;     // gather included
  } else {
    float* cg_dst = M.dense_l > 0 ? M.lev[0].r : M.cg1;
    if ((rc = launch_k(c, gather_cg32_kernel, nblk(c->ncg, 8), 256, 0, st, (const float*)M.r1,
                       (const int*)c->d_gptr, (const int*)c->d_gent, (const float*)c->d_wdg32, (const int*)c->d_pos,
                       cg_dst, (int)c->ncg, (const float*)nullptr, (float*)nullptr, (float*)nullptr, 0.0f)))
      return rc;
    if ((rc = vcycle32(c, cg_dst, st))) return rc;
  }
  if ((rc = transfer32(c, nullptr, nullptr, cur, M.lev[0].e, st))) return rc;
  for (int it = 0; it < nsm; ++it) {
    float* out = (it == nsm - 1) ? z : other;
    if ((rc = smooth_step(c, cur, rs, out, st, ws(nsm - 1 - it)))) return rc;
    other = cur;
    cur = out;
  }
  if (nsm == 0) CK(c, cudaMemcpyAsync(z, cur, sizeof(float) * c->nonods, cudaMemcpyDeviceToDevice, st));
  return DG_OK;
}

// flag[q] |= 1 if x_q (row q of the RHS-major (nrhs, n) array) has an entry
// other than +-0 (NaN counts as nonzero); grid (blocks, nrhs).  A zero start
// needs no FP64 apply: b - A 0 = b exactly.
__global__ void bnonzero_kernel(const double* __restrict__ x, int64_t n, int* __restrict__ flag) {
  const int q = blockIdx.y;
  bool nz = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    nz |= !(x[(int64_t)q * n + i] == 0.0);
  nz = __syncthreads_or(nz);
  if (nz && threadIdx.x == 0) atomicOr(flag + q, 1);
}

template <typename ST>
__global__ void convert_f64_f32_kernel(const ST* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)a[k];
}

template <typename ST>
__global__ void convert_f64_bf16_kernel(const ST* __restrict__ a, __nv_bfloat16* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = __float2bfloat16_rn((float)a[k]);
}

// Deterministic start vector of the power iteration: a hash of the index
// mapped to [-1, 1).
__global__ void probe_init_kernel(float* __restrict__ v, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t h = (uint32_t)k * 2654435761u + 0x9e3779b9u;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  v[k] = (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
}

__global__ void sub_f32_kernel(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ y,
                               int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] = a[k] - b[k];
}

// Damping of the two DG-level smoothing steps of the mixed preconditioner:
// the roots of the degree-2 Chebyshev polynomial on [beta / 8, beta] for the
// block-Jacobi operator A_ee^-1 A, beta = 1.05 x its largest eigenvalue,
// estimated by power iteration with the preconditioner's own smoothing
// kernel (W A v = v - smooth(v, b = 0), W = w A_ee^-1; at most 40 steps,
// stopped when the estimate moves by less than 1e-3).  Step 0 takes the
// smaller factor.  c2 and c3: lambda_max ~ 1.96, factors (0.56, 1.92);
// c2 80 inner iterations (exact stop) against 100 with the uniform
// w = 0.8, c3 90 against 120.  Without a usable estimate the steps keep the
// uniform damping.
int norm32(dg_ctx* c, const float* z, double* out, cudaStream_t st);

int set_smoother_schedule(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  const int64_t n = c->nonods;
  float* v = M.t1;
  float* zb = M.t2;
  float* u = M.t3;
  int rc;
  for (float& f : c->mixed_wscale) f = 1.0f;
  probe_init_kernel<<<nblk(n, 256), 256, 0, st>>>(v, n);
  bump();
  CK(c, cudaMemsetAsync(zb, 0, sizeof(float) * n, st));
  if ((rc = norm32(c, v, c->d_scal, st))) return rc;
  scale_kernel<float><<<nblk(n, 256), 256, 0, st>>>(v, c->d_scal, v, n);
  bump();
  // the estimates of a run of steps stay on the device (d_scal[1 + it]) and
  // are read once per run, not once per step; the stop is the first step
  // it >= 8 whose estimate moved by at most 1e-3 (later steps of the run
  // change nothing that is used)
  constexpr int kMaxIts = 40;
  double lam = 0.0, prev = -1.0;
  std::vector<double> lams(kMaxIts, 0.0);
  bool stop = false;
  for (int it0 = 0; it0 < kMaxIts && !stop;) {
    const int run = it0 == 0 ? 9 : std::min(8, kMaxIts - it0);
    for (int it = it0; it < it0 + run; ++it) {
      if ((rc = smooth_step(c, v, zb, u, st, nullptr))) return rc;   // u = v - W A v (c = W zb = 0)
      sub_f32_kernel<<<nblk(n, 256), 256, 0, st>>>(v, u, v, n);                 // v <- W A v
      bump();
      if ((rc = norm32(c, v, c->d_scal + 1 + it, st))) return rc;
      scale_kernel<float><<<nblk(n, 256), 256, 0, st>>>(v, c->d_scal + 1 + it, v, n);
      bump();
    }
    CK(c, cudaMemcpyAsync(lams.data() + it0, c->d_scal + 1 + it0, sizeof(double) * run, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    for (int it = it0; it < it0 + run; ++it) {
      lam = lams[it];
      if (!(lam > 0.0) || !std::isfinite(lam)) return DG_OK;
      if (it >= 8 && std::fabs(lam - prev) <= 1e-3 * lam) {
        stop = true;
        break;
      }
      prev = lam;
    }
    it0 += run;
  }
  CKL(c);
  const double lmax = lam / c->mixed_smooth_w;   // of A_ee^-1 A
  const int deg = std::min(kMaxSmoothSteps, std::max(2, mixed_steps(c)));
  cheb_factors(c, lmax, deg, c->cheb_ratio, c->mixed_wscale);
  c->smoother_lmax = lmax;
  if (c->verbose)
    std::fprintf(stderr, "[build_mixed] smoother: lambda_max(A_ee^-1 A) ~ %.4f, degree %d, damping %.4f .. %.4f\n",
                 lmax, deg, c->mixed_wscale[0] * c->mixed_smooth_w, c->mixed_wscale[deg - 1] * c->mixed_smooth_w);
  return DG_OK;
}

// Five blocks per element copies of the operator (FP32; BF16 when the
// preconditioner reads BF16), read by the plain kernels and the batched solve.
int build_blk5(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  const size_t nb = (size_t)c->B * (c->F + 1) * c->N * c->N;
  if (!M.blk && (rc = dalloc(c, &M.blk, nb))) return rc;
  if (c->D == 3 && c->f32_tma)
    convert_f64_f32_chunk20_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk,
                                                                          (int64_t)c->B * (c->F + 1));
  else
    convert_f64_f32_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk, (int64_t)nb);
  bump();
  if (c->precond_bf16) {
    if (!M.blk16 && (rc = dalloc(c, &M.blk16, nb))) return rc;
    if (c->D == 3)   // chunked layout read by residual_bf16c20_kernel
      convert_f64_bf16_chunk20_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk16,
                                                                             (int64_t)c->B * (c->F + 1));
    else
      convert_f64_bf16_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk16, (int64_t)nb);
    bump();
  }
  CKL(c);
  M.has5 = true;
  return DG_OK;
}

int build_mixed(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  const auto t0 = std::chrono::steady_clock::now();
  if ((rc = set_tma_smem<__nv_bfloat16, 6, 2, 3, true>(c)) || (rc = set_tma_smem<__nv_bfloat16, 8, 2, 2, true>(c)) ||
      (rc = set_tma_smem<__nv_bfloat16, 4, 2, 4, true>(c)) || (rc = set_tma_smem<float, 4, 2, 3, false>(c)) ||
      (rc = set_tma_smem<float, 4, 2, 2, true>(c)) || (rc = set_scaled_smem_all(c)))
    return rc;
  const size_t nw = (size_t)c->B * c->N * c->N;
  if (!M.t1) {
    for (float** t : {&M.t1, &M.t2, &M.t3, &M.t4, &M.t5, &M.t6})
      if ((rc = dalloc(c, t, (size_t)c->nonods))) return rc;
    if ((rc = dalloc(c, &M.cg1, (size_t)c->ncg))) return rc;
    if ((rc = dalloc(c, &M.r1, (size_t)c->B * c->NC))) return rc;
  }
  if (!M.W && (rc = dalloc(c, &M.W, nw))) return rc;
  // operator copies: shared-face arrays for the 3D bulk-copy kernels, else
  // five blocks per element
  M.sf = c->D == 3 && c->shared_faces && c->d_fref5 && c->f32_tma && c->bf16_tma && c->precond_bf16;
  M.has5 = false;
  if (M.sf) {
    const int64_t ns = (int64_t)c->B + c->nface_sh;
    if (!M.sblk32 && (rc = dalloc(c, &M.sblk32, (size_t)ns * 400))) return rc;
    if (!M.sblk16 && (rc = dalloc(c, &M.sblk16, (size_t)ns * 400))) return rc;
    convert_gather_chunk20_kernel<float><<<nblk(ns * 400, 256), 256, 0, st>>>(c->d_blk, c->d_sfsrc, M.sblk32, ns);
    bump();
    convert_gather_chunk20_kernel<__nv_bfloat16><<<nblk(ns * 400, 256), 256, 0, st>>>(c->d_blk, c->d_sfsrc,
                                                                                        M.sblk16, ns);
    bump();
    CKL(c);
  } else if ((rc = build_blk5(c, st))) {
    return rc;
  }
  auto vt = [&](const char* what) {   // verbose phase timings
    if (!c->verbose) return;
    cudaStreamSynchronize(st);
    std::fprintf(stderr, "[build_mixed] %s done at %.2f ms\n", what,
                 std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  };
  vt("operator copies");
  // smoother matrices of the mixed preconditioner
  if (c->mixed_smoother != 1 && (rc = ensure_w64(c, st))) return rc;   // the reference's smoother copied
  const double* Wsrc = c->d_W;
  const float* Wsrc32 = nullptr;
  double* Winv = nullptr;
  if (c->mixed_smoother == 1) {
    // scratch kept with the context: a cudaFree here would wait for every
    // stream of the device (other contexts' solves on a serving GPU)
    if (!M.winv && (rc = dalloc(c, &M.winv, nw))) return rc;
    Winv = M.winv;
    // inverted in FP32: the copies it feeds are FP32 / BF16, and the FP64
    // inverse ran at the FP64 pipe's rate (21 ms at 280k tets against 1 ms)
    float* W32 = reinterpret_cast<float*>(M.winv);
    CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
    if (c->D == 3)
      block_inverse32_kernel<20, 4><<<nblk(c->B, 8), 256, 0, st>>>(c->d_blk, W32, c->B, (float)c->mixed_smooth_w,
                                                                   c->d_err);
    else
      block_inverse32_kernel<10, 3><<<nblk(c->B, 8), 256, 0, st>>>(c->d_blk, W32, c->B, (float)c->mixed_smooth_w,
                                                                   c->d_err);
    bump();
    Wsrc32 = W32;
    vt("block inverses");
  }
  auto copies = [&](auto src) -> int {
    if (c->D == 3 && c->f32_tma)
      convert_f64_f32_chunk20_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(src, M.W, (int64_t)c->B);
    else
      convert_f64_f32_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(src, M.W, (int64_t)nw);
    bump();
    if (c->precond_bf16) {
      int r2;
      if (!M.W16 && (r2 = dalloc(c, &M.W16, nw))) return r2;
      if (c->D == 3)
        convert_f64_bf16_chunk20_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(src, M.W16, (int64_t)c->B);
      else
        convert_f64_bf16_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(src, M.W16, (int64_t)nw);
      bump();
    }
    return DG_OK;
  };
  if ((rc = Wsrc32 ? copies(Wsrc32) : copies(Wsrc))) return rc;
  if (Winv) {
    int herr = 0;
    CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (herr) return fail(c, DG_ERR_NUMERIC, "element block with a non-positive pivot (not positive definite)");
  }
  vt("smoother copies");
  // scaled face blocks of the BF16 bulk-copy smoothing steps (the smoother
  // must be the damped block inverse: its self block is then w I)
  M.sc = c->scaled_faces && c->D == 3 && c->precond_bf16 && c->bf16_tma && !M.sf && Wsrc32 != nullptr;
  if (M.sc) {
    if (!M.scblk16 && (rc = dalloc(c, &M.scblk16, (size_t)c->B * 4 * 400))) return rc;
    if (!M.chat && (rc = dalloc(c, &M.chat, (size_t)c->nonods))) return rc;
    scaled_faces_kernel<<<(unsigned)c->B, 400, 0, st>>>(Wsrc32, c->d_blk, M.scblk16, (int64_t)c->B);
    bump();
    CKL(c);
    vt("scaled face blocks");
  }
  if (M.lev.size() != c->lev.size()) {
    M.lev.assign(c->lev.size(), Lev32());
    for (size_t l = 0; l < c->lev.size(); ++l) {
      Lev32& L = M.lev[l];
      const DevLevel& D = c->lev[l];
      L.n = D.n;
      L.rowptr = D.rowptr;
      L.col = D.col;
      L.up = D.up;
      int nnz = 0;
      CK(c, cudaMemcpyAsync(&nnz, D.rowptr + D.n, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      if ((rc = dalloc(c, &L.val, (size_t)nnz))) return rc;
      for (float** t : {&L.diag, &L.e, &L.e2, &L.r, &L.rr})
        if ((rc = dalloc(c, t, (size_t)L.n))) return rc;
    }
  }
  for (size_t l = 0; l < c->lev.size(); ++l) {
    Lev32& L = M.lev[l];
    const DevLevel& D = c->lev[l];
    int nnz = 0;
    CK(c, cudaMemcpyAsync(&nnz, D.rowptr + D.n, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    convert_f64_f32_kernel<<<nblk(nnz, 256), 256, 0, st>>>(D.val, L.val, nnz);
    bump();
    convert_f64_f32_kernel<<<nblk(D.n, 256), 256, 0, st>>>(D.diag, L.diag, D.n);
    bump();
  }
  if (c->verbose) CK(c, cudaStreamSynchronize(st));
  const auto t1 = std::chrono::steady_clock::now();
  // exact coarse solve on the first level with at most dense_max rows
  M.dense_l = -1;
  if (c->dense_max32 > 0) {
    const SfcHierarchy& h = c->sfc_h;
    int lc = -1;
    for (int l = 0; l < h.nlevel; ++l)
      if (h.sizes[l] <= c->dense_max32) { lc = l; break; }
    if (lc >= 0) {
      const int n = (int)h.sizes[lc];
      // augmented [A | I] assembled on the host from the level's device CSR
      // (its values are formed on the device after the first build),
      // inverted on the GPU
      const DevLevel& DL = c->lev[lc];
      std::vector<int> drp(n + 1);
      CK(c, cudaMemcpyAsync(drp.data(), DL.rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      std::vector<int> dcl(drp[n]);
      std::vector<double> dvl(drp[n]);
      CK(c, cudaMemcpyAsync(dcl.data(), DL.col, sizeof(int) * drp[n], cudaMemcpyDeviceToHost, st));
      CK(c, cudaMemcpyAsync(dvl.data(), DL.val, sizeof(double) * drp[n], cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      std::vector<double> Gh((size_t)n * 2 * n, 0.0);
      for (int i = 0; i < n; ++i) {
        for (int k = drp[i]; k < drp[i + 1]; ++k) Gh[(size_t)i * 2 * n + dcl[k]] += dvl[k];
        Gh[(size_t)i * 2 * n + n + i] = 1.0;
      }
      // augmented matrix and pivot row / column (FP64 form) or the FP32
      // augmented matrix, panel copy and block inverse, kept with the context
      const size_t gneed = std::max(Gh.size() + 3 * (size_t)n,
                                    (Gh.size() + (size_t)kGjB * n + (size_t)kGjB * kGjB + 1) / 2);
      if (M.gj_cap < gneed) {
        if ((rc = dalloc(c, &M.gj, gneed))) return rc;
        M.gj_cap = gneed;
      }
      if (!M.dense_inv || c->dense_n != n) {
        if ((rc = dalloc(c, &M.dense_inv, (size_t)n * n))) return rc;
        c->dense_n = n;
      }
      CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
      if (c->dense_fp64) {
        // one pivot per launch pair, FP64 (DG_DENSE_FP64=1)
        double* G = M.gj;
        double* fcol = G + Gh.size();
        double* prow = fcol + n;
        CK(c, cudaMemcpyAsync(G, Gh.data(), sizeof(double) * Gh.size(), cudaMemcpyHostToDevice, st));
        for (int k = 0; k < n; ++k) {
          gj_prep_kernel<<<nblk(2 * n - k > n ? 2 * n - k : n, 256), 256, 0, st>>>(G, n, k, fcol, prow, c->d_err);
          gj_update_kernel<<<dim3(nblk(2 * n - k, 256), n), 256, 0, st>>>(G, n, k, fcol, prow);
        }
        bump(2 * (long long)n);
        gj_extract_kernel<<<nblk((int64_t)n * n, 256), 256, 0, st>>>(G, n, M.dense_inv);
        bump();
      } else {
        // blocked FP32 form in the same scratch: G (n x 2n), C (n x kGjB), Dinv
        float* G = reinterpret_cast<float*>(M.gj);
        float* C = G + Gh.size();
        float* Dinv = C + (size_t)n * kGjB;
        std::vector<float> Gf(Gh.begin(), Gh.end());
        CK(c, cudaMemcpyAsync(G, Gf.data(), sizeof(float) * Gf.size(), cudaMemcpyHostToDevice, st));
        for (int k0 = 0; k0 < n; k0 += kGjB) {
          const int b = std::min(kGjB, n - k0);
          gjb_copy_kernel<<<nblk((int64_t)n * b, 256), 256, 0, st>>>(G, n, k0, b, C);
          gjb_dinv_kernel<<<1, 256, 0, st>>>(C, k0, b, Dinv, c->d_err);
          gjb_rows_kernel<<<nblk(n + b, 128), 128, 0, st>>>(G, n, k0, b, Dinv);
          gjb_update_kernel<<<dim3((unsigned)((n + 63) / 64), (unsigned)((n + 63) / 64)), 256, 0, st>>>(G, n, k0, b,
                                                                                                     C);
          bump(4);
        }
        gjb_extract_kernel<<<nblk((int64_t)n * n, 256), 256, 0, st>>>(G, n, M.dense_inv);
        bump();
      }
      int herr = 0;
      CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      CKL(c);
      if (herr == 0) M.dense_l = lc;
    }
  }
  CKL(c);
  if ((rc = setup_vcycle_cluster(c, st))) return rc;
  M.built = true;
  if (!M.d_ws && (rc = dalloc(c, &M.d_ws, kMaxSmoothSteps))) return rc;
  if (!c->omegas_set && c->mixed_smoother == 1) {
    if ((rc = set_smoother_schedule(c, st))) return rc;
  } else if (!c->omegas_set) {
    for (float& f : c->mixed_wscale) f = 1.0f;
  }
  CK(c, cudaMemcpyAsync(M.d_ws, c->mixed_wscale, sizeof(float) * kMaxSmoothSteps, cudaMemcpyHostToDevice, st));
  CK(c, cudaStreamSynchronize(st));
  if (c->verbose)
    std::fprintf(stderr, "[build_mixed] ms: copies + smoother blocks + levels %.2f, dense coarse inverse (%d rows) %.2f\n",
                 std::chrono::duration<double, std::milli>(t1 - t0).count(), c->dense_n,
                 std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count());
  return DG_OK;
}

int ensure_krylov32(dg_ctx* c, int m) {
  Mixed& M = mixed_of(c);
  if (M.vcap >= m + 1) return DG_OK;
  int rc;
  if ((rc = dalloc(c, &M.V, (size_t)(m + 1) * c->nonods))) return rc;
  if ((rc = dalloc(c, &M.Z, (size_t)m * c->nonods))) return rc;
  if ((rc = dalloc(c, &M.H, (size_t)(m + 1) * m))) return rc;
  if (!M.part) {
    M.nblk4 = (int)((c->nonods / 4 + RED_TB - 1) / RED_TB);
    if ((rc = dalloc(c, &M.part, (size_t)std::max(M.nblk4, 1) * KMAXV))) return rc;
    if ((rc = dalloc(c, &M.gs_cnt, 64))) return rc;
    CK(c, cudaMemset(M.gs_cnt, 0, sizeof(unsigned) * 64));
  }
  if (!M.gv) {   // sized for the largest restart length (256)
    if ((rc = dalloc(c, &M.gv, (size_t)3 * 256 + 2))) return rc;
    if ((rc = dalloc(c, &M.kdone, 1))) return rc;
  }
  M.vcap = m + 1;
  return DG_OK;
}

int norm32(dg_ctx* c, const float* z, double* out, cudaStream_t st) { return norm_t<float>(c, z, out, st); }

// ---------------------------------------------------------------------------
// FP32 Gram-Schmidt kernels on float4 (vector length a multiple of 4, every
// vector 16-byte aligned).  Each thread keeps one float4 of z and the same
// float4 of up to 8 basis vectors in flight per step; per-thread sums are
// FP32, the block and grid sums FP64, in a fixed order (deterministic).

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// partial[bx * KMAXV + i0 + q] = sum over this block's slice of V[i0+q] . z,
// i0 = 8 * blockIdx.y.  The grid covers the vectors once (one float4 per
// thread when gridDim.x * TB >= n4), so all nine loads of a thread are in
// flight together; per-thread and in-warp sums are FP32 (a warp sums at most
// a few hundred products), the warps of a block and the blocks are combined
// in FP64.  GB300's FP64 pipe is narrow: FP64 shuffle trees per thread cost
// more than the memory traffic here.
template <int TB>
__global__ void __launch_bounds__(TB) mdot8_f32_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                       const float* __restrict__ z, int64_t n4,
                                                       double* __restrict__ partial) {
  pdl_wait_then_trigger();
  __shared__ float red[TB / 32][8];
  const int i0 = blockIdx.y * 8;
  const int cnt = min(8, nv - i0);
  float acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0f;
  const float4* z4 = reinterpret_cast<const float4*>(z);
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n4; k += (int64_t)gridDim.x * TB) {
    const float4 zv = z4[k];
    float4 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      v[q] = q < cnt ? reinterpret_cast<const float4*>(V + (size_t)(i0 + q) * ld)[k] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      acc[q] = fmaf(v[q].x, zv.x, acc[q]);
      acc[q] = fmaf(v[q].y, zv.y, acc[q]);
      acc[q] = fmaf(v[q].z, zv.z, acc[q]);
      acc[q] = fmaf(v[q].w, zv.w, acc[q]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float a = warp_sum_f(acc[q]);
    if (lane == 0) red[wid][q] = a;
  }
  __syncthreads();
  if (threadIdx.x < cnt) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += (double)red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * KMAXV + i0 + threadIdx.x] = s;
  }
}

// z -= sum_i V[i] h[i] (nv <= 256); with want_norm also
// partial[bx * KMAXV] = this block's slice of |z_new|^2 (FP32 within a warp,
// FP64 across warps)
template <int TB>
__global__ void __launch_bounds__(TB) axpy8_f32_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                       const double* __restrict__ h, float* __restrict__ z,
                                                       int64_t n4, double* __restrict__ partial, int want_norm) {
  pdl_wait_then_trigger();
  __shared__ float hs[256];
  __shared__ float red[TB / 32];
  for (int i = threadIdx.x; i < nv; i += TB) hs[i] = (float)h[i];
  __syncthreads();
  float acc = 0.0f;
  float4* z4 = reinterpret_cast<float4*>(z);
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n4; k += (int64_t)gridDim.x * TB) {
    float4 zv = z4[k];
    for (int i0 = 0; i0 < nv; i0 += 8) {
      float4 v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        v[q] = (i0 + q < nv) ? reinterpret_cast<const float4*>(V + (size_t)(i0 + q) * ld)[k]
                             : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float hq = (i0 + q < nv) ? hs[i0 + q] : 0.0f;
        zv.x -= v[q].x * hq;
        zv.y -= v[q].y * hq;
        zv.z -= v[q].z * hq;
        zv.w -= v[q].w * hq;
      }
    }
    z4[k] = zv;
    if (want_norm) {
      acc = fmaf(zv.x, zv.x, acc);
      acc = fmaf(zv.y, zv.y, acc);
      acc = fmaf(zv.z, zv.z, acc);
      acc = fmaf(zv.w, zv.w, acc);
    }
  }
  if (!want_norm) return;
  const float a = warp_sum_f(acc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += (double)red[w];
    partial[(int64_t)blockIdx.x * KMAXV] = s;
  }
}

// Hessenberg column j: Hc[i] = h1[i] (+ h2[i] when h2) for i < nv;
// Hc[nv] = |z| = sqrt(sum of the norm partials); *inv = 1 / |z| in FP32.
// One block, fixed summation order.
__global__ void cgs_finish_kernel(const double* __restrict__ partial, int nblk, const double* __restrict__ h1,
                                  const double* __restrict__ h2, int nv, double* __restrict__ Hc,
                                  float* __restrict__ inv) {
  pdl_wait_then_trigger();
  __shared__ double red[32];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) Hc[i] = h2 ? h1[i] + h2[i] : h1[i];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[(int64_t)b * KMAXV];
  s = warp_sum(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[w];
    t = sqrt(t);
    Hc[nv] = t;
    *inv = (float)(1.0 / t);
  }
}

// v = z * (*inv), float4
__global__ void scale4_f32_kernel(const float* __restrict__ z, const float* __restrict__ inv, float* __restrict__ v,
                                  int64_t n4) {
  pdl_wait_then_trigger();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n4) return;
  const float s = *inv;
  float4 a = reinterpret_cast<const float4*>(z)[k];
  a.x *= s;
  a.y *= s;
  a.z *= s;
  a.w *= s;
  reinterpret_cast<float4*>(v)[k] = a;
}

// The same dots with the block reduction fused: each CTA writes its partial
// sums, and the last CTA of a grid row (arrival counter) adds the rows'
// partials in block order -- warp q sums vector q's partials, lanes strided,
// then a fixed shuffle tree -- and writes h[i0 + q]; it resets the counter
// for the next launch.  One launch per step instead of two.
template <int TB>
__global__ void __launch_bounds__(TB) mdot8r_f32_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                        const float* __restrict__ z, int64_t n4,
                                                        double* __restrict__ partial, double* __restrict__ h,
                                                        unsigned* __restrict__ cnt_arr) {
  pdl_wait_then_trigger();
  __shared__ float red[TB / 32][8];
  __shared__ bool last;
  const int i0 = blockIdx.y * 8;
  const int cnt = min(8, nv - i0);
  float acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0f;
  const float4* z4 = reinterpret_cast<const float4*>(z);
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n4; k += (int64_t)gridDim.x * TB) {
    const float4 zv = z4[k];
    float4 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      v[q] = q < cnt ? reinterpret_cast<const float4*>(V + (size_t)(i0 + q) * ld)[k] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      acc[q] = fmaf(v[q].x, zv.x, acc[q]);
      acc[q] = fmaf(v[q].y, zv.y, acc[q]);
      acc[q] = fmaf(v[q].z, zv.z, acc[q]);
      acc[q] = fmaf(v[q].w, zv.w, acc[q]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float a = warp_sum_f(acc[q]);
    if (lane == 0) red[wid][q] = a;
  }
  __syncthreads();
  if (threadIdx.x < cnt) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += (double)red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * KMAXV + i0 + threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&cnt_arr[blockIdx.y], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (wid < cnt) {
    double s = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&partial[(int64_t)b * KMAXV + i0 + wid]);
    s = warp_sum(s);
    if (lane == 0) h[i0 + wid] = s;
  }
  if (threadIdx.x == 0) cnt_arr[blockIdx.y] = 0u;
}

// z -= sum_i V[i] h[i] with |z_new|^2, and in the last CTA (arrival
// counter) the Hessenberg column: Hc[i] = h1[i] (+ h2[i]), Hc[nv] = |z|,
// *inv = 1 / |z| -- the update and cgs_finish_kernel in one launch.
template <int TB>
__global__ void __launch_bounds__(TB) axpy8f_f32_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                        const double* __restrict__ h, float* __restrict__ z,
                                                        int64_t n4, double* __restrict__ partial,
                                                        const double* __restrict__ h1, const double* __restrict__ h2,
                                                        double* __restrict__ Hc, float* __restrict__ inv,
                                                        unsigned* __restrict__ cnt) {
  pdl_wait_then_trigger();
  __shared__ float hs[256];
  __shared__ float red[TB / 32];
  __shared__ bool last;
  for (int i = threadIdx.x; i < nv; i += TB) hs[i] = (float)h[i];
  __syncthreads();
  float acc = 0.0f;
  float4* z4 = reinterpret_cast<float4*>(z);
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n4; k += (int64_t)gridDim.x * TB) {
    float4 zv = z4[k];
    for (int i0 = 0; i0 < nv; i0 += 8) {
      float4 v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        v[q] = (i0 + q < nv) ? reinterpret_cast<const float4*>(V + (size_t)(i0 + q) * ld)[k]
                             : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float hq = (i0 + q < nv) ? hs[i0 + q] : 0.0f;
        zv.x -= v[q].x * hq;
        zv.y -= v[q].y * hq;
        zv.z -= v[q].z * hq;
        zv.w -= v[q].w * hq;
      }
    }
    z4[k] = zv;
    acc = fmaf(zv.x, zv.x, acc);
    acc = fmaf(zv.y, zv.y, acc);
    acc = fmaf(zv.z, zv.z, acc);
    acc = fmaf(zv.w, zv.w, acc);
  }
  const float a = warp_sum_f(acc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += (double)red[w];
    partial[(int64_t)blockIdx.x * KMAXV] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = threadIdx.x; i < nv; i += TB) Hc[i] = h2 ? h1[i] + h2[i] : h1[i];
  if (wid == 0) {
    double s = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&partial[(int64_t)b * KMAXV]);
    s = warp_sum(s);
    if (lane == 0) {
      const double t = sqrt(s);
      Hc[nv] = t;
      *inv = (float)(1.0 / t);
      *cnt = 0u;
    }
  }
}

// h[0..nv) = V^T z with the float4 kernels (nv <= KMAXV per call)
int mdot4_f32(dg_ctx* c, const float* V, int nv, const float* z, double* h, cudaStream_t st) {
  const int64_t n4 = c->nonods / 4;
  for (int off = 0; off < nv; off += KMAXV) {
    const int cnt = std::min(KMAXV, nv - off);
    int rc;
    Mixed& M = mixed_of(c);
    if (c->gs_fused) {
      if ((rc = launch_k2(c, mdot8r_f32_kernel<RED_TB>, dim3(M.nblk4, (cnt + 7) / 8), RED_TB, 0, st,
                          (const float*)(V + (size_t)off * c->nonods), (int64_t)c->nonods, cnt, z, n4, M.part,
                          h + off, M.gs_cnt)))
        return rc;
      continue;
    }
    if ((rc = launch_k2(c, mdot8_f32_kernel<RED_TB>, dim3(M.nblk4, (cnt + 7) / 8), RED_TB, 0, st,
                        (const float*)(V + (size_t)off * c->nonods), (int64_t)c->nonods, cnt, z, n4, M.part)))
      return rc;
    if ((rc = launch_k(c, reduce_partial_kernel, cnt, 256, 0, st, (const double*)M.part, M.nblk4, cnt, h + off, 0,
                       0)))
      return rc;
  }
  return DG_OK;
}

// Gram-Schmidt of w against V[0..j] (FP32 vectors; CGS2 or, with
// mixed_cgs_passes = 1, one classical pass); writes the FP64 Hessenberg
// column j and V[j+1] = w / |w|.
int cgs2_32(dg_ctx* c, int j, float* w, int m, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  if (c->nonods % 4 != 0) return cgs2_t<float>(c, M.V, M.H, j, w, m, st);
  const int nv = j + 1;
  const int64_t n4 = c->nonods / 4;
  double* Hc = M.H + (size_t)j * (m + 1);
  const bool two = c->mixed_cgs_passes != 1;
  float* inv = reinterpret_cast<float*>(c->d_scal + 1);
  int rc;
  if ((rc = mdot4_f32(c, M.V, nv, w, c->d_h1, st))) return rc;
  if (two) {
    if ((rc = launch_k(c, axpy8_f32_kernel<RED_TB>, M.nblk4, RED_TB, 0, st, (const float*)M.V, (int64_t)c->nonods,
                       nv, (const double*)c->d_h1, w, n4, M.part, 0)))
      return rc;
    if ((rc = mdot4_f32(c, M.V, nv, w, c->d_h2, st))) return rc;
  }
  if (c->gs_fused) {
    // the last update with |w|^2 and the Hessenberg column in one launch
    if ((rc = launch_k(c, axpy8f_f32_kernel<RED_TB>, M.nblk4, RED_TB, 0, st, (const float*)M.V, (int64_t)c->nonods,
                       nv, (const double*)(two ? c->d_h2 : c->d_h1), w, n4, M.part, (const double*)c->d_h1,
                       two ? (const double*)c->d_h2 : (const double*)nullptr, Hc, inv, M.gs_cnt + 32)))
      return rc;
  } else {
    if ((rc = launch_k(c, axpy8_f32_kernel<RED_TB>, M.nblk4, RED_TB, 0, st, (const float*)M.V, (int64_t)c->nonods,
                       nv, (const double*)(two ? c->d_h2 : c->d_h1), w, n4, M.part, 1)))
      return rc;
    if ((rc = launch_k(c, cgs_finish_kernel, 1, 256, 0, st, (const double*)M.part, M.nblk4, (const double*)c->d_h1,
                       two ? (const double*)c->d_h2 : (const double*)nullptr, nv, Hc, inv)))
      return rc;
  }
  if ((rc = launch_k(c, scale4_f32_kernel, nblk(n4, 256), 256, 0, st, (const float*)w, (const float*)inv,
                     M.V + (size_t)nv * c->nonods, n4)))
    return rc;
  CKL(c);
  return DG_OK;
}

// Incremental Givens QR of the inner Hessenberg matrix, one FP64 thread:
// rotations 0..j-1 (kept in gv) carried down column j of H, then rotation j
// and the least-squares residual |g[j+1]| of the j+1 step Krylov space.  At
// or below the threshold (or NaN) the step count goes to *kdone and, inside a
// chunk graph, the conditional node of step j+1 is switched off, so the
// remaining steps of the chunk are skipped on the device.  H is not changed:
// the host solves the least-squares problem from H itself.
__global__ void givens_check_kernel(const double* __restrict__ H, int m, int j, double* __restrict__ gv,
                                    int* __restrict__ kdone, cudaGraphConditionalHandle next, int has_next) {
  pdl_wait_then_trigger();
  if (threadIdx.x != 0) return;
  double* cs = gv;
  double* sn = gv + m;
  double* g = gv + 2 * m;
  const double thresh = gv[3 * m + 1];
  const double* h = H + (size_t)j * (m + 1);
  double hi = h[0];
  for (int i = 0; i < j; ++i) hi = -sn[i] * hi + cs[i] * h[i + 1];
  const double hj1 = h[j + 1];
  const double r = sqrt(hi * hi + hj1 * hj1);
  double cr = 1.0, sr = 0.0;
  if (r > 0.0) {
    cr = hi / r;
    sr = hj1 / r;
  }
  cs[j] = cr;
  sn[j] = sr;
  const double gj = g[j];
  g[j] = cr * gj;
  g[j + 1] = -sr * gj;
  const bool done = !(fabs(g[j + 1]) > thresh);
  if (done && *kdone == 0) *kdone = j + 1;
  if (has_next) cudaGraphSetConditional(next, done ? 0u : 1u);
}

// inner Arnoldi step j: z_j = M v_j (kept), w = A z_j, Gram-Schmidt, then
// the device-side convergence test
int arnoldi32_step(dg_ctx* c, int j, int m, cudaStream_t st, cudaGraphConditionalHandle next, int has_next) {
  Mixed& M = mixed_of(c);
  int rc;
  float* zj = M.Z + (size_t)j * c->nonods;
  if ((rc = precond32(c, M.V + (size_t)j * c->nonods, zj, st))) return rc;
  if ((rc = residual32(c, zj, nullptr, M.t1, nullptr, RF_NEG, st))) return rc;   // t1 = A z_j
  if ((rc = cgs2_32(c, j, M.t1, m, st))) return rc;
  if (!c->cond_graph) return DG_OK;
  return launch_k(c, givens_check_kernel, 1, 32, 0, st, (const double*)M.H, m, j, M.gv, M.kdone, next, has_next);
}

int arnoldi32_steps(dg_ctx* c, int j0, int cnt, int m, cudaStream_t st) {
  int rc;
  for (int j = j0; j < j0 + cnt; ++j)
    if ((rc = arnoldi32_step(c, j, m, st, 0, 0))) return rc;
  return DG_OK;
}

// Graph of steps j0 .. j0+cnt-1, each step the body of an IF conditional
// node; the node of step j0 runs at every launch (default 1), the others run
// when the preceding step's convergence test leaves them on.  kern[i] =
// kernels of step i.  Returns cudaSuccess or the first CUDA error (the caller
// then falls back to plain captured chunks).
cudaError_t build_cond_chunk(dg_ctx* c, int j0, int cnt, int m, cudaGraphExec_t* exec, std::vector<int>& kern,
                             int* rc_out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphConditionalHandle> h(cnt);
  for (int i = 0; i < cnt && e == cudaSuccess; ++i)
    e = cudaGraphConditionalHandleCreate(&h[i], g, i == 0 ? 1u : 0u, cudaGraphCondAssignDefault);
  cudaGraphNode_t prev = nullptr;
  kern.assign(cnt, 0);
  for (int i = 0; i < cnt && e == cudaSuccess; ++i) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h[i];
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, g, prev ? &prev : nullptr, nullptr, prev ? 1 : 0, &p);
    if (e != cudaSuccess) break;
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(c->cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) break;
    const long long k0 = g_launches.load();
    const int rc = arnoldi32_step(c, j0 + i, m, c->cap_stream, i + 1 < cnt ? h[i + 1] : 0, i + 1 < cnt ? 1 : 0);
    kern[i] = (int)(g_launches.load() - k0);
    g_launches.fetch_sub(kern[i]);   // captured, not launched
    cudaGraph_t got = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(c->cap_stream, &got);
    if (rc) {
      *rc_out = rc;
      cudaGraphDestroy(g);
      return cudaSuccess;
    }
    e = ee;
    prev = node;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// Runs steps j0 .. j0+cnt-1 (one chunk).  *mode: 0 = direct launches (all
// steps ran, kernels already counted), 1 = plain chunk graph (all steps ran),
// 2 = conditional chunk graph (steps up to the convergence test's step ran).
int run_arnoldi32(dg_ctx* c, int j0, int cnt, int m, int chunk, cudaStream_t st, int* mode) {
  Mixed& M = mixed_of(c);
  *mode = 0;
  if (!c->use_graph) return arnoldi32_steps(c, j0, cnt, m, st);
  if (M.g_m != m || M.g_chunk != chunk || M.g_vptr != M.V) {
    for (auto& g : M.graphs)
      if (g) cudaGraphExecDestroy(g);
    M.graphs.assign((m + chunk - 1) / chunk, nullptr);
    M.g_kern.assign(M.graphs.size(), std::vector<int>());
    M.g_cond.assign(M.graphs.size(), false);
    M.g_m = m;
    M.g_chunk = chunk;
    M.g_vptr = M.V;
  }
  const int gi = j0 / chunk;
  if (cnt != std::min(chunk, m - j0) || j0 % chunk) return arnoldi32_steps(c, j0, cnt, m, st);
  if (!M.graphs[gi]) {
    if (!c->cap_stream) CK(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    M.g_cond.resize(M.graphs.size());
    M.g_cond[gi] = false;
    if (M.cond && c->cond_graph) {
      int rc = DG_OK;
      const cudaError_t e = build_cond_chunk(c, j0, cnt, m, &M.graphs[gi], M.g_kern[gi], &rc);
      if (rc) return rc;
      if (e != cudaSuccess) {   // no conditional nodes here: plain chunks from now on
        cudaGetLastError();
        if (c->verbose) std::fprintf(stderr, "[dg_solve_mixed] conditional chunk graph: %s\n", cudaGetErrorString(e));
        M.cond = false;
        M.graphs[gi] = nullptr;
      } else {
        M.g_cond[gi] = true;
      }
    }
    if (!M.graphs[gi]) {
      CK(c, cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
      const long long k0 = g_launches.load();
      int rc = arnoldi32_steps(c, j0, cnt, m, c->cap_stream);
      const int nk = (int)(g_launches.load() - k0);
      g_launches.fetch_sub(nk);
      M.g_kern[gi].assign(cnt, nk / std::max(cnt, 1));
      cudaGraph_t g = nullptr;
      cudaError_t ee = cudaStreamEndCapture(c->cap_stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ee != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
      cudaError_t ie = cudaGraphInstantiate(&M.graphs[gi], g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    }
  }
  CK(c, cudaGraphLaunch(M.graphs[gi], st));
  *mode = M.g_cond[gi] ? 2 : 1;
  return DG_OK;
}

// Kernel count of the first `ran` steps of the chunk graph starting at j0
long long chunk_kernels(dg_ctx* c, int j0, int ran) {
  Mixed& M = mixed_of(c);
  const int gi = j0 / std::max(M.g_chunk, 1);
  long long k = 0;
  if (gi < (int)M.g_kern.size())
    for (int i = 0; i < ran && i < (int)M.g_kern[gi].size(); ++i) k += M.g_kern[gi][i];
  return k;
}

// Givens least squares on the leading (k+1) x k block of the column-major
// (m+1) x m Hessenberg; returns the residual estimate |g_k|.
double hessenberg_ls(const std::vector<double>& Hcm, int m, int k, double beta, std::vector<double>& y, bool& ok) {
  std::vector<double> R((size_t)(k + 1) * k);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i <= k; ++i) R[(size_t)i * k + j] = Hcm[(size_t)j * (m + 1) + i];
  std::vector<double> g(k + 1, 0.0);
  g[0] = beta;
  ok = true;
  for (int j = 0; j < k; ++j) {
    double a = R[(size_t)j * k + j], b = R[(size_t)(j + 1) * k + j];
    double r = std::hypot(a, b);
    if (r == 0.0) { ok = false; return NAN; }
    double cs = a / r, sn = b / r;
    for (int q = j; q < k; ++q) {
      double t1 = R[(size_t)j * k + q], t2 = R[(size_t)(j + 1) * k + q];
      R[(size_t)j * k + q] = cs * t1 + sn * t2;
      R[(size_t)(j + 1) * k + q] = -sn * t1 + cs * t2;
    }
    double g1 = g[j], g2 = g[j + 1];
    g[j] = cs * g1 + sn * g2;
    g[j + 1] = -sn * g1 + cs * g2;
  }
  y.assign(k, 0.0);
  for (int i = k - 1; i >= 0; --i) {
    double s = g[i];
    for (int q = i + 1; q < k; ++q) s -= R[(size_t)i * k + q] * y[q];
    if (R[(size_t)i * k + i] == 0.0) { ok = false; return NAN; }
    y[i] = s / R[(size_t)i * k + i];
  }
  return std::fabs(g[k]);
}

// Launch-shape autotuner for the single-RHS bulk-copy kernels: times every
// candidate shape (elements per group, stages, CTAs per SM) of the BF16
// smoothing step on zeroed scratch vectors with CUDA events (one warm launch,
// then 5 timed) and keeps the fastest.  Runs once per operator build before
// any graph capture; cached graphs are dropped when the choice changes.
int autotune_mixed(dg_ctx* c, cudaStream_t st) {
  if (!c->autotune || c->D != 3 || !c->precond_bf16 || !c->bf16_tma) return DG_OK;
  Mixed& M = mixed_of(c);
  const int64_t n = c->nonods;
  CK(c, cudaMemsetAsync(M.t2, 0, sizeof(float) * n, st));
  CK(c, cudaMemsetAsync(M.t3, 0, sizeof(float) * n, st));
  cudaEvent_t e0, e1;
  CK(c, cudaEventCreate(&e0));
  CK(c, cudaEventCreate(&e1));
  const int before = c->tma_variant;
  float best = 1e30f;
  int bestv = 0;
  for (int v = 0; v < kTmaVariants; ++v) {
    c->tma_variant = v;
    int rc = launch_bf16_tma(c, M, M.t3, M.t2, nullptr, M.t4, RF_SMOOTH, st);
    if (!rc) CK(c, cudaEventRecord(e0, st));
    for (int it = 0; it < 5 && !rc; ++it) rc = launch_bf16_tma(c, M, M.t3, M.t2, nullptr, M.t4, RF_SMOOTH, st);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    CK(c, cudaEventRecord(e1, st));
    CK(c, cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(c, cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      bestv = v;
    }
  }
  c->tma_variant = bestv;
  bool changed = bestv != before;
  float best_sc = 0.0f;
  if (M.sc && !c->sc_pinned) {   // the scaled-face step's shape, timed the same way
    const int before_sc = c->sc_variant;
    best_sc = 1e30f;
    int bv = 0;
    for (int v = 0; v < kScVariants; ++v) {
      c->sc_variant = v;
      int rc = launch_scaled(c, M.scblk16, M.t3, M.t2, M.t4, st, nullptr);
      if (!rc) CK(c, cudaEventRecord(e0, st));
      for (int it = 0; it < 5 && !rc; ++it) rc = launch_scaled(c, M.scblk16, M.t3, M.t2, M.t4, st, nullptr);
      if (rc) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
      }
      CK(c, cudaEventRecord(e1, st));
      CK(c, cudaEventSynchronize(e1));
      float ms = 0.0f;
      CK(c, cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_sc) {
        best_sc = ms;
        bv = v;
      }
    }
    c->sc_variant = bv;
    changed = changed || bv != before_sc;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (changed) {
    for (auto& g : M.graphs)
      if (g) cudaGraphExecDestroy(g);
    M.graphs.clear();
    M.g_m = 0;
  }
  if (c->verbose) {
    std::fprintf(stderr, "[autotune] bulk-copy smoothing shape %d (%.1f us per launch)\n", bestv, best * 1e3f / 5.0f);
    if (M.sc && !c->sc_pinned)
      std::fprintf(stderr, "[autotune] scaled-face smoothing shape %d (%.1f us per launch)\n", c->sc_variant,
                   best_sc * 1e3f / 5.0f);
  }
  return DG_OK;
}

}  // namespace

// ===========================================================================
extern "C" int dg_solve_mixed(dg_ctx* c, double* x, const double* b, double tol, int32_t m, int32_t max_its,
                              double inner_rtol, int32_t* its_out, double* res_out, int32_t* outer_out,
                              void* stream) {
  if (!c || !x || !b) return set_thread_error(DG_ERR_ARG, "dg_solve_mixed: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_solve_mixed: operator not built");
  if (m <= 0 || m > 256 || max_its < 0 || !(inner_rtol > 0.0 && inner_rtol < 1.0))
    return fail(c, DG_ERR_ARG, "dg_solve_mixed: need 1 <= m <= 256 and 0 < inner_rtol < 1");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
    if ((rc = autotune_mixed(c, st))) return rc;
  }
  if ((rc = ensure_krylov32(c, m))) return rc;
  CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));   // bulk-copy wait time-outs land here
  const int chunk = std::max(1, std::min(c->mixed_chunk, m));
  const int64_t n = c->nonods;
  double* r64 = c->d_t2;
  float* rhs32 = M.t2;
  float* d32 = M.t6;
  float* V0 = M.V;
  // starting residual: r = b for a zero x (no FP64 apply), else b - A x
  if (!M.nzflag && (rc = dalloc(c, &M.nzflag, 1))) return rc;
  CK(c, cudaMemsetAsync(M.nzflag, 0, sizeof(int), st));
  bnonzero_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(2 * c->nsm, (n + 255) / 256)), 256, 0, st>>>(
      x, n, M.nzflag);
  bump();
  CKL(c);
  int nzx = 1;
  CK(c, cudaMemcpyAsync(&nzx, M.nzflag, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  if (nzx) {
    if ((rc = residual(c, x, b, r64, nullptr, 0, st))) return rc;
  } else {
    CK(c, cudaMemcpyAsync(r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  }
  if ((rc = norm2(c, r64, c->d_scal, st))) return rc;
  double rn;
  if ((rc = read_scalar(c, c->d_scal, &rn, st))) return rc;
  int its = 0, outer = 0, status = DG_OK;
  std::vector<double> Hh((size_t)(m + 1) * m), y;
  while (rn > tol && its < max_its) {
    if (!std::isfinite(rn)) {
      status = DG_ERR_NUMERIC;
      c->err = "mixed solve: non-finite residual";
      break;
    }
    f64_to_f32_kernel<<<nblk(n, 256), 256, 0, st>>>(r64, rhs32, n, 1.0 / rn);
    bump();
    zero_f32_kernel<<<nblk(n, 256), 256, 0, st>>>(d32, n);
    bump();
    CKL(c);
    // solve the inner system only as far as the outer tolerance still needs
    const double target = std::max(inner_rtol, 0.5 * tol / rn);
    double beta0 = -1.0;
    bool inner_done = false;
    while (!inner_done && its < max_its) {
      // inner residual rhs - A d (d = 0 on the first cycle) into V0
      if (beta0 < 0.0) {
        CK(c, cudaMemcpyAsync(V0, rhs32, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
      } else {
        if ((rc = residual32(c, d32, rhs32, V0, nullptr, 0, st))) return rc;
      }
      if ((rc = norm32(c, V0, c->d_scal, st))) return rc;
      double beta;
      if ((rc = read_scalar(c, c->d_scal, &beta, st))) return rc;
      if (beta0 < 0.0) beta0 = beta;
      if (!(beta > target * beta0) || !std::isfinite(beta)) break;
      scale_kernel<float><<<nblk(n, 256), 256, 0, st>>>(V0, c->d_scal, V0, n);
      bump();
      CK(c, cudaMemsetAsync(M.H, 0, sizeof(double) * (m + 1) * m, st));
      // device-side convergence test: g = beta e1, threshold target * beta0
      M.gv_host.assign((size_t)3 * m + 2, 0.0);
      M.gv_host[2 * m] = beta;
      M.gv_host[3 * m + 1] = target * beta0;
      CK(c, cudaMemcpyAsync(M.gv, M.gv_host.data(), sizeof(double) * M.gv_host.size(), cudaMemcpyHostToDevice, st));
      CK(c, cudaMemsetAsync(M.kdone, 0, sizeof(int), st));
      int k = 0;
      bool conv = false, ok = true;
      // least-squares residual after the previous chunk (k_last steps); with
      // adaptive chunks a chunk that the observed rate says ends past the
      // target is cut to the predicted step count, so a refinement step
      // stops within a step of its target instead of up to chunk - 1 past it
      double est_last = beta;
      int k_last = 0;
      for (int j0 = 0; j0 < m;) {
        int cnt = std::min(chunk, m - j0);
        if (c->adaptive_chunk && k_last > 0 && est_last > target * beta0) {
          const double rate = std::pow(est_last / beta, 1.0 / k_last);
          if (rate > 0.0 && rate < 1.0) {
            const double need = std::ceil(std::log(target * beta0 / est_last) / std::log(rate));
            if (need >= 1.0 && need < (double)cnt) cnt = (int)need;
          }
        }
        int mode = 0, kd = 0;
        if ((rc = run_arnoldi32(c, j0, cnt, m, chunk, st, &mode))) return rc;
        CK(c, cudaMemcpyAsync(Hh.data(), M.H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
        CK(c, cudaMemcpyAsync(&kd, M.kdone, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(c, cudaStreamSynchronize(st));
        // steps that ran: all of the chunk, or (conditional chunk graph) up to
        // the step that met the threshold; the solution uses the Krylov space
        // of that step either way
        const int ran = (kd > 0 && mode == 2) ? kd - j0 : cnt;
        if (mode != 0) bump(chunk_kernels(c, j0, ran));
        its += ran;
        k = kd > 0 ? kd : j0 + cnt;
        double est = hessenberg_ls(Hh, m, k, beta, y, ok);
        if (!ok) break;
        if (kd > 0 || est <= target * beta0) {
          conv = true;
          break;
        }
        if (its >= max_its) break;
        est_last = est;
        k_last = k;
        j0 += cnt;
      }
      if (!ok) {
        status = DG_ERR_NUMERIC;
        c->err = "mixed solve: singular Hessenberg matrix";
        break;
      }
      CK(c, cudaMemcpyAsync(c->d_y, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
      combine32_kernel<<<nblk(n, 256), 256, 0, st>>>(M.Z, n, k, c->d_y, d32, n);
      bump();
      CKL(c);
      inner_done = conv;
    }
    if (status != DG_OK) break;
    axpy_f32_to_f64_kernel<<<nblk(n, 256), 256, 0, st>>>(x, d32, n, rn);
    bump();
    CKL(c);
    ++outer;
    const double rn_prev = rn;
    if ((rc = residual(c, x, b, r64, nullptr, 0, st))) return rc;
    if ((rc = norm2(c, r64, c->d_scal, st))) return rc;
    if ((rc = read_scalar(c, c->d_scal, &rn, st))) return rc;
    if (c->verbose)
      std::fprintf(stderr, "[dg_solve_mixed] outer %d: inner its total %d, target %.2e, |r| %.3e -> %.3e (x%.2e)\n",
                   outer, its, target, rn_prev, rn, rn / rn_prev);
  }
  if (its_out) *its_out = its;
  if (res_out) *res_out = rn;
  if (outer_out) *outer_out = outer;
  {
    int herr = 0;
    CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (herr == 3) {
      c->err = "mixed solve: a bulk-copy wait of the preconditioner timed out";
      return DG_ERR_CUDA;
    }
    if (herr == 5) {
      c->err = "mixed solve: shared-face table not in owner order";
      return DG_ERR_STATE;
    }
  }
  if (status == DG_OK && rn > tol) {
    c->err = "mixed solve reached the iteration limit";
    return DG_ERR_NOCONV;
  }
  return status;
}

// y = A x with the FP32 copy of the operator (FP32 vectors)
extern "C" int dg_apply_f32(dg_ctx* c, const float* x, float* y, void* stream) {
  if (!c || !x || !y) return set_thread_error(DG_ERR_ARG, "dg_apply_f32: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_apply_f32: operator not built");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  return residual32(c, x, nullptr, y, nullptr, RF_NEG, st);
}

// V-cycle legs of the mixed preconditioner as cluster launches (-1 = auto,
// 0 = the launch chain, 8 / 16 = that cluster size when it fits).  Takes
// effect at once for a built mixed operator; cached graphs are dropped.
extern "C" int dg_set_vcycle_cluster(dg_ctx* c, int32_t cluster, int32_t* chosen) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_vcycle_cluster: null context");
  if (cluster != -1 && cluster != 0 && cluster != 8 && cluster != 16)
    return fail(c, DG_ERR_ARG, "dg_set_vcycle_cluster: cluster must be -1, 0, 8 or 16");
  CK(c, cudaSetDevice(c->dev));
  c->vc32_cluster = cluster;
  Mixed& M = mixed_of(c);
  for (auto& g : M.graphs)
    if (g) cudaGraphExecDestroy(g);
  M.graphs.clear();
  M.g_m = 0;
  int rc;
  if (M.built && (rc = setup_vcycle_cluster(c, nullptr))) return rc;
  if (chosen) *chosen = M.built ? M.vc_cs : -1;
  return DG_OK;
}

// z = the mixed preconditioner (FP32 V-cycle with the BF16/FP32 block copies)
// applied once to r, FP32 vectors -- the reduced-precision counterpart of
// _um_left_precond.
extern "C" int dg_precond_f32(dg_ctx* c, const float* r, float* z, void* stream) {
  if (!c || !r || !z) return set_thread_error(DG_ERR_ARG, "dg_precond_f32: null argument");
  if (r == z) return fail(c, DG_ERR_ARG, "dg_precond_f32: z must not alias r");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_precond_f32: operator not built");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  return precond32(c, r, z, st);
}

// One smoothing step of the mixed preconditioner on FP32 vectors:
// x_out = x + W_pc (b - A_pc x), with the preconditioner's stored blocks
// (BF16 when precond_bf16) and smoother matrices -- the reduced-precision
// form of get_residual_or_smooth(do_smooth=True).  x_out must not alias x.
extern "C" int dg_smooth_pc(dg_ctx* c, const float* x, const float* b, float* x_out, void* stream) {
  if (!c || !x || !b || !x_out) return set_thread_error(DG_ERR_ARG, "dg_smooth_pc: null argument");
  if (x_out == x) return fail(c, DG_ERR_ARG, "dg_smooth_pc: x_out must not alias x");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_smooth_pc: operator not built");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  if (M.sc) {   // as the preconditioner runs it: c = W b first, then the scaled-face step
    if ((rc = launch_bf16_tma(c, M, nullptr, b, nullptr, x_out, RF_ZEROX | RF_SMOOTH, st, nullptr, M.chat)))
      return rc;
    return launch_scaled(c, M.scblk16, x, M.chat, x_out, st, nullptr);
  }
  return residual_pc(c, x, b, nullptr, x_out, RF_SMOOTH, st);
}

extern "C" int dg_smooth_scaled(dg_ctx* c, const float* x, const float* cv, float* x_out, void* stream) {
  if (!c || !x || !cv || !x_out) return set_thread_error(DG_ERR_ARG, "dg_smooth_scaled: null argument");
  if (x_out == x) return fail(c, DG_ERR_ARG, "dg_smooth_scaled: x_out must not alias x");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_smooth_scaled: operator not built");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  if (!M.sc) return fail(c, DG_ERR_STATE, "dg_smooth_scaled: the scaled face blocks are not in use");
  return launch_scaled(c, M.scblk16, x, cv, x_out, st, nullptr);
}

// Options of the mixed-precision preconditioner (take effect at the next
// mixed solve): smoother 0 = three point-Jacobi sweeps as the reference,
// 1 = damped block inverse smooth_w * A_ee^{-1}; precond_bf16 != 0 stores
// the preconditioner's blocks in BF16; dense_max = rows of the first SFC
// level solved exactly by a dense inverse (0 = V-cycle down to one node).
extern "C" int dg_set_mixed_options(dg_ctx* c, int32_t smoother, double smooth_w, int32_t precond_bf16,
                                    int32_t dense_max) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_mixed_options: null context");
  if ((smoother != 0 && smoother != 1) || !(smooth_w > 0.0 && smooth_w <= 2.0) || dense_max < 0 ||
      dense_max > 8192)
    return fail(c, DG_ERR_ARG, "dg_set_mixed_options: smoother 0|1, 0 < smooth_w <= 2, 0 <= dense_max <= 8192");
  c->mixed_smoother = smoother;
  c->mixed_smooth_w = smooth_w;
  c->precond_bf16 = precond_bf16 != 0;
  c->dense_max32 = dense_max;
  c->mixed_version = -1;   // rebuild the mixed operator copies
  Mixed& M = mixed_of(c);
  for (auto& g : M.graphs)
    if (g) cudaGraphExecDestroy(g);
  M.graphs.clear();
  M.g_m = 0;
  return DG_OK;
}

// Launch options: use_graph != 0 replays the Arnoldi cycles / chunks as CUDA
// graphs, use_pdl != 0 links the kernels of a mixed inner step by
// programmatic dependent launch.  Cached graphs are dropped and captured
// again with the new options at the next solve.
extern "C" int dg_set_launch_options(dg_ctx* c, int32_t use_graph, int32_t use_pdl) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_launch_options: null context");
  CK(c, cudaSetDevice(c->dev));
  c->use_graph = use_graph != 0;
  c->use_pdl = use_pdl != 0;
  if (c->arnoldi_exec) {
    cudaGraphExecDestroy(c->arnoldi_exec);
    c->arnoldi_exec = nullptr;
  }
  Mixed& M = mixed_of(c);
  for (auto& g : M.graphs)
    if (g) cudaGraphExecDestroy(g);
  M.graphs.clear();
  M.g_m = 0;
  return DG_OK;
}
