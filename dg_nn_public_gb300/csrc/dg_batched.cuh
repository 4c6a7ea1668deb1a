// Batched mixed-precision solve: up to kNR right-hand sides on one operator
// (P3 tetrahedra), in lockstep.  Included into dg_solver.cu after
// dg_mixed.cuh; it reuses the mixed-precision operator copies (chunked FP32
// and BF16 blocks, BF16 smoother matrices, FP32 SFC levels, dense coarse
// inverse) and adds batched kernels on RHS-interleaved vectors:
//
//   X[(e * 20 + n) * kNR + r]      (element-major, then node, then RHS)
//
// so that one node of an element is a contiguous run of kNR values and every
// kernel reads the stored blocks once for all right-hand sides.
//
//   outer (FP64, per RHS):  r_k = b_k - A x_k with the FP64 blocks; stop the
//                           RHS when ||r_k|| <= tol_k
//   inner (FP32, batched):  right-preconditioned flexible GMRES(m) on
//                           A d_k = r_k / ||r_k|| for all active k together,
//                           one Hessenberg matrix per RHS (host, FP64);
//                           classical Gram-Schmidt per RHS
//   x_k += ||r_k|| d_k
#pragma once

namespace {

constexpr int kNR = 64;   // right-hand sides per batch (lanes of the batched kernels)

// ---------------------------------------------------------------------------
// r = b - A x (FP32 sums) for kNR right-hand sides, one CTA per element
// (128 threads): warp w owns rows 5w .. 5w+4, lane l owns RHS 2l, 2l+1.
// The element's five blocks (chunked row layout, FP32 or BF16), its
// smoother matrix (with RF_SMOOTH) and the gathered x of the element and its
// four face neighbours (5 x 20 x kNR FP32) are staged in shared memory;
// four columns of a block row are one 16-byte (FP32) or 8-byte (BF16) word.
// Flags as residual_kernel: RF_ZEROX (x = 0), RF_NEG (r = A x - b),
// RF_RESTRICT (r1 = P^T res per corner), RF_SMOOTH (x_out = x + W res).
template <typename MT>
struct BRow4;

template <>
struct BRow4<float> {
  // columns n .. n+3 (n a multiple of 4) of row m of a chunked FP32 block
  static __device__ __forceinline__ float4 get(const float* blk, int m, int n) {
    return *reinterpret_cast<const float4*>(blk + (n >> 2) * 80 + m * 4);
  }
};

template <>
struct BRow4<__nv_bfloat16> {
  static __device__ __forceinline__ float4 get(const __nv_bfloat16* blk, int m, int n) {
    const int off = n < 8 ? m * 8 + n : (n < 16 ? kC20Off1 + m * 8 + (n - 8) : kC20Off2 + m * 4);
    const uint2 w = *reinterpret_cast<const uint2*>(blk + off);
    return make_float4(bf_lo(w.x), bf_hi(w.x), bf_lo(w.y), bf_hi(w.y));
  }
};

template <typename MT>
__global__ void __launch_bounds__(128) bres_kernel(const MT* __restrict__ blk, const MT* __restrict__ W,
                                                   const int* __restrict__ nbe, const float* __restrict__ x,
                                                   const float* __restrict__ b, float* __restrict__ r,
                                                   float* __restrict__ x_out, int64_t B, int flags,
                                                   const float* __restrict__ P, float* __restrict__ r1,
                                                   const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4;
  const float ws = wsp ? *wsp : 1.0f;
  constexpr int BLK = N * N;                     // entries per block
  constexpr int EL_BYTES = (F + 1) * BLK * (int)sizeof(MT);
  constexpr int W_BYTES = BLK * (int)sizeof(MT);
  __shared__ __align__(16) unsigned char As[EL_BYTES];
  __shared__ __align__(16) unsigned char Ws[W_BYTES];
  __shared__ __align__(16) float xs[F + 1][N][kNR];
  __shared__ __align__(16) float rs[N][kNR];
  __shared__ float Ps[N * F];   // P converted once per CTA, not per use (FP64 conversions are slow here)
  __shared__ int nbs[F];
  const int64_t e = blockIdx.x;
  if (e >= B) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  if (tid < F) nbs[tid] = nbe[e * F + tid];
  if ((flags & RF_RESTRICT) && tid < N * F) Ps[tid] = (float)P[tid];
  if (!zerox) {
    const uint4* src = reinterpret_cast<const uint4*>(blk + e * (F + 1) * BLK);
    for (int i = tid; i < EL_BYTES / 16; i += 128) reinterpret_cast<uint4*>(As)[i] = src[i];
  }
  if (smooth) {
    const uint4* src = reinterpret_cast<const uint4*>(W + e * BLK);
    for (int i = tid; i < W_BYTES / 16; i += 128) reinterpret_cast<uint4*>(Ws)[i] = src[i];
  }
  __syncthreads();
  if (!zerox) {
    // 5 blocks x 20 nodes x kNR values = 5 * 20 * 16 float4; loads first
    constexpr int kItems = (F + 1) * N * (kNR / 4);
    constexpr int kPer = (kItems + 127) / 128;
    float4 v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * 128;
      v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i < kItems) {
        const int bb = i / (N * (kNR / 4)), rem = i - (i / (N * (kNR / 4))) * (N * (kNR / 4));
        const int64_t src_e = bb == 0 ? e : (int64_t)nbs[bb - 1];
        if (src_e >= 0) v[u] = reinterpret_cast<const float4*>(x + src_e * N * kNR)[rem];
      }
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * 128;
      if (i < kItems) reinterpret_cast<float4*>(&xs[0][0][0])[i] = v[u];
    }
  }
  __syncthreads();
  const int m0 = warp * 5, r0 = lane * 2;
  float acc[5][2];
#pragma unroll
  for (int i = 0; i < 5; ++i) acc[i][0] = acc[i][1] = 0.0f;
  if (!zerox) {
    const MT* A = reinterpret_cast<const MT*>(As);
#pragma unroll 1
    for (int bb = 0; bb <= F; ++bb) {
      if (bb > 0 && nbs[bb - 1] < 0) continue;
      const MT* Ab = A + bb * BLK;
#pragma unroll
      for (int n = 0; n < N; n += 4) {
        float4 a[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) a[i] = BRow4<MT>::get(Ab, m0 + i, n);
        const float2 x0 = *reinterpret_cast<const float2*>(&xs[bb][n][r0]);
        const float2 x1 = *reinterpret_cast<const float2*>(&xs[bb][n + 1][r0]);
        const float2 x2 = *reinterpret_cast<const float2*>(&xs[bb][n + 2][r0]);
        const float2 x3 = *reinterpret_cast<const float2*>(&xs[bb][n + 3][r0]);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          acc[i][0] = fmaf(a[i].x, x0.x, acc[i][0]);
          acc[i][1] = fmaf(a[i].x, x0.y, acc[i][1]);
          acc[i][0] = fmaf(a[i].y, x1.x, acc[i][0]);
          acc[i][1] = fmaf(a[i].y, x1.y, acc[i][1]);
          acc[i][0] = fmaf(a[i].z, x2.x, acc[i][0]);
          acc[i][1] = fmaf(a[i].z, x2.y, acc[i][1]);
          acc[i][0] = fmaf(a[i].w, x3.x, acc[i][0]);
          acc[i][1] = fmaf(a[i].w, x3.y, acc[i][1]);
        }
      }
    }
  }
  float res[5][2];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const int64_t o = (e * N + m0 + i) * kNR + r0;
    float2 bv = make_float2(0.f, 0.f);
    if (b) bv = *reinterpret_cast<const float2*>(b + o);
    res[i][0] = bv.x - acc[i][0];
    res[i][1] = bv.y - acc[i][1];
    if (r) {
      const float s = (flags & RF_NEG) ? -1.0f : 1.0f;
      *reinterpret_cast<float2*>(r + o) = make_float2(s * res[i][0], s * res[i][1]);
    }
  }
  if (flags & (RF_RESTRICT | RF_SMOOTH)) {
#pragma unroll
    for (int i = 0; i < 5; ++i) *reinterpret_cast<float2*>(&rs[m0 + i][r0]) = make_float2(res[i][0], res[i][1]);
    __syncthreads();
    if (flags & RF_RESTRICT) {
      // r1[(e*4 + c) * kNR + q] = sum_n P[n][c] rs[n][q]; 4 x kNR outputs, 2 per thread
      for (int o = tid; o < F * kNR; o += 128) {
        const int cc = o / kNR, q = o % kNR;
        float t = 0.0f;
#pragma unroll
        for (int n = 0; n < N; ++n) t += Ps[n * F + cc] * rs[n][q];
        r1[(e * F + cc) * kNR + q] = t;
      }
    }
    if (smooth) {
      const MT* Wm = reinterpret_cast<const MT*>(Ws);
      float c[5][2];
#pragma unroll
      for (int i = 0; i < 5; ++i) c[i][0] = c[i][1] = 0.0f;
#pragma unroll
      for (int n = 0; n < N; n += 4) {
        const float2 q0 = *reinterpret_cast<const float2*>(&rs[n][r0]);
        const float2 q1 = *reinterpret_cast<const float2*>(&rs[n + 1][r0]);
        const float2 q2 = *reinterpret_cast<const float2*>(&rs[n + 2][r0]);
        const float2 q3 = *reinterpret_cast<const float2*>(&rs[n + 3][r0]);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          const float4 w = BRow4<MT>::get(Wm, m0 + i, n);
          c[i][0] = fmaf(w.x, q0.x, c[i][0]);
          c[i][1] = fmaf(w.x, q0.y, c[i][1]);
          c[i][0] = fmaf(w.y, q1.x, c[i][0]);
          c[i][1] = fmaf(w.y, q1.y, c[i][1]);
          c[i][0] = fmaf(w.z, q2.x, c[i][0]);
          c[i][1] = fmaf(w.z, q2.y, c[i][1]);
          c[i][0] = fmaf(w.w, q3.x, c[i][0]);
          c[i][1] = fmaf(w.w, q3.y, c[i][1]);
        }
      }
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const int64_t o = (e * N + m0 + i) * kNR + r0;
        float2 xo = make_float2(ws * c[i][0], ws * c[i][1]);
        if (!zerox) {
          xo.x += xs[0][m0 + i][r0];
          xo.y += xs[0][m0 + i][r0 + 1];
        }
        *reinterpret_cast<float2*>(x_out + o) = xo;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The same step with BF16 blocks on the tensor cores (warp-level
// mma.sync m16n8k16 / m16n8k8, BF16 inputs, FP32 accumulation).  Per element
// Y (20 x kNR) = A_stack (20 x 100) X_stack (100 x kNR): the A operand is the
// element's BF16 blocks in the chunked row layout, read directly as
// fragments (columns 0-15 of a block = one k16 step over chunks 0 and 1,
// columns 16-19 = one k8 step over chunk 2 with the upper half zeroed); the
// B operand is X_stack in shared memory as [k][RHS] BF16 rows (k = 24 *
// block + node, nodes 20..23 zero; 144-byte rows, so the eight rows an
// ldmatrix reads fall in distinct banks), loaded with ldmatrix.trans.  x is
// split into BF16 hi + lo parts (two MMAs each), so x keeps ~16 bits through
// the product.  One CTA per element, 4 warps; warp w owns RHS 16w .. 16w+15.
// The smoothing product W res goes through the tensor cores the same way.
constexpr int kXK = 120;        // k slots (5 blocks x 24)
constexpr int kXRow = 144;      // bytes per k slot row (64 BF16 + 16 bytes pad)

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_bf16_1688(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

__device__ __forceinline__ void ldm_x2_trans(uint32_t& r0, uint32_t& r1, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_addr(p)));
}

__device__ __forceinline__ void ldm_x1_trans(uint32_t& r0, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x1.trans.shared.b16 {%0}, [%1];" : "=r"(r0) : "r"(smem_addr(p)));
}

// hi / lo BF16 parts of four consecutive values, stored at two 8-byte words
// (lower column in the low half of each 32-bit word); two values per
// conversion instruction, round to nearest even as a per-value conversion
__device__ __forceinline__ void store_split4(unsigned char* hi, unsigned char* lo, float4 v) {
  const __nv_bfloat162 h01 = __floats2bfloat162_rn(v.x, v.y), h23 = __floats2bfloat162_rn(v.z, v.w);
  const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
  const __nv_bfloat162 l01 = __floats2bfloat162_rn(v.x - f01.x, v.y - f01.y);
  const __nv_bfloat162 l23 = __floats2bfloat162_rn(v.z - f23.x, v.w - f23.y);
  uint2 H, L;
  H.x = *reinterpret_cast<const uint32_t*>(&h01);
  H.y = *reinterpret_cast<const uint32_t*>(&h23);
  L.x = *reinterpret_cast<const uint32_t*>(&l01);
  L.y = *reinterpret_cast<const uint32_t*>(&l23);
  *reinterpret_cast<uint2*>(hi) = H;
  *reinterpret_cast<uint2*>(lo) = L;
}

// one block (20x20 BF16, chunked) times the slab of k slots kb .. kb+23 of
// Xs (hi or lo): accumulates into acc[mt][nt], m tiles mt = 0, 1 (rows 0-15,
// 16-31), n tiles nt = 0, 1 (RHS rbase + 8 nt ..)
template <int NT>
__device__ __forceinline__ void mma_block_t(float (&acc)[2][NT][4], const unsigned char* blk, const unsigned char* Xs,
                                            int kb, int rbase, int lane) {
  const int g = lane >> 2, t = lane & 3;
  uint32_t a[2][4], a8[2][2];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int r0 = mt * 16 + g, r1 = r0 + 8;
    const bool v0 = r0 < 20, v1 = r1 < 20;
    a[mt][0] = v0 ? *reinterpret_cast<const uint32_t*>(blk + r0 * 16 + 4 * t) : 0u;
    a[mt][1] = v1 ? *reinterpret_cast<const uint32_t*>(blk + r1 * 16 + 4 * t) : 0u;
    a[mt][2] = v0 ? *reinterpret_cast<const uint32_t*>(blk + 2 * kC20Off1 + r0 * 16 + 4 * t) : 0u;
    a[mt][3] = v1 ? *reinterpret_cast<const uint32_t*>(blk + 2 * kC20Off1 + r1 * 16 + 4 * t) : 0u;
    a8[mt][0] = (v0 && t < 2) ? *reinterpret_cast<const uint32_t*>(blk + 2 * kC20Off2 + r0 * 8 + 4 * t) : 0u;
    a8[mt][1] = (v1 && t < 2) ? *reinterpret_cast<const uint32_t*>(blk + 2 * kC20Off2 + r1 * 8 + 4 * t) : 0u;
  }
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int q0 = rbase + nt * 8;
    uint32_t b0, b1, b8;
    // lanes 0-15: rows kb .. kb+15 (two 8x8 matrices); lanes 0-7: rows kb+16 .. kb+23
    ldm_x2_trans(b0, b1, Xs + (size_t)(kb + (lane & 15)) * kXRow + q0 * 2);
    ldm_x1_trans(b8, Xs + (size_t)(kb + 16 + (lane & 7)) * kXRow + q0 * 2);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      mma_bf16_16816(acc[mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
      mma_bf16_1688(acc[mt][nt], a8[mt][0], a8[mt][1], b8);
    }
  }
}

__device__ __forceinline__ void mma_block(float (&acc)[2][2][4], const unsigned char* blk, const unsigned char* Xs,
                                          int kb, int rbase, int lane) {
  mma_block_t<2>(acc, blk, Xs, kb, rbase, lane);
}

template <int NWARP>
__global__ void __launch_bounds__(NWARP * 32) bres_mma_kernel(const __nv_bfloat16* __restrict__ blk,
                                                       const __nv_bfloat16* __restrict__ W,
                                                       const int* __restrict__ nbe, const float* __restrict__ x,
                                                       const float* __restrict__ b, float* __restrict__ r,
                                                       float* __restrict__ x_out, int64_t B, int flags,
                                                       const float* __restrict__ P, float* __restrict__ r1,
                                                       const float* __restrict__ wsp, float* __restrict__ c_out) {
  constexpr int N = 20, F = 4;
  const float ws = wsp ? *wsp : 1.0f;
  __shared__ __align__(16) unsigned char As[(F + 1) * 800];
  __shared__ __align__(16) unsigned char Ws[800];
  __shared__ __align__(16) unsigned char Xhi[kXK * kXRow];
  __shared__ __align__(16) unsigned char Xlo[kXK * kXRow];
  __shared__ __align__(16) float rs[N][kNR];
  __shared__ float Ps[N * F];   // P converted once per CTA, not per use (FP64 conversions are slow here)
  __shared__ int nbs[F];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  if (tid < F) nbs[tid] = nbe[e * F + tid];
  if (flags & RF_RESTRICT)
    for (int i = tid; i < N * F; i += NWARP * 32) Ps[i] = (float)P[i];
  if (!zerox)
    for (int i = tid; i < (F + 1) * 800 / 16; i += NWARP * 32)
      reinterpret_cast<uint4*>(As)[i] = reinterpret_cast<const uint4*>(blk + e * 2000)[i];
  if (smooth)
    for (int i = tid; i < 800 / 16; i += NWARP * 32) reinterpret_cast<uint4*>(Ws)[i] = reinterpret_cast<const uint4*>(W + e * 400)[i];
  // zero pad slots (nodes 20..23 of every block): 5 x 4 rows x 64 RHS, hi and lo
  for (int i = tid; i < (F + 1) * 4 * (kNR / 4); i += NWARP * 32) {
    const int bb = i / (4 * (kNR / 4)), rem = i % (4 * (kNR / 4));
    const int row = bb * 24 + 20 + rem / (kNR / 4), q4 = rem % (kNR / 4);
    *reinterpret_cast<uint2*>(Xhi + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
    *reinterpret_cast<uint2*>(Xlo + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
  }
  __syncthreads();
  constexpr int NT = 8 / NWARP;                            // n8 tiles per warp
  const int rbase = warp * 8 * NT;
  float acc[2][NT][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.0f;
  // the epilogue's b and x values of this thread, loaded with the gather
  float2 bpre[2][2][NT], xpre[2][2][NT];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int row = mt * 16 + g + 8 * hh;
        const int64_t o = (e * N + row) * kNR + rbase + nt * 8 + 2 * t;
        const bool ok = row < N;
        bpre[mt][hh][nt] = (ok && b) ? *reinterpret_cast<const float2*>(b + o) : make_float2(0.f, 0.f);
        xpre[mt][hh][nt] = (ok && smooth && !zerox) ? *reinterpret_cast<const float2*>(x + o) : make_float2(0.f, 0.f);
      }
  if (!zerox) {
    // X_stack rows: slot 24 bb + n = x[nb_bb][n][:] (hi / lo), coalesced
    // float4 reads; all of a thread's loads are issued before the first
    // conversion, so the gather costs one round trip, not thirteen
    constexpr int kItems = (F + 1) * N * (kNR / 4);          // 1600 float4
    constexpr int kPer = (kItems + NWARP * 32 - 1) / (NWARP * 32);
    float4 v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * NWARP * 32;
      v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i < kItems) {
        const int bb = i / (N * (kNR / 4)), rem = i % (N * (kNR / 4));
        const int64_t src_e = bb == 0 ? e : (int64_t)nbs[bb - 1];
        if (src_e >= 0) v[u] = reinterpret_cast<const float4*>(x + src_e * N * kNR)[rem];
      }
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * NWARP * 32;
      if (i < kItems) {
        const int bb = i / (N * (kNR / 4)), rem = i % (N * (kNR / 4));
        const int n = rem / (kNR / 4), q4 = rem % (kNR / 4);
        const int row = bb * 24 + n;
        store_split4(Xhi + row * kXRow + q4 * 8, Xlo + row * kXRow + q4 * 8, v[u]);
      }
    }
    __syncthreads();
#pragma unroll 1
    for (int bb = 0; bb <= F; ++bb) {
      if (bb > 0 && nbs[bb - 1] < 0) continue;
      mma_block_t<NT>(acc, As + bb * 800, Xhi, bb * 24, rbase, lane);
      mma_block_t<NT>(acc, As + bb * 800, Xlo, bb * 24, rbase, lane);
    }
  }
  // epilogue: rows (mt*16 + g [+8]), RHS rbase + nt*8 + 2t (+1)
  const float sgn = (flags & RF_NEG) ? -1.0f : 1.0f;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int row = mt * 16 + g + 8 * hh;
      if (row >= N) continue;
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int q = rbase + nt * 8 + 2 * t;
        const int64_t o = (e * N + row) * kNR + q;
        const float2 bv = bpre[mt][hh][nt];
        const float2 res = make_float2(bv.x - acc[mt][nt][2 * hh], bv.y - acc[mt][nt][2 * hh + 1]);
        if (r) *reinterpret_cast<float2*>(r + o) = make_float2(sgn * res.x, sgn * res.y);
        *reinterpret_cast<float2*>(&rs[row][q]) = res;
      }
    }
  if (!(flags & (RF_RESTRICT | RF_SMOOTH))) return;
  __syncthreads();
  if (flags & RF_RESTRICT) {
    for (int o = tid; o < F * kNR; o += NWARP * 32) {
      const int cc = o / kNR, q = o % kNR;
      float s = 0.0f;
#pragma unroll
      for (int n = 0; n < N; ++n) s += Ps[n * F + cc] * rs[n][q];
      r1[(e * F + cc) * kNR + q] = s;
    }
  }
  if (smooth) {
    // res rows into slots 0..19 (slots 20..23 are still zero)
    for (int i = tid; i < N * (kNR / 4); i += NWARP * 32) {
      const int n = i / (kNR / 4), q4 = i % (kNR / 4);
      store_split4(Xhi + n * kXRow + q4 * 8, Xlo + n * kXRow + q4 * 8, reinterpret_cast<const float4*>(&rs[n][0])[q4]);
    }
    __syncthreads();
    float c2[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) c2[mt][nt][i] = 0.0f;
    mma_block_t<NT>(c2, Ws, Xhi, 0, rbase, lane);
    mma_block_t<NT>(c2, Ws, Xlo, 0, rbase, lane);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int row = mt * 16 + g + 8 * hh;
        if (row >= N) continue;
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const int q = rbase + nt * 8 + 2 * t;
          const int64_t o = (e * N + row) * kNR + q;
          const float2 xv = xpre[mt][hh][nt];
          *reinterpret_cast<float2*>(x_out + o) =
              make_float2(ws * c2[mt][nt][2 * hh] + xv.x, ws * c2[mt][nt][2 * hh + 1] + xv.y);
          // W res, kept for the scaled-face steps (bsc_mma_kernel)
          if (c_out) *reinterpret_cast<float2*>(c_out + o) = make_float2(c2[mt][nt][2 * hh], c2[mt][nt][2 * hh + 1]);
        }
      }
  }
}

// ---------------------------------------------------------------------------
// Batched smoothing step on the scaled face blocks S_ef = W_e A_ef (BF16,
// chunked, four per element; the single-RHS form is smooth_scaled_tma_kernel):
//   X_out = X + s (C - w X - sum_f S_ef X_nb(f)),   C = W B,
// C formed by the zero-start step (c_out of bres_mma_kernel).  The face
// products run on the tensor cores as in bres_mma_kernel (x split into BF16
// hi + lo, mma.sync m16n8k16 + m16n8k8), but per element there are four
// block products instead of five, no smoother product and no second
// shared-memory round: the epilogue works on the accumulators directly.
template <int NWARP>
__global__ void __launch_bounds__(NWARP * 32) bsc_mma_kernel(const __nv_bfloat16* __restrict__ sblk,
                                                      const int* __restrict__ nbe, const float* __restrict__ x,
                                                      const float* __restrict__ cv, float* __restrict__ x_out,
                                                      int64_t B, float w, const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4;
  const float ws = wsp ? *wsp : 1.0f;
  __shared__ __align__(16) unsigned char As[F * 800];
  __shared__ __align__(16) unsigned char Xhi[F * 24 * kXRow];
  __shared__ __align__(16) unsigned char Xlo[F * 24 * kXRow];
  __shared__ int nbs[F];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  if (tid < F) nbs[tid] = nbe[e * F + tid];
  for (int i = tid; i < F * 800 / 16; i += NWARP * 32)
    reinterpret_cast<uint4*>(As)[i] = reinterpret_cast<const uint4*>(sblk + e * F * 400)[i];
  for (int i = tid; i < F * 4 * (kNR / 4); i += NWARP * 32) {   // zero pad slots (nodes 20..23)
    const int bb = i / (4 * (kNR / 4)), rem = i % (4 * (kNR / 4));
    const int row = bb * 24 + 20 + rem / (kNR / 4), q4 = rem % (kNR / 4);
    *reinterpret_cast<uint2*>(Xhi + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
    *reinterpret_cast<uint2*>(Xlo + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
  }
  constexpr int NT = 8 / NWARP;
  const int rbase = warp * 8 * NT;
  float acc[2][NT][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.0f;
  // the epilogue's c and x values of this thread, loaded with the gather
  float2 cpre[2][2][NT], xpre[2][2][NT];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int row = mt * 16 + g + 8 * hh;
        const int64_t o = (e * N + row) * kNR + rbase + nt * 8 + 2 * t;
        const bool ok = row < N;
        cpre[mt][hh][nt] = ok ? *reinterpret_cast<const float2*>(cv + o) : make_float2(0.f, 0.f);
        xpre[mt][hh][nt] = ok ? *reinterpret_cast<const float2*>(x + o) : make_float2(0.f, 0.f);
      }
  __syncthreads();   // nbs
  {
    constexpr int kItems = F * N * (kNR / 4);   // 1280 float4
    constexpr int kPer = (kItems + NWARP * 32 - 1) / (NWARP * 32);
    float4 v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * NWARP * 32;
      v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i < kItems) {
        const int bb = i / (N * (kNR / 4)), rem = i % (N * (kNR / 4));
        const int64_t src_e = nbs[bb];
        if (src_e >= 0) v[u] = reinterpret_cast<const float4*>(x + src_e * N * kNR)[rem];
      }
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = tid + u * NWARP * 32;
      if (i < kItems) {
        const int bb = i / (N * (kNR / 4)), rem = i % (N * (kNR / 4));
        const int n = rem / (kNR / 4), q4 = rem % (kNR / 4);
        const int row = bb * 24 + n;
        store_split4(Xhi + row * kXRow + q4 * 8, Xlo + row * kXRow + q4 * 8, v[u]);
      }
    }
  }
  __syncthreads();
#pragma unroll 1
  for (int bb = 0; bb < F; ++bb) {
    if (nbs[bb] < 0) continue;
    mma_block_t<NT>(acc, As + bb * 800, Xhi, bb * 24, rbase, lane);
    mma_block_t<NT>(acc, As + bb * 800, Xlo, bb * 24, rbase, lane);
  }
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int row = mt * 16 + g + 8 * hh;
      if (row >= N) continue;
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int64_t o = (e * N + row) * kNR + rbase + nt * 8 + 2 * t;
        const float2 xv = xpre[mt][hh][nt], cc = cpre[mt][hh][nt];
        *reinterpret_cast<float2*>(x_out + o) =
            make_float2(xv.x + ws * (cc.x - fmaf(w, xv.x, acc[mt][nt][2 * hh])),
                        xv.y + ws * (cc.y - fmaf(w, xv.y, acc[mt][nt][2 * hh + 1])));
      }
    }
}

// ---------------------------------------------------------------------------
// Persistent, pipelined form of bres_mma_kernel: kBS CTAs per SM walk the
// elements e = blockIdx.x, + gridDim.x, ...; an element's operands arrive by
// bulk copies (cp.async.bulk, mbarrier completion) into a ring of kBStages
// shared-memory stages -- its BF16 blocks (4,000 B), its smoother matrix
// (800 B), the x slabs of the element and its face neighbours (5 x 5,120 B)
// and its b slab (5,120 B) -- so that the copies of the next element are in
// flight while this one is converted to BF16 hi / lo rows and multiplied on
// the tensor cores.  Same arithmetic as bres_mma_kernel (same results).
// Every mbarrier wait is bounded: on time-out *err = 3, the CTA waits
// (bounded) for its own copies in flight and returns.
constexpr int kBStages = 2;
constexpr int kBS = 2;                                   // CTAs per SM
constexpr int kSlab = 20 * kNR * 4;                      // 5,120 bytes: one element's x (or b) slab
constexpr int kStOffW = 4000, kStOffX = 4800, kStOffB = 4800 + 5 * kSlab;
constexpr int kStageB = kStOffB + kSlab;                 // 35,520 bytes
constexpr int kBDyn = kBStages * kStageB + 2 * kXK * kXRow + 20 * kNR * 4;   // stages + Xhi/Xlo + rs

constexpr int kBT = 256;                                 // threads: 8 warps, warp w owns RHS 8w .. 8w+7
__global__ void __launch_bounds__(kBT, kBS) bres_mma_tma_kernel(
    const __nv_bfloat16* __restrict__ blk, const __nv_bfloat16* __restrict__ W, const int* __restrict__ nbe,
    const float* __restrict__ x, const float* __restrict__ b, float* __restrict__ r, float* __restrict__ x_out,
    int64_t B, int flags, const float* __restrict__ P, float* __restrict__ r1, int* __restrict__ err,
    const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4;
  const float ws = wsp ? *wsp : 1.0f;
  extern __shared__ __align__(128) unsigned char bsm[];
  unsigned char* stages = bsm;
  unsigned char* Xhi = bsm + kBStages * kStageB;
  unsigned char* Xlo = Xhi + kXK * kXRow;
  float(*rs)[kNR] = reinterpret_cast<float(*)[kNR]>(Xlo + kXK * kXRow);
  __shared__ __align__(8) uint64_t bar[kBStages];
  __shared__ int nbs[kBStages][F];
  __shared__ float Ps[N][F];
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  const int64_t stride = gridDim.x;
  for (int i = tid; i < N * F; i += kBT) Ps[i / F][i % F] = (float)P[i];
  // zero pad slots (nodes 20..23 of every block), never overwritten
  for (int i = tid; i < (F + 1) * 4 * (kNR / 4); i += kBT) {
    const int bb = i / (4 * (kNR / 4)), rem = i % (4 * (kNR / 4));
    const int row = bb * 24 + 20 + rem / (kNR / 4), q4 = rem % (kNR / 4);
    *reinterpret_cast<uint2*>(Xhi + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
    *reinterpret_cast<uint2*>(Xlo + row * kXRow + q4 * 8) = make_uint2(0u, 0u);
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int s2 = 0; s2 < kBStages; ++s2) mbar_init(&bar[s2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // thread 0 issues the copies of the CTA's k-th element into stage k % kBStages
  auto issue = [&](int64_t k, int4 nb) {
    const int64_t e = blockIdx.x + k * stride;
    if (e >= B) return;
    const int s2 = (int)(k % kBStages);
    unsigned char* st = stages + (size_t)s2 * kStageB;
    nbs[s2][0] = nb.x;
    nbs[s2][1] = nb.y;
    nbs[s2][2] = nb.z;
    nbs[s2][3] = nb.w;
    const int nbv[F] = {nb.x, nb.y, nb.z, nb.w};
    uint32_t bytes = 0;
    if (!zerox) {
      bytes += 4000 + kSlab;
      for (int f = 0; f < F; ++f)
        if (nbv[f] >= 0) bytes += kSlab;
    }
    if (smooth) bytes += 800;
    if (b) bytes += kSlab;
    mbar_expect_tx(&bar[s2], bytes);
    if (!zerox) {
      bulk_copy_g2s(st, blk + e * 2000, 4000, &bar[s2]);
      bulk_copy_g2s(st + kStOffX, x + e * (int64_t)N * kNR, kSlab, &bar[s2]);
      for (int f = 0; f < F; ++f)
        if (nbv[f] >= 0) bulk_copy_g2s(st + kStOffX + (1 + f) * kSlab, x + (int64_t)nbv[f] * N * kNR, kSlab, &bar[s2]);
    }
    if (smooth) bulk_copy_g2s(st + kStOffW, W + e * 400, 800, &bar[s2]);
    if (b) bulk_copy_g2s(st + kStOffB, b + e * (int64_t)N * kNR, kSlab, &bar[s2]);
  };
  auto load_nb = [&](int64_t k) {
    const int64_t e = blockIdx.x + k * stride;
    return e < B ? reinterpret_cast<const int4*>(nbe)[e] : make_int4(-1, -1, -1, -1);
  };
  int4 nb_next = make_int4(-1, -1, -1, -1);
  if (tid == 0) {
    for (int k = 0; k < kBStages; ++k) issue(k, load_nb(k));
    nb_next = load_nb(kBStages);
  }
  const int rbase = warp * 8;
  const float sgn = (flags & RF_NEG) ? -1.0f : 1.0f;
  int64_t k = 0;
  for (int64_t e = blockIdx.x; e < B; e += stride, ++k) {
    const int s2 = (int)(k % kBStages);
    if (!mbar_wait_bounded(&bar[s2], (uint32_t)((k / kBStages) & 1))) {
      atomicExch(err, 3);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    const unsigned char* st = stages + (size_t)s2 * kStageB;
    const float* xst = reinterpret_cast<const float*>(st + kStOffX);   // [5][20][kNR]
    const float* bst = reinterpret_cast<const float*>(st + kStOffB);   // [20][kNR]
    float acc[2][1][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < 1; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.0f;
    if (!zerox) {
      for (int i = tid; i < (F + 1) * N * (kNR / 4); i += kBT) {
        const int bb = i / (N * (kNR / 4)), rem = i % (N * (kNR / 4));
        if (bb > 0 && nbs[s2][bb - 1] < 0) continue;
        const int n = rem / (kNR / 4), q4 = rem % (kNR / 4);
        const int row = bb * 24 + n;
        store_split4(Xhi + row * kXRow + q4 * 8, Xlo + row * kXRow + q4 * 8,
                     reinterpret_cast<const float4*>(xst)[i]);
      }
      __syncthreads();
#pragma unroll 1
      for (int bb = 0; bb <= F; ++bb) {
        if (bb > 0 && nbs[s2][bb - 1] < 0) continue;
        mma_block_t<1>(acc, st + bb * 800, Xhi, bb * 24, rbase, lane);
        mma_block_t<1>(acc, st + bb * 800, Xlo, bb * 24, rbase, lane);
      }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int row = mt * 16 + g + 8 * hh;
        if (row >= N) continue;
#pragma unroll
        for (int nt = 0; nt < 1; ++nt) {
          const int q = rbase + nt * 8 + 2 * t;
          const int64_t o = (e * N + row) * kNR + q;
          const float2 bv = b ? *reinterpret_cast<const float2*>(bst + row * kNR + q) : make_float2(0.f, 0.f);
          const float2 res = make_float2(bv.x - acc[mt][nt][2 * hh], bv.y - acc[mt][nt][2 * hh + 1]);
          if (r) *reinterpret_cast<float2*>(r + o) = make_float2(sgn * res.x, sgn * res.y);
          *reinterpret_cast<float2*>(&rs[row][q]) = res;
        }
      }
    if (flags & (RF_RESTRICT | RF_SMOOTH)) {
      __syncthreads();   // rs complete; Xhi / Xlo no longer read by the MMAs
      if (flags & RF_RESTRICT) {
        for (int o = tid; o < F * kNR; o += kBT) {
          const int cc = o / kNR, q = o % kNR;
          float sum = 0.0f;
#pragma unroll
          for (int n = 0; n < N; ++n) sum += Ps[n][cc] * rs[n][q];
          r1[(e * F + cc) * kNR + q] = sum;
        }
      }
      if (smooth) {
        for (int i = tid; i < N * (kNR / 4); i += kBT) {
          const int n = i / (kNR / 4), q4 = i % (kNR / 4);
          store_split4(Xhi + n * kXRow + q4 * 8, Xlo + n * kXRow + q4 * 8,
                       reinterpret_cast<const float4*>(&rs[n][0])[q4]);
        }
        __syncthreads();
        float c2[2][1][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < 1; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) c2[mt][nt][i] = 0.0f;
        mma_block_t<1>(c2, st + kStOffW, Xhi, 0, rbase, lane);
        mma_block_t<1>(c2, st + kStOffW, Xlo, 0, rbase, lane);
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const int row = mt * 16 + g + 8 * hh;
            if (row >= N) continue;
#pragma unroll
            for (int nt = 0; nt < 1; ++nt) {
              const int q = rbase + nt * 8 + 2 * t;
              const int64_t o = (e * N + row) * kNR + q;
              float2 xo = make_float2(ws * c2[mt][nt][2 * hh], ws * c2[mt][nt][2 * hh + 1]);
              if (!zerox) {
                const float2 xv = *reinterpret_cast<const float2*>(xst + row * kNR + q);
                xo.x += xv.x;
                xo.y += xv.y;
              }
              *reinterpret_cast<float2*>(x_out + o) = xo;
            }
          }
      }
    }
    __syncthreads();   // stage s2, Xhi / Xlo and rs free again
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(k + kBStages, nb_next);
      nb_next = load_nb(k + kBStages + 1);
    }
  }
  if (abort_flag && tid == 0) {
    for (int64_t j = k; j < k + kBStages; ++j) {
      if (blockIdx.x + j * stride >= B) break;
      (void)mbar_wait_bounded(&bar[j % kBStages], (uint32_t)((j / kBStages) & 1));
    }
  }
}

}  // namespace

#include "dg_batched_tc.cuh"

namespace {

// ---------------------------------------------------------------------------
// DG <-> CG P1 transfers and SFC levels on kNR columns (thread per (row, RHS))

// out[pos(i)][q] = sum over DG copies (e, c) of vertex i of w_ec * r1[(e, c)][q];
// the vertex's entries and weights are staged once per CTA (kNR at a time),
// so each FP64 weight is converted once, not once per RHS
__global__ void bgather_kernel(const float* __restrict__ r1, const int* __restrict__ gptr,
                               const int* __restrict__ gent, const float* __restrict__ wdg,
                               const int* __restrict__ pos, float* __restrict__ out, int ncg) {
  __shared__ int es[kNR];
  __shared__ float ws[kNR];
  const int i = blockIdx.x;
  const int q = threadIdx.x;
  if (i >= ncg) return;
  const int k0 = gptr[i], k1 = gptr[i + 1];
  float acc = 0.0f;
  for (int kb = k0; kb < k1; kb += kNR) {
    const int cnt = min(kNR, k1 - kb);
    __syncthreads();   // the previous chunk is consumed
    if (q < cnt) {
      const int ent = gent[kb + q];
      es[q] = ent;
      ws[q] = (float)wdg[ent];
    }
    __syncthreads();
    for (int k = 0; k < cnt; ++k) acc += ws[k] * r1[(int64_t)es[k] * kNR + q];
  }
  out[(int64_t)pos[i] * kNR + q] = acc;
}

// x[(e, n)][q] += sum_c P[n][c] * w_ec * ecg[pos(p1cg[e][c])][q]; one CTA of
// 320 threads per element: thread (n, quad of 4 RHS)
__global__ void __launch_bounds__(320) bprolong_kernel(float* __restrict__ x, const float* __restrict__ ecg,
                                                       const int* __restrict__ pos, const int* __restrict__ p1cg,
                                                       const float* __restrict__ wdg, const float* __restrict__ P,
                                                       int64_t B) {
  __shared__ int vp[4];
  __shared__ float wc[4];
  __shared__ float Ps[20][4];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  if (tid < 4) {
    vp[tid] = pos[p1cg[e * 4 + tid]];
    wc[tid] = (float)wdg[e * 4 + tid];
  }
  if (tid < 80) Ps[tid / 4][tid % 4] = (float)P[tid];
  __syncthreads();
  const int n = tid / (kNR / 4), q4 = tid % (kNR / 4);
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float4 ev = reinterpret_cast<const float4*>(ecg + (int64_t)vp[c] * kNR)[q4];
    const float f = Ps[n][c] * wc[c];
    v.x += f * ev.x;
    v.y += f * ev.y;
    v.z += f * ev.z;
    v.w += f * ev.w;
  }
  float4* xp = reinterpret_cast<float4*>(x + (e * 20 + n) * kNR) + q4;
  float4 xv = *xp;
  xv.x += v.x;
  xv.y += v.y;
  xv.z += v.z;
  xv.w += v.w;
  *xp = xv;
}

// rr = b - A e_in;  e_out = e_in + w rr / diag (e_in = NULL: zero guess)
__global__ void bjacobi_kernel(const int* __restrict__ rowptr, const int* __restrict__ col,
                               const float* __restrict__ val, const float* __restrict__ diag,
                               const float* __restrict__ e_in, const float* __restrict__ b,
                               float* __restrict__ e_out, float* __restrict__ rr_out, int n, float w) {
  const int i = blockIdx.x * (blockDim.x / kNR) + threadIdx.x / kNR;
  const int q = threadIdx.x % kNR;
  if (i >= n) return;
  float s = 0.0f;
  if (e_in)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * e_in[(int64_t)col[k] * kNR + q];
  const int64_t o = (int64_t)i * kNR + q;
  const float rr = b[o] - s;
  e_out[o] = (e_in ? e_in[o] : 0.0f) + rr / diag[i] * w;
  if (rr_out) rr_out[o] = rr;
}

__global__ void brestrict_kernel(const float* __restrict__ rr, const float* __restrict__ e, float* __restrict__ r_next,
                                 float* __restrict__ e_next, int n, int nn) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nn * kNR) return;
  const int i = (int)(t / kNR), q = (int)(t % kNR);
  const int a = 2 * i, bq = 2 * i + 1;
  r_next[t] = rr[(int64_t)a * kNR + q] + (bq < n ? rr[(int64_t)bq * kNR + q] : 0.0f);
  e_next[t] = e[(int64_t)a * kNR + q] + (bq < n ? e[(int64_t)bq * kNR + q] : 0.0f);
}

__global__ void bprolong_lev_kernel(float* __restrict__ e, const float* __restrict__ e_next, const int* __restrict__ up,
                                    int n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * kNR) return;
  const int i = (int)(t / kNR), q = (int)(t % kNR);
  e[t] += e_next[(int64_t)up[i] * kNR + q];
}

// E = Ainv R on the dense coarse level: 8-row tiles (enough CTAs for the
// GPU at ~1,000 rows), k in tiles of 64 staged in shared memory; 128
// threads, each 1 row x 4 RHS
__global__ void __launch_bounds__(128) bdense_kernel(const float* __restrict__ Ainv, const float* __restrict__ R,
                                                     float* __restrict__ E, int n) {
  __shared__ float As[8][65];
  __shared__ __align__(16) float Rs[64][kNR];
  const int row0 = blockIdx.x * 8;
  const int tid = threadIdx.x;
  const int rr = tid / 16, q4 = tid % 16;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k0 = 0; k0 < n; k0 += 64) {
    for (int i = tid; i < 8 * 64; i += 128) {
      const int r = i / 64, k = i % 64;
      As[r][k] = (row0 + r < n && k0 + k < n) ? Ainv[(int64_t)(row0 + r) * n + k0 + k] : 0.0f;
    }
    for (int i = tid; i < 64 * (kNR / 4); i += 128) {
      const int k = i / (kNR / 4), qq = i % (kNR / 4);
      reinterpret_cast<float4*>(&Rs[k][0])[qq] =
          k0 + k < n ? reinterpret_cast<const float4*>(R + (int64_t)(k0 + k) * kNR)[qq] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
      const float4 rv = reinterpret_cast<const float4*>(&Rs[k][0])[q4];
      const float a = As[rr][k];
      acc.x = fmaf(a, rv.x, acc.x);
      acc.y = fmaf(a, rv.y, acc.y);
      acc.z = fmaf(a, rv.z, acc.z);
      acc.w = fmaf(a, rv.w, acc.w);
    }
    __syncthreads();
  }
  if (row0 + rr < n) reinterpret_cast<float4*>(E + (int64_t)(row0 + rr) * kNR)[q4] = acc;
}

// The same product with the k loop staged by asynchronous copies: CTA tile
// 16 rows x 64 RHS (one CTA per SM at ~2,300 rows), 128 threads of 2 rows x
// 4 RHS each, k tiles of 128 double-buffered in shared memory (cp.async,
// 16-byte pieces).  Each output is one FMA chain over k = 0, 1, ..., n-1, as
// in bdense_kernel, so both give the same bits.
constexpr int kDnRows = 16, kDnK = 128;
constexpr int kDnSmem = 2 * (kDnRows * kDnK + kDnK * kNR) * 4;   // 81,920 bytes

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool full) {
  // full = false: zero-fill the 16 bytes (src-size 0), src stays in bounds
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(full ? 16 : 0)
               : "memory");
}

__global__ void __launch_bounds__(128) bdense2_kernel(const float* __restrict__ Ainv, const float* __restrict__ R,
                                                      float* __restrict__ E, int n) {
  extern __shared__ __align__(16) float dn_smem[];
  float* As = dn_smem;                                // [2][kDnRows][kDnK]
  float* Rs = dn_smem + 2 * kDnRows * kDnK;           // [2][kDnK][kNR]
  const int row0 = blockIdx.x * kDnRows;
  const int tid = threadIdx.x;
  const int ty = tid / 16, tx = tid % 16;             // rows 2 ty, 2 ty + 1; RHS 4 tx .. 4 tx + 3
  const bool vec = (n & 3) == 0;                      // 16-byte aligned rows of Ainv
  auto stage = [&](int buf, int k0) {
    float* as = As + buf * kDnRows * kDnK;
    float* rs = Rs + buf * kDnK * kNR;
    for (int i = tid; i < kDnRows * (kDnK / 4); i += 128) {
      const int r = i / (kDnK / 4), k4 = i % (kDnK / 4);
      const int row = row0 + r, k = k0 + 4 * k4;
      if (vec) {
        const bool ok = row < n && k < n;
        cp_async16(as + r * kDnK + 4 * k4, Ainv + (ok ? (int64_t)row * n + k : 0), ok);
      } else {
        for (int u = 0; u < 4; ++u)
          as[r * kDnK + 4 * k4 + u] = (row < n && k + u < n) ? Ainv[(int64_t)row * n + k + u] : 0.0f;
      }
    }
    for (int i = tid; i < kDnK * (kNR / 4); i += 128) {
      const int k = i / (kNR / 4), q4 = i % (kNR / 4);
      const bool ok = k0 + k < n;
      cp_async16(rs + k * kNR + 4 * q4, R + (ok ? (int64_t)(k0 + k) * kNR + 4 * q4 : 0), ok);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
  const int nt = (n + kDnK - 1) / kDnK;
  stage(0, 0);
  for (int it = 0; it < nt; ++it) {
    const int buf = it & 1;
    if (it + 1 < nt) {
      stage(buf ^ 1, (it + 1) * kDnK);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const float* as = As + buf * kDnRows * kDnK;
    const float* rs = Rs + buf * kDnK * kNR;
    const int kmax = min(kDnK, n - it * kDnK);
    for (int k = 0; k < kmax; ++k) {
      const float a0 = as[(2 * ty) * kDnK + k], a1 = as[(2 * ty + 1) * kDnK + k];
      const float4 rv = reinterpret_cast<const float4*>(rs + k * kNR)[tx];
      acc0.x = fmaf(a0, rv.x, acc0.x);
      acc0.y = fmaf(a0, rv.y, acc0.y);
      acc0.z = fmaf(a0, rv.z, acc0.z);
      acc0.w = fmaf(a0, rv.w, acc0.w);
      acc1.x = fmaf(a1, rv.x, acc1.x);
      acc1.y = fmaf(a1, rv.y, acc1.y);
      acc1.z = fmaf(a1, rv.z, acc1.z);
      acc1.w = fmaf(a1, rv.w, acc1.w);
    }
    __syncthreads();   // the buffer is refilled by the next stage call
  }
  const int r0 = row0 + 2 * ty, r1 = r0 + 1;
  if (r0 < n) reinterpret_cast<float4*>(E + (int64_t)r0 * kNR)[tx] = acc0;
  if (r1 < n) reinterpret_cast<float4*>(E + (int64_t)r1 * kNR)[tx] = acc1;
}

// ---------------------------------------------------------------------------
// Gram-Schmidt per RHS on interleaved vectors.  A block is 256 threads =
// 4 row lanes x kNR RHS; per-thread sums FP32, the 4 lanes and the blocks
// combined in FP64 (fixed order).

// partial[(blk * 32 + j) * kNR + q] = sum over the block's rows of V_j[row][q] z[row][q],
// j = 8 blockIdx.y .. +7; 256 threads = 16 row lanes x 16 RHS quads
__global__ void __launch_bounds__(256) bmdot_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                    const float* __restrict__ z, int64_t n,
                                                    double* __restrict__ partial) {
  __shared__ float4 red[16][8][kNR / 4];
  const int q4 = threadIdx.x % 16, lane = threadIdx.x / 16;
  const int j0 = blockIdx.y * 8;
  const int cnt = min(8, nv - j0);
  float4 acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int64_t step = (int64_t)gridDim.x * 16;
  for (int64_t row = (int64_t)blockIdx.x * 16 + lane; row < n; row += 2 * step) {
    // two rows per iteration: 18 loads in flight per thread
    const int64_t row2 = row + step;
    const bool has2 = row2 < n;
    const float4 zv = reinterpret_cast<const float4*>(z + row * kNR)[q4];
    const float4 zv2 = has2 ? reinterpret_cast<const float4*>(z + row2 * kNR)[q4] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 v[8], v2[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      v[j] = j < cnt ? reinterpret_cast<const float4*>(V + (size_t)(j0 + j) * ld + row * kNR)[q4]
                     : make_float4(0.f, 0.f, 0.f, 0.f);
      v2[j] = (j < cnt && has2) ? reinterpret_cast<const float4*>(V + (size_t)(j0 + j) * ld + row2 * kNR)[q4]
                                : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      acc[j].x = fmaf(v[j].x, zv.x, acc[j].x);
      acc[j].y = fmaf(v[j].y, zv.y, acc[j].y);
      acc[j].z = fmaf(v[j].z, zv.z, acc[j].z);
      acc[j].w = fmaf(v[j].w, zv.w, acc[j].w);
      acc[j].x = fmaf(v2[j].x, zv2.x, acc[j].x);
      acc[j].y = fmaf(v2[j].y, zv2.y, acc[j].y);
      acc[j].z = fmaf(v2[j].z, zv2.z, acc[j].z);
      acc[j].w = fmaf(v2[j].w, zv2.w, acc[j].w);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) red[lane][j][q4] = acc[j];
  __syncthreads();
  for (int o = threadIdx.x; o < cnt * kNR; o += 256) {
    const int j = o / kNR, q = o % kNR;
    double s = 0.0;
    for (int l = 0; l < 16; ++l) s += (double)reinterpret_cast<const float*>(&red[l][j][0])[q];
    partial[((int64_t)blockIdx.x * 32 + j0 + j) * kNR + q] = s;
  }
}

// Low-register forms of the per-RHS Gram-Schmidt kernels (the float4 forms
// above hold 16 or 32 float4 loads per thread: 112 / 255 registers, a
// quarter / an eighth of the SM's warps).  A thread handles 4 RHS of one row
// per iteration and at most 8 basis vectors at a time (~64 registers), 256
// threads per block and 4 blocks per SM, so a block row streams with half
// the SM's warps, each with 8 16-byte loads in flight.
__global__ void __launch_bounds__(256, 4) bmdot2_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                       const float* __restrict__ z, int64_t n,
                                                       double* __restrict__ partial) {
  __shared__ float4 red[16][8][kNR / 4];
  const int q4 = threadIdx.x % 16, lane = threadIdx.x / 16;
  const int j0 = blockIdx.y * 8;
  const int cnt = min(8, nv - j0);
  float4 acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t row = (int64_t)blockIdx.x * 16 + lane; row < n; row += (int64_t)gridDim.x * 16) {
    const float4 zv = reinterpret_cast<const float4*>(z + row * kNR)[q4];
    float4 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      v[j] = j < cnt ? reinterpret_cast<const float4*>(V + (size_t)(j0 + j) * ld + row * kNR)[q4]
                     : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      acc[j].x = fmaf(v[j].x, zv.x, acc[j].x);
      acc[j].y = fmaf(v[j].y, zv.y, acc[j].y);
      acc[j].z = fmaf(v[j].z, zv.z, acc[j].z);
      acc[j].w = fmaf(v[j].w, zv.w, acc[j].w);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) red[lane][j][q4] = acc[j];
  __syncthreads();
  for (int o = threadIdx.x; o < cnt * kNR; o += 256) {
    const int j = o / kNR, q = o % kNR;
    double sum = 0.0;
    for (int l = 0; l < 16; ++l) sum += (double)reinterpret_cast<const float*>(&red[l][j][0])[q];
    partial[((int64_t)blockIdx.x * 32 + j0 + j) * kNR + q] = sum;
  }
}

__global__ void __launch_bounds__(256, 4) baxpy2_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                       const double* __restrict__ h, float* __restrict__ z,
                                                       int64_t n, double* __restrict__ partial) {
  __shared__ float4 hs[32][kNR / 4];
  __shared__ float4 red[16][kNR / 4];
  const int q4 = threadIdx.x % 16, lane = threadIdx.x / 16;
  for (int o = threadIdx.x; o < 32 * kNR; o += 256)
    reinterpret_cast<float*>(&hs[0][0])[o] = o < nv * kNR ? (float)h[o] : 0.0f;
  __syncthreads();
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t row = (int64_t)blockIdx.x * 16 + lane; row < n; row += (int64_t)gridDim.x * 16) {
    float4* zp = reinterpret_cast<float4*>(z + row * kNR) + q4;
    float4 zv = *zp;
    for (int i0 = 0; i0 < nv; i0 += 8) {
      float4 v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        v[j] = i0 + j < nv ? reinterpret_cast<const float4*>(V + (size_t)(i0 + j) * ld + row * kNR)[q4]
                           : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 hv = hs[(i0 + j) & 31][q4];
        zv.x -= v[j].x * hv.x;
        zv.y -= v[j].y * hv.y;
        zv.z -= v[j].z * hv.z;
        zv.w -= v[j].w * hv.w;
      }
    }
    *zp = zv;
    acc.x = fmaf(zv.x, zv.x, acc.x);
    acc.y = fmaf(zv.y, zv.y, acc.y);
    acc.z = fmaf(zv.z, zv.z, acc.z);
    acc.w = fmaf(zv.w, zv.w, acc.w);
  }
  red[lane][q4] = acc;
  __syncthreads();
  if (threadIdx.x < kNR) {
    double sum = 0.0;
    for (int l = 0; l < 16; ++l) sum += (double)reinterpret_cast<const float*>(&red[l][0])[threadIdx.x];
    partial[(int64_t)blockIdx.x * kNR + threadIdx.x] = sum;
  }
}

// h[j * kNR + q] = sum over blocks of partial[(blk * 32 + j) * kNR + q]:
// block (j, RHS group of 16) of 1024 threads = 64 lanes x 16 RHS; lane l
// sums blocks l, l + 64, ... with eight loads in flight, then the 64 lane
// sums in a fixed tree
__global__ void __launch_bounds__(1024) breduce2_kernel(const double* __restrict__ partial, int nblk,
                                                         double* __restrict__ h) {
  __shared__ double red[64][16];
  const int j = blockIdx.x, qi = threadIdx.x % 16, lane = threadIdx.x / 16;
  const int q = blockIdx.y * 16 + qi;
  double sum = 0.0;
  for (int b0 = lane; b0 < nblk; b0 += 64 * 8) {
    double v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int bk = b0 + 64 * i;
      v[i] = bk < nblk ? partial[((int64_t)bk * 32 + j) * kNR + q] : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) sum += v[i];
  }
  red[lane][qi] = sum;
  __syncthreads();
  for (int w = 32; w >= 1; w >>= 1) {
    if (lane < w) red[lane][qi] += red[lane + w][qi];
    __syncthreads();
  }
  if (lane == 0) h[j * kNR + q] = red[0][qi];
}

// bfinish_kernel with the norm partials summed by 1024 threads (16 lanes x
// 64 RHS, eight loads in flight per lane, fixed tree)
__global__ void __launch_bounds__(1024) bfinish2_kernel(const double* __restrict__ partial, int nblk,
                                                         const double* __restrict__ h, int nv, int j, int m,
                                                         double* __restrict__ H, float* __restrict__ inv) {
  __shared__ double red[16][kNR];
  const int q = threadIdx.x % kNR, lane = threadIdx.x / kNR;
  double sum = 0.0;
  for (int b0 = lane; b0 < nblk; b0 += 16 * 8) {
    double v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int bk = b0 + 16 * i;
      v[i] = bk < nblk ? partial[(int64_t)bk * kNR + q] : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) sum += v[i];
  }
  red[lane][q] = sum;
  __syncthreads();
  for (int w = 8; w >= 1; w >>= 1) {
    if (lane < w) red[lane][q] += red[lane + w][q];
    __syncthreads();
  }
  if (lane == 0) {
    double* Hq = H + (size_t)q * (m + 1) * m + (size_t)j * (m + 1);
    for (int i = 0; i < nv; ++i) Hq[i] = h[i * kNR + q];
    const double t = sqrt(red[0][q]);
    Hq[nv] = t;
    inv[q] = t > 0.0 ? (float)(1.0 / t) : 0.0f;
  }
}

// h[j * kNR + q] = sum over blocks of partial[(blk * 32 + j) * kNR + q]
__global__ void breduce_kernel(const double* __restrict__ partial, int nblk, int nv, double* __restrict__ h) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nv * kNR) return;
  const int j = o / kNR, q = o % kNR;
  double s = 0.0;
  for (int bk = 0; bk < nblk; ++bk) s += partial[((int64_t)bk * 32 + j) * kNR + q];
  h[o] = s;
}

// z[row][q] -= sum_j V_j[row][q] h[j][q]; partial[blk * kNR + q] = slice of |z_new[:, q]|^2
__global__ void __launch_bounds__(256) baxpy_kernel(const float* __restrict__ V, int64_t ld, int nv,
                                                    const double* __restrict__ h, float* __restrict__ z, int64_t n,
                                                    double* __restrict__ partial) {
  __shared__ float4 hs[32][kNR / 4];
  __shared__ float4 red[16][kNR / 4];
  const int q4 = threadIdx.x % 16, lane = threadIdx.x / 16;
  for (int o = threadIdx.x; o < 32 * kNR; o += 256)
    reinterpret_cast<float*>(&hs[0][0])[o] = o < nv * kNR ? (float)h[o] : 0.0f;
  __syncthreads();
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t row = (int64_t)blockIdx.x * 16 + lane; row < n; row += (int64_t)gridDim.x * 16) {
    float4* zp = reinterpret_cast<float4*>(z + row * kNR) + q4;
    float4 zv = *zp;
    // all (up to 32) basis loads of the row are issued before the first use
    float4 v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j)
      v[j] = j < nv ? reinterpret_cast<const float4*>(V + (size_t)j * ld + row * kNR)[q4]
                    : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float4 hv = hs[j][q4];
      zv.x -= v[j].x * hv.x;
      zv.y -= v[j].y * hv.y;
      zv.z -= v[j].z * hv.z;
      zv.w -= v[j].w * hv.w;
    }
    *zp = zv;
    acc.x = fmaf(zv.x, zv.x, acc.x);
    acc.y = fmaf(zv.y, zv.y, acc.y);
    acc.z = fmaf(zv.z, zv.z, acc.z);
    acc.w = fmaf(zv.w, zv.w, acc.w);
  }
  red[lane][q4] = acc;
  __syncthreads();
  if (threadIdx.x < kNR) {
    const int q = threadIdx.x;
    double s = 0.0;
    for (int l = 0; l < 16; ++l) s += (double)reinterpret_cast<const float*>(&red[l][0])[q];
    partial[(int64_t)blockIdx.x * kNR + q] = s;
  }
}

// Hessenberg column j of every RHS q (H[q][(m+1) * m], column-major):
// H_q[i][j] = h[i][q] for i < nv, H_q[nv][j] = |z_q|; inv[q] = 1/|z_q| (0 if 0)
__global__ void bfinish_kernel(const double* __restrict__ partial, int nblk, const double* __restrict__ h, int nv,
                               int j, int m, double* __restrict__ H, float* __restrict__ inv) {
  const int q = threadIdx.x;
  if (q >= kNR) return;
  double* Hq = H + (size_t)q * (m + 1) * m + (size_t)j * (m + 1);
  for (int i = 0; i < nv; ++i) Hq[i] = h[i * kNR + q];
  double s = 0.0;
  for (int bk = 0; bk < nblk; ++bk) s += partial[(int64_t)bk * kNR + q];
  const double t = sqrt(s);
  Hq[nv] = t;
  inv[q] = t > 0.0 ? (float)(1.0 / t) : 0.0f;
}

// v[row][q] = z[row][q] * inv[q]  (float4; total a multiple of kNR)
__global__ void bscale_kernel(const float* __restrict__ z, const float* __restrict__ inv, float* __restrict__ v,
                              int64_t total) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // float4 index
  if (t * 4 >= total) return;
  const int q = (int)((t * 4) % kNR);
  float4 a = reinterpret_cast<const float4*>(z)[t];
  a.x *= inv[q];
  a.y *= inv[q + 1];
  a.z *= inv[q + 2];
  a.w *= inv[q + 3];
  reinterpret_cast<float4*>(v)[t] = a;
}

// d[row][q] += sum_j Z_j[row][q] y[j][q]; y (k <= 32 rows of kNR) is
// converted to FP32 once per CTA into shared memory, not once per entry
__global__ void __launch_bounds__(256) bcombine_kernel(const float* __restrict__ Z, int64_t ld, int k,
                                                       const double* __restrict__ y, float* __restrict__ d,
                                                       int64_t total) {
  __shared__ float ys[32 * kNR];
  for (int o = threadIdx.x; o < k * kNR; o += blockDim.x) ys[o] = (float)y[o];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int q = (int)(t % kNR);
  float s = d[t];
  for (int j = 0; j < k; ++j) s += Z[(size_t)j * ld + t] * ys[j * kNR + q];
  d[t] = s;
}

// column norms^2 of an interleaved vector: partial[blk * kNR + q]
__global__ void __launch_bounds__(256) bnorm_kernel(const float* __restrict__ z, int64_t n,
                                                    double* __restrict__ partial) {
  __shared__ float red[4][kNR];
  const int q = threadIdx.x % kNR, lane4 = threadIdx.x / kNR;
  float acc = 0.0f;
  for (int64_t row = (int64_t)blockIdx.x * 4 + lane4; row < n; row += (int64_t)gridDim.x * 4) {
    const float v = z[row * kNR + q];
    acc = fmaf(v, v, acc);
  }
  red[lane4][q] = acc;
  __syncthreads();
  if (threadIdx.x < kNR) {
    double s = 0.0;
    for (int l = 0; l < 4; ++l) s += (double)red[l][threadIdx.x];
    partial[(int64_t)blockIdx.x * kNR + threadIdx.x] = s;
  }
}

// out[q] = sqrt(sum_blk partial[blk * kNR + q]); inv[q] = 1/out (0 if 0)
__global__ void bnorm_finish_kernel(const double* __restrict__ partial, int nblk, double* __restrict__ out,
                                    float* __restrict__ inv) {
  const int q = threadIdx.x;
  if (q >= kNR) return;
  double s = 0.0;
  for (int bk = 0; bk < nblk; ++bk) s += partial[(int64_t)bk * kNR + q];
  const double t = sqrt(s);
  out[q] = t;
  if (inv) inv[q] = t > 0.0 ? (float)(1.0 / t) : 0.0f;
}

// interleave: out[row][q] = (float)(in_q[row] * s[q]) for q < nrhs (in_q = in + q * n), 0 beyond
__global__ void binterleave_kernel(const double* __restrict__ in, int64_t n, int nrhs, const double* __restrict__ s,
                                   float* __restrict__ out) {
  __shared__ float tile[32][33];
  const int64_t row0 = (int64_t)blockIdx.x * 32;
  const int q0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const int q = q0 + k;
    const int64_t row = row0 + tx;
    float v = 0.0f;
    if (q < nrhs && row < n) v = (float)(in[(int64_t)q * n + row] * s[q]);
    tile[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int64_t row = row0 + k;
    if (row < n) out[row * kNR + q0 + tx] = tile[tx][k];
  }
}

// de-interleave and update: x_q[row] += a[q] * d[row][q] (FP64) for q < nrhs
__global__ void bupdate_kernel(double* __restrict__ x, int64_t n, int nrhs, const double* __restrict__ a,
                               const float* __restrict__ d) {
  __shared__ float tile[32][33];
  const int64_t row0 = (int64_t)blockIdx.x * 32;
  const int q0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += 8) {
    const int64_t row = row0 + k;
    tile[k][tx] = row < n ? d[row * kNR + q0 + tx] : 0.0f;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int q = q0 + k;
    const int64_t row = row0 + tx;
    if (q < nrhs && row < n && a[q] != 0.0) x[(int64_t)q * n + row] += a[q] * (double)tile[tx][k];
  }
}

// ---------------------------------------------------------------------------
struct BatchState {
  int m = 0;
  float *V = nullptr, *Z = nullptr;
  float *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *t6 = nullptr;
  float* r1 = nullptr;                      // (B * 4, kNR)
  std::vector<float*> lr, le, le2, lrr;     // per SFC level (n_l, kNR)
  double *H = nullptr, *part = nullptr, *h = nullptr, *nrm = nullptr, *scl = nullptr, *y = nullptr;
  float* inv = nullptr;
  double* r64 = nullptr;                    // (kNR, nonods) FP64 residuals, RHS-major
  float* chat = nullptr;                    // C = W R of the scaled-face steps (nonods, kNR)
  // damping factors of the batched preconditioner's smoothing steps (its own
  // Chebyshev degree and interval, from the mixed build's lambda_max)
  float* d_wsb = nullptr;
  int wsb_version = -1;
  int nblk = 0;
  // BF16 blocks + smoother matrices in the padded tensor-core layout of
  // bres_tc05_kernel (5,760 bytes per element), rebuilt per mixed build
  __nv_bfloat16* tc = nullptr;
  int tc_version = -1;
  // smoothing-kernel autotuner: per-variant microseconds of one launch
  // (-1 = not timed), the mixed build it was taken for
  float tune_us[kBatchedVariants] = {-1.f, -1.f, -1.f, -1.f, -1.f, -1.f, -1.f};
  int tune_version = -1;
  // the preconditioner's iterates in the split tensor-core layout (variant 5)
  unsigned char *xs1 = nullptr, *xs2 = nullptr;
  // one CUDA graph per inner Arnoldi step index j (preconditioner, apply,
  // Gram-Schmidt), the kernels each one launches, and the state it was
  // captured for: any change of that state drops them all
  std::vector<cudaGraphExec_t> step_graph;
  std::vector<int> step_kern;
  std::vector<const void*> step_key;
  ~BatchState() {
    for (auto& g : step_graph)
      if (g) cudaGraphExecDestroy(g);
  }
};

void destroy_batch(void* batch) { delete static_cast<BatchState*>(batch); }

int ensure_split(dg_ctx* c, BatchState& S) {
  int rc;
  if (!S.xs1 && (rc = dalloc(c, &S.xs1, (size_t)c->B * kSplit))) return rc;
  if (!S.xs2 && (rc = dalloc(c, &S.xs2, (size_t)c->B * kSplit))) return rc;
  return DG_OK;
}

// the padded tensor-core layout of the preconditioner's BF16 blocks
int ensure_tc_layout(dg_ctx* c, Mixed& M, BatchState& S, cudaStream_t st) {
  if (S.tc && S.tc_version == c->mixed_version) return DG_OK;
  int rc;
  if (!S.tc && (rc = dalloc(c, &S.tc, (size_t)c->B * (kTcElem / 2)))) return rc;
  const int64_t tot = c->B * (int64_t)(kTcElem / 2);
  tc_layout_kernel<<<nblk(tot, 256), 256, 0, st>>>(M.blk16, M.W16, c->d_nbe, S.tc, c->B);
  bump();
  CKL(c);
  S.tc_version = c->mixed_version;
  return DG_OK;
}

BatchState& batch_of(Mixed& M) {
  if (!M.batch) M.batch = new BatchState();
  return *static_cast<BatchState*>(M.batch);
}

int ensure_batch(dg_ctx* c, int m) {
  Mixed& M = mixed_of(c);
  BatchState& S = batch_of(M);
  int rc;
  const size_t nv = (size_t)c->nonods * kNR;
  if (!S.t1) {
    for (float** t : {&S.t1, &S.t2, &S.t3, &S.t4, &S.t6})
      if ((rc = dalloc(c, t, nv))) return rc;
    if ((rc = dalloc(c, &S.r1, (size_t)c->B * 4 * kNR))) return rc;
    S.nblk = 2 * c->nsm;
    // partial sums for up to 4 * nsm blocks (the low-register Gram-Schmidt)
    if ((rc = dalloc(c, &S.part, (size_t)4 * c->nsm * 32 * kNR))) return rc;
    if ((rc = dalloc(c, &S.h, (size_t)32 * kNR))) return rc;
    if ((rc = dalloc(c, &S.nrm, (size_t)kNR))) return rc;
    if ((rc = dalloc(c, &S.scl, (size_t)kNR))) return rc;
    if ((rc = dalloc(c, &S.y, (size_t)32 * kNR))) return rc;
    if ((rc = dalloc(c, &S.inv, (size_t)kNR))) return rc;
    if ((rc = dalloc(c, &S.r64, (size_t)c->nonods * kNR))) return rc;
    S.lr.assign(M.lev.size(), nullptr);
    S.le = S.le2 = S.lrr = S.lr;
    for (size_t l = 0; l < M.lev.size(); ++l) {
      const size_t n = (size_t)M.lev[l].n * kNR;
      if ((rc = dalloc(c, &S.lr[l], n)) || (rc = dalloc(c, &S.le[l], n)) || (rc = dalloc(c, &S.le2[l], n)) ||
          (rc = dalloc(c, &S.lrr[l], n)))
        return rc;
    }
  }
  if (S.m < m) {
    if ((rc = dalloc(c, &S.V, (size_t)(m + 1) * nv))) return rc;
    if ((rc = dalloc(c, &S.Z, (size_t)m * nv))) return rc;
    if ((rc = dalloc(c, &S.H, (size_t)kNR * (m + 1) * m))) return rc;
    S.m = m;
  }
  return DG_OK;
}

template <typename MT>
int bres(dg_ctx* c, const MT* blk, const MT* W, const float* x, const float* b, float* r, float* x_out, int flags,
         float* r1, cudaStream_t st, const float* ws = nullptr) {
  if (c->B > 0)
    bres_kernel<MT><<<(unsigned)c->B, 128, 0, st>>>(blk, W, c->d_nbe, x, b, r, x_out, c->B, flags, c->d_P32, r1, ws);
  bump();
  CKL(c);
  return DG_OK;
}

// split-x smoothing step (bres_tcs_kernel); x_out is split with RF_OUT_SPLIT
int btcs(dg_ctx* c, BatchState& S, const unsigned char* xs, const float* b, void* xo, int flags, float* rr1,
         const float* ws, cudaStream_t st) {
  if (!S.tc || ((flags & RF_SMOOTH) && !xo) || ((flags & RF_RESTRICT) && !rr1) || !b)
    return fail(c, DG_ERR_STATE, "batched split-x step: operand buffers not set up");
  if (c->batched_kernel == 6) {   // warp-specialized, one CTA per SM
    const unsigned g = (unsigned)std::min<int64_t>(c->B, (int64_t)c->nsm);
    if (g)
      bres_tcw_kernel<<<g, kTwT, kTwDyn, st>>>(S.tc, c->d_nbe, xs, b, xo, c->B, flags | (xs ? 0 : RF_ZEROX), c->d_P32,
                                               rr1, c->d_err, ws);
    bump();
    CKL(c);
    return DG_OK;
  }
  const unsigned g = (unsigned)std::min<int64_t>(c->B, (int64_t)c->nsm * kTsCTA);
  if (g)
    bres_tcs_kernel<<<g, kTcT, kTsDyn, st>>>(S.tc, c->d_nbe, xs, b, nullptr, xo, c->B, flags | (xs ? 0 : RF_ZEROX),
                                             c->d_P32, rr1, c->d_err, ws);
  bump();
  CKL(c);
  return DG_OK;
}

// One batched smoothing / residual step with the preconditioner's BF16
// copies, by kernel variant: 0 CUDA cores (one CTA per element), 1 / 2
// mma.sync with 4 / 8 warps per element, 3 mma.sync persistent bulk-copy,
// 4 tcgen05 persistent bulk-copy (accumulators in tensor memory), 5 tcgen05
// on split x (the iterate already in the operand layout; FP32 x is split
// first here, bprecond keeps its iterates split), 6 the same warp-specialized
int bsmooth(dg_ctx* c, Mixed& M, BatchState& S, int variant, const float* xx, const float* b, float* xo, int flags,
            float* rr1, const float* ws, cudaStream_t st) {
  switch (variant) {
    case 0:
      return bres<__nv_bfloat16>(c, M.blk16, M.W16, xx, b, nullptr, xo, flags, rr1, st, ws);
    case 1:
    case 2:
      if (c->B > 0) {
        if (variant == 2)
          bres_mma_kernel<8><<<(unsigned)c->B, 256, 0, st>>>(M.blk16, M.W16, c->d_nbe, xx, b, nullptr, xo, c->B,
                                                             flags, c->d_P32, rr1, ws, nullptr);
        else
          bres_mma_kernel<4><<<(unsigned)c->B, 128, 0, st>>>(M.blk16, M.W16, c->d_nbe, xx, b, nullptr, xo, c->B,
                                                             flags, c->d_P32, rr1, ws, nullptr);
      }
      bump();
      CKL(c);
      return DG_OK;
    case 3: {
      const unsigned g = (unsigned)std::min<int64_t>(c->B, (int64_t)c->nsm * kBS);
      if (g)
        bres_mma_tma_kernel<<<g, kBT, kBDyn, st>>>(M.blk16, M.W16, c->d_nbe, xx, b, nullptr, xo, c->B, flags, c->d_P32,
                                                   rr1, c->d_err, ws);
      bump();
      CKL(c);
      return DG_OK;
    }
    case 4: {
      int rc;
      if ((rc = ensure_tc_layout(c, M, S, st))) return rc;
      const unsigned g = (unsigned)std::min<int64_t>(c->B, (int64_t)c->nsm * kTcCTA);
      if (g)
        bres_tc05_kernel<<<g, kTcT, kTcDyn, st>>>(S.tc, c->d_nbe, xx, b, nullptr, xo, c->B, flags, c->d_P32, rr1,
                                                  c->d_err, ws);
      bump();
      CKL(c);
      return DG_OK;
    }
    default: {
      // split-x form on FP32 vectors: x converted to the split layout first
      // (the preconditioner itself keeps its iterates split, bprecond)
      int rc;
      if ((rc = ensure_tc_layout(c, M, S, st)) || (rc = ensure_split(c, S))) return rc;
      if (xx) {
        const int64_t items = c->B * 20 * (kNR / 4);
        to_split_kernel<<<nblk(items, 256), 256, 0, st>>>(xx, S.xs1, c->B);
        bump();
      }
      return btcs(c, S, xx ? S.xs1 : nullptr, b, xo, flags & ~RF_OUT_SPLIT, rr1, ws, st);
    }
  }
}

// The batched preconditioner's smoothing steps on the scaled face blocks
// (bsc_mma_kernel) need the single-RHS scaled copy and the mma.sync forms
// for the zero-start step (which forms C) and the restriction.
bool batched_scaled(dg_ctx* c, const Mixed& M) {
  return M.sc && c->precond_bf16 && c->batched_kernel >= 1 && c->batched_kernel <= 4;
}

// zero-start step X_out = s W B that also keeps C = W B
int bzero_start_scaled(dg_ctx* c, Mixed& M, BatchState& S, const float* b, float* xo, const float* ws,
                       cudaStream_t st) {
  int rc;
  if (!S.chat && (rc = dalloc(c, &S.chat, (size_t)c->nonods * kNR))) return rc;
  if (c->B > 0)
    bres_mma_kernel<4><<<(unsigned)c->B, 128, 0, st>>>(M.blk16, M.W16, c->d_nbe, nullptr, b, nullptr, xo, c->B,
                                                       RF_ZEROX | RF_SMOOTH, c->d_P32, nullptr, ws, S.chat);
  bump();
  CKL(c);
  return DG_OK;
}

int bsmooth_scaled(dg_ctx* c, Mixed& M, const float* xx, const float* cv, float* xo, const float* ws,
                   cudaStream_t st) {
  if (c->B > 0)
    bsc_mma_kernel<4><<<(unsigned)c->B, 128, 0, st>>>(M.scblk16, c->d_nbe, xx, cv, xo, c->B, (float)c->mixed_smooth_w,
                                                      ws);
  bump();
  CKL(c);
  return DG_OK;
}

// Smoothing-kernel autotuner of the batched solve: times every variant of
// the full smoothing step (x and b given) on zeroed scratch vectors with
// CUDA events (one warm launch, then 3 timed) once per mixed build, before
// any graph capture, and keeps the fastest; DG_BATCHED_KERNEL pins one.
int autotune_batched(dg_ctx* c, Mixed& M, BatchState& S, cudaStream_t st) {
  if (c->batched_pinned || S.tune_version == c->mixed_version) return DG_OK;
  const size_t nv = (size_t)c->nonods * kNR;
  CK(c, cudaMemsetAsync(S.t1, 0, sizeof(float) * nv, st));
  CK(c, cudaMemsetAsync(S.t2, 0, sizeof(float) * nv, st));
  cudaEvent_t e0, e1;
  CK(c, cudaEventCreate(&e0));
  CK(c, cudaEventCreate(&e1));
  float best = 1e30f;
  int bestv = c->batched_kernel;
  if (!c->precond_bf16) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return DG_OK;
  }
  int rc0;
  if ((rc0 = ensure_tc_layout(c, M, S, st)) || (rc0 = ensure_split(c, S))) return rc0;
  CK(c, cudaMemsetAsync(S.xs1, 0, (size_t)c->B * kSplit, st));
  const int keep = c->batched_kernel;
  auto one = [&](int v) -> int {
    if (v >= 5) {   // split-iterate forms: btcs follows c->batched_kernel
      c->batched_kernel = v;
      const int rc2 = btcs(c, S, S.xs1, S.t2, S.xs2, RF_SMOOTH | RF_OUT_SPLIT, nullptr, nullptr, st);
      c->batched_kernel = keep;
      return rc2;
    }
    return bsmooth(c, M, S, v, S.t1, S.t2, S.t6, RF_SMOOTH, nullptr, nullptr, st);
  };
  for (int v = 0; v < kBatchedVariants; ++v) {
    int rc = one(v);
    if (!rc) CK(c, cudaEventRecord(e0, st));
    for (int it = 0; it < 3 && !rc; ++it) rc = one(v);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    CK(c, cudaEventRecord(e1, st));
    CK(c, cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(c, cudaEventElapsedTime(&ms, e0, e1));
    S.tune_us[v] = ms * 1e3f / 3.0f;
    if (ms < best) {
      best = ms;
      bestv = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->batched_kernel = bestv;
  S.tune_version = c->mixed_version;
  if (c->verbose)
    std::fprintf(stderr, "[autotune] batched smoothing kernel %d (%.1f us per launch)\n", bestv, best * 1e3f / 3.0f);
  return DG_OK;
}

// Smoothing steps per leg of the batched preconditioner: DG_BATCHED_SWEEPS,
// else DG_MIXED_SWEEPS, else kBatchedChebSteps with the damped block
// inverse; with DG_MIXED_OMEGAS or without a lambda_max estimate the
// single-RHS schedule
bool batched_own_schedule(const dg_ctx* c) {
  return c->batched_sweeps >= 0 || (c->mixed_sweeps < 0 && c->mixed_smoother == 1 && !c->omegas_set &&
                                    c->smoother_lmax > 0.0);
}

int batched_steps(const dg_ctx* c) {
  if (!batched_own_schedule(c)) return mixed_steps(c);
  return c->batched_sweeps >= 0 ? c->batched_sweeps : kBatchedChebSteps;
}

// the batched factors on the device, once per mixed build
int ensure_batched_schedule(dg_ctx* c, Mixed& M, BatchState& S, cudaStream_t st) {
  if (S.d_wsb && S.wsb_version == c->mixed_version) return DG_OK;
  int rc;
  if (!S.d_wsb && (rc = dalloc(c, &S.d_wsb, kMaxSmoothSteps))) return rc;
  float f[kMaxSmoothSteps];
  for (int k = 0; k < kMaxSmoothSteps; ++k) f[k] = c->mixed_wscale[k];
  const int nsm = batched_steps(c);
  if (batched_own_schedule(c) && nsm >= 2 && c->smoother_lmax > 0.0)
    cheb_factors(c, c->smoother_lmax, std::min(kMaxSmoothSteps, nsm), c->cheb_ratio_b, f);
  CK(c, cudaMemcpyAsync(S.d_wsb, f, sizeof(f), cudaMemcpyHostToDevice, st));
  CK(c, cudaStreamSynchronize(st));
  S.wsb_version = c->mixed_version;
  (void)M;
  return DG_OK;
}

// batched preconditioner (same schedule as precond32, dense coarse level)
int bprecond(dg_ctx* c, const float* r, float* z, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  BatchState& S = batch_of(M);
  int rc;
  const int nsm = batched_steps(c);
  const float w = (float)c->cfg.jac_wei;
  float* cur = S.t3;
  float* other = S.t4;
  const bool bf = c->precond_bf16;
  // DG-level smoothing step k damped like the single-RHS preconditioner
  auto wsk = [&](int k) -> const float* {
    return ((nsm >= 2 && nsm <= kMaxSmoothSteps) || c->omegas_set) && k < kMaxSmoothSteps ? S.d_wsb + k : nullptr;
  };
  auto pc = [&](const float* xx, float* xo, int flags, float* rr1, const float* ws) -> int {
    if (bf) return bsmooth(c, M, S, c->batched_kernel, xx, r, xo, flags, rr1, ws, st);
    return bres<float>(c, M.blk, M.W, xx, r, nullptr, xo, flags, rr1, st, ws);
  };
  // split-x pipeline: the iterate stays in the tensor-core operand layout
  // from the first smoothing step to the last, which writes z in FP32
  const bool split = bf && c->batched_kernel >= 5;
  // scaled face blocks for the smoothing steps after the zero-start one
  const bool sc = !split && batched_scaled(c, M);
  unsigned char* scur = nullptr;
  unsigned char* soth = nullptr;
  if (split) {
    if ((rc = ensure_tc_layout(c, M, S, st)) || (rc = ensure_split(c, S))) return rc;
    scur = S.xs1;   // allocated by ensure_split just above
    soth = S.xs2;
    if ((rc = btcs(c, S, nullptr, r, scur, RF_ZEROX | RF_SMOOTH | RF_OUT_SPLIT, nullptr, wsk(0), st))) return rc;
    for (int it = 1; it < nsm; ++it) {
      if ((rc = btcs(c, S, scur, r, soth, RF_SMOOTH | RF_OUT_SPLIT, nullptr, wsk(it), st))) return rc;
      std::swap(scur, soth);
    }
    if ((rc = btcs(c, S, scur, r, nullptr, RF_RESTRICT, S.r1, nullptr, st))) return rc;
  } else if (sc) {
    if ((rc = bzero_start_scaled(c, M, S, r, cur, wsk(0), st))) return rc;
    for (int it = 1; it < nsm; ++it) {
      if ((rc = bsmooth_scaled(c, M, cur, S.chat, other, wsk(it), st))) return rc;
      std::swap(cur, other);
    }
    if ((rc = pc(cur, nullptr, RF_RESTRICT, S.r1, nullptr))) return rc;
  } else {
    if ((rc = pc(nullptr, cur, RF_ZEROX | RF_SMOOTH, nullptr, wsk(0)))) return rc;
    for (int it = 1; it < nsm; ++it) {
      if ((rc = pc(cur, other, RF_SMOOTH, nullptr, wsk(it)))) return rc;
      std::swap(cur, other);
    }
    if ((rc = pc(cur, nullptr, RF_RESTRICT, S.r1, nullptr))) return rc;
  }
  bgather_kernel<<<(unsigned)c->ncg, kNR, 0, st>>>(S.r1, c->d_gptr, c->d_gent, c->d_wdg32, c->d_pos, S.lr[0],
                                                   (int)c->ncg);
  bump();
  const int lc = M.dense_l;
  for (int l = 0; l < lc; ++l) {
    const int n = M.lev[l].n;
    const unsigned g = nblk((int64_t)n, 4);
    for (int it = 0; it <= c->cfg.pre_smooth_its; ++it) {
      const bool last = it == c->cfg.pre_smooth_its;
      const float* ein = (l == 0 && it == 0) ? nullptr : S.le[l];
      bjacobi_kernel<<<g, 4 * kNR, 0, st>>>(M.lev[l].rowptr, M.lev[l].col, M.lev[l].val, M.lev[l].diag, ein, S.lr[l],
                                            S.le2[l], last ? S.lrr[l] : nullptr, n, w);
      bump();
      std::swap(S.le[l], S.le2[l]);
    }
    const int nn = M.lev[l + 1].n;
    brestrict_kernel<<<nblk((int64_t)nn * kNR, 256), 256, 0, st>>>(S.lrr[l], S.le[l], S.lr[l + 1], S.le[l + 1], n, nn);
    bump();
  }
  bdense2_kernel<<<nblk(M.lev[lc].n, kDnRows), 128, kDnSmem, st>>>(M.dense_inv, S.lr[lc], S.le[lc], M.lev[lc].n);
  bump();
  for (int l = lc - 1; l >= 0; --l) {
    const int n = M.lev[l].n;
    bprolong_lev_kernel<<<nblk((int64_t)n * kNR, 256), 256, 0, st>>>(S.le[l], S.le[l + 1], M.lev[l].up, n);
    bump();
    for (int it = 0; it < c->cfg.post_smooth_its; ++it) {
      bjacobi_kernel<<<nblk((int64_t)n, 4), 4 * kNR, 0, st>>>(M.lev[l].rowptr, M.lev[l].col, M.lev[l].val,
                                                              M.lev[l].diag, S.le[l], S.lr[l], S.le2[l], nullptr, n, w);
      bump();
      std::swap(S.le[l], S.le2[l]);
    }
  }
  if (split) {
    bprolong_split_kernel<<<(unsigned)c->B, 20 * (kNR / 4), 0, st>>>(scur, S.le[0], c->d_pos, c->d_p1cg, c->d_wdg32,
                                                                   c->d_P32, c->B);
    bump();
    for (int it = 0; it < nsm; ++it) {
      const bool last_step = it == nsm - 1;
      if ((rc = btcs(c, S, scur, r, last_step ? (void*)z : (void*)soth, RF_SMOOTH | (last_step ? 0 : RF_OUT_SPLIT),
                     nullptr, wsk(nsm - 1 - it), st)))
        return rc;
      std::swap(scur, soth);
    }
    CKL(c);
    return DG_OK;
  }
  bprolong_kernel<<<(unsigned)c->B, 20 * (kNR / 4), 0, st>>>(cur, S.le[0], c->d_pos, c->d_p1cg, c->d_wdg32, c->d_P32,
                                                             c->B);
  bump();
  for (int it = 0; it < nsm; ++it) {
    float* out = (it == nsm - 1) ? z : other;
    if ((rc = sc ? bsmooth_scaled(c, M, cur, S.chat, out, wsk(nsm - 1 - it), st)
                 : pc(cur, out, RF_SMOOTH, nullptr, wsk(nsm - 1 - it))))
      return rc;
    other = cur;
    cur = out;
  }
  CKL(c);
  return DG_OK;
}

// Gram-Schmidt of w against V[0..j] for every RHS; writes H_q column j and V[j+1]
int bcgs(dg_ctx* c, int j, float* w, int m, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  BatchState& S = batch_of(M);
  const int nv = j + 1;
  const int64_t ld = c->nonods * kNR;
  if (c->batched_gs2) {
    // low-register forms, 4 blocks per SM
    const int g = 4 * c->nsm;
    bmdot2_kernel<<<dim3(g, (nv + 7) / 8), 256, 0, st>>>(S.V, ld, nv, w, c->nonods, S.part);
    breduce2_kernel<<<dim3(nv, kNR / 16), 1024, 0, st>>>(S.part, g, S.h);
    baxpy2_kernel<<<g, 256, 0, st>>>(S.V, ld, nv, S.h, w, c->nonods, S.part);
    bfinish2_kernel<<<1, 1024, 0, st>>>(S.part, g, S.h, nv, j, m, S.H, S.inv);
  } else {
    bmdot_kernel<<<dim3(S.nblk, (nv + 7) / 8), 256, 0, st>>>(S.V, ld, nv, w, c->nonods, S.part);
    breduce_kernel<<<nblk((int64_t)nv * kNR, 256), 256, 0, st>>>(S.part, S.nblk, nv, S.h);
    baxpy_kernel<<<S.nblk, 256, 0, st>>>(S.V, ld, nv, S.h, w, c->nonods, S.part);
    bfinish_kernel<<<1, kNR, 0, st>>>(S.part, S.nblk, S.h, nv, j, m, S.H, S.inv);
  }
  bscale_kernel<<<nblk(ld / 4, 256), 256, 0, st>>>(w, S.inv, S.V + (size_t)nv * ld, ld);
  bump(5);
  CKL(c);
  return DG_OK;
}

// Inner Arnoldi step j of the batched flexible GMRES: z_j = P(v_j),
// w = -A z_j, Gram-Schmidt of w against v_0..v_j into H column j and v_j+1.
int bstep(dg_ctx* c, int j, int m, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  BatchState& S = batch_of(M);
  const int64_t ld = c->nonods * kNR;
  float* zj = S.Z + (size_t)j * ld;
  int rc;
  if ((rc = bprecond(c, S.V + (size_t)j * ld, zj, st))) return rc;
  if ((rc = bres<float>(c, M.blk, M.W, zj, nullptr, S.t1, nullptr, RF_NEG, nullptr, st))) return rc;
  return bcgs(c, j, S.t1, m, st);
}

// Runs step j as one CUDA graph launch.  The graph of each j is captured at
// its first use and replayed in every later restart cycle and solve; its
// kernel arguments are fixed device pointers (basis column j, scratch,
// operator copies), so it is kept while the state in `key` below holds and
// captured again after any change (restart length, reallocated basis,
// kernel variant, operator rebuild, preconditioner options).  Buffers that
// the step would allocate or lay out on first use are set up before the
// capture, so the graph holds kernels only.
int run_bstep(dg_ctx* c, int j, int m, cudaStream_t st) {
  if (!c->use_graph) return bstep(c, j, m, st);
  Mixed& M = mixed_of(c);
  BatchState& S = batch_of(M);
  auto tag = [](int64_t v) { return reinterpret_cast<const void*>(static_cast<intptr_t>(v)); };
  const std::vector<const void*> key = {
      tag(m),
      tag(c->batched_kernel),
      tag(c->mixed_version),
      tag(c->precond_bf16),
      tag(c->batched_gs2),
      tag(c->cfg.pre_smooth_its),
      tag(c->cfg.post_smooth_its),
      tag(c->omegas_set),
      tag(batched_steps(c)),
      S.d_wsb,
      tag(M.dense_l),
      S.V,
      S.Z,
      M.blk,
      M.blk16,
      M.dense_inv,
      tag(batched_scaled(c, M)),
      M.scblk16,
  };
  if (key != S.step_key) {
    for (auto& g : S.step_graph)
      if (g) cudaGraphExecDestroy(g);
    S.step_graph.assign(m, nullptr);
    S.step_kern.assign(m, 0);
    S.step_key = key;
  }
  if (!S.step_graph[j]) {
    int rc;
    if (c->precond_bf16 && c->batched_kernel >= 4 && (rc = ensure_tc_layout(c, M, S, st))) return rc;
    if (c->precond_bf16 && c->batched_kernel >= 5 && (rc = ensure_split(c, S))) return rc;
    if (batched_scaled(c, M) && !S.chat && (rc = dalloc(c, &S.chat, (size_t)c->nonods * kNR))) return rc;
    if (!c->cap_stream) CK(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    CK(c, cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    const long long k0 = g_launches.load();
    rc = bstep(c, j, m, c->cap_stream);
    const int nk = (int)(g_launches.load() - k0);
    g_launches.fetch_sub(nk);   // captured, not launched
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(c->cap_stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ee != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("batched step capture: ") + cudaGetErrorString(ee));
    const cudaError_t ie = cudaGraphInstantiate(&S.step_graph[j], g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      S.step_graph[j] = nullptr;
      return fail(c, DG_ERR_CUDA, std::string("batched step instantiate: ") + cudaGetErrorString(ie));
    }
    S.step_kern[j] = nk;
  }
  CK(c, cudaGraphLaunch(S.step_graph[j], st));
  bump(S.step_kern[j]);
  return DG_OK;
}

}  // namespace

// Batched mixed-precision solve of nrhs <= 64 systems A x_q = b_q on one
// operator (P3 tetrahedra): x and b are (nrhs, nonods) FP64, RHS-major;
// each x_q starts from its content and stops at ||b_q - A x_q|| <= tol[q]
// (FP64 true residual).  its / res (per RHS, may be NULL) receive the inner
// iterations run while q was active and the final residual norm.
extern "C" int dg_solve_mixed_batched(dg_ctx* c, double* x, const double* b, int32_t nrhs, const double* tol,
                                      int32_t m, int32_t max_its, double inner_rtol, int32_t* its_out,
                                      double* res_out, void* stream) {
  if (!c || !x || !b || !tol) return set_thread_error(DG_ERR_ARG, "dg_solve_mixed_batched: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_solve_mixed_batched: operator not built");
  if (c->D != 3) return fail(c, DG_ERR_ARG, "dg_solve_mixed_batched: P3 tetrahedra only");
  if (nrhs < 1 || nrhs > kNR || m < 1 || m > 31 || max_its < 0 || !(inner_rtol > 0.0 && inner_rtol < 1.0))
    return fail(c, DG_ERR_ARG, "dg_solve_mixed_batched: need 1 <= nrhs <= 64, 1 <= m <= 31, 0 < inner_rtol < 1");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  if (!M.has5 && (rc = build_blk5(c, st))) return rc;   // the batched kernels read five blocks per element
  if (M.dense_l < 0) return fail(c, DG_ERR_STATE, "dg_solve_mixed_batched: needs the dense coarse level");
  if (!c->f32_tma) return fail(c, DG_ERR_STATE, "dg_solve_mixed_batched: needs the chunked FP32 block layout");
  if ((rc = ensure_batch(c, m))) return rc;
  CK(c, cudaFuncSetAttribute(bres_mma_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBDyn));
  CK(c, cudaFuncSetAttribute(bres_tc05_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcDyn));
  CK(c, cudaFuncSetAttribute(bres_tcs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTsDyn));
  CK(c, cudaFuncSetAttribute(bres_tcw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTwDyn));
  CK(c, cudaFuncSetAttribute(bdense2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDnSmem));
  if ((rc = autotune_batched(c, M, batch_of(M), st))) return rc;
  if ((rc = ensure_batched_schedule(c, M, batch_of(M), st))) return rc;
  CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));   // bulk-copy wait time-outs land here
  BatchState& S = batch_of(M);
  const int64_t n = c->nonods;
  const int64_t ld = n * kNR;
  const dim3 tgrid((unsigned)((n + 31) / 32), kNR / 32), tblock(32, 8);
  std::vector<double> rn(kNR, 0.0), tolv(kNR, 0.0), target(kNR, 0.0), beta0(kNR, 0.0), a(kNR, 0.0);
  std::vector<int32_t> its(kNR, 0);
  std::vector<char> active(kNR, 0);
  for (int q = 0; q < nrhs; ++q) tolv[q] = tol[q];
  std::vector<double> Hh((size_t)kNR * (m + 1) * m), ybuf((size_t)32 * kNR), nrm(kNR), rnew(kNR);
  // FP64 residuals r_q = b_q - A x_q (one FP64 apply per RHS, bound by the
  // FP64 pipe) for the RHS in `redo`; the others keep r_q and |r_q|: a zero
  // start gives r_q = b_q exactly, and an RHS that no refinement step
  // updated keeps its x_q
  std::vector<char> redo(kNR, 0);
  auto outer_residuals = [&]() -> int {
    int r2;
    for (int q = 0; q < nrhs; ++q) {
      if (!redo[q]) continue;
      if (redo[q] == 2) {
        CK(c, cudaMemcpyAsync(S.r64 + (size_t)q * n, b + (size_t)q * n, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                              st));
      } else if ((r2 = residual(c, x + (size_t)q * n, b + (size_t)q * n, S.r64 + (size_t)q * n, nullptr, 0, st))) {
        return r2;
      }
      if ((r2 = norm2(c, S.r64 + (size_t)q * n, c->d_scal + q, st))) return r2;
    }
    CK(c, cudaMemcpyAsync(rnew.data(), c->d_scal, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    for (int q = 0; q < nrhs; ++q)
      if (redo[q]) rn[q] = rnew[q];
    return DG_OK;
  };
  {
    // which starting x_q are zero (2: r_q = b_q) or not (1: FP64 residual)
    int* flag = reinterpret_cast<int*>(S.h);   // scratch until the first inner step
    CK(c, cudaMemsetAsync(flag, 0, sizeof(int) * kNR, st));
    bnonzero_kernel<<<dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(2 * c->nsm, (n + 255) / 256)), nrhs), 256,
                      0, st>>>(x, n, flag);
    bump();
    CKL(c);
    std::vector<int> nz(kNR, 0);
    CK(c, cudaMemcpyAsync(nz.data(), flag, sizeof(int) * nrhs, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    for (int q = 0; q < nrhs; ++q) redo[q] = nz[q] ? 1 : 2;
  }
  if ((rc = outer_residuals())) return rc;
  int total = 0, status = DG_OK;
  while (total < max_its) {
    int nact = 0;
    for (int q = 0; q < kNR; ++q) {
      active[q] = q < nrhs && std::isfinite(rn[q]) && rn[q] > tolv[q];
      nact += active[q];
      a[q] = active[q] ? 1.0 / rn[q] : 0.0;
    }
    for (int q = 0; q < nrhs; ++q)
      if (!std::isfinite(rn[q])) status = DG_ERR_NUMERIC;
    if (nact == 0 || status) break;
    // rhs32 = r64 / |r| (inactive columns zero), d32 = 0
    CK(c, cudaMemcpyAsync(S.scl, a.data(), sizeof(double) * kNR, cudaMemcpyHostToDevice, st));
    binterleave_kernel<<<tgrid, tblock, 0, st>>>(S.r64, n, nrhs, S.scl, S.t2);
    bump();
    CK(c, cudaMemsetAsync(S.t6, 0, sizeof(float) * ld, st));
    for (int q = 0; q < kNR; ++q) target[q] = active[q] ? std::max(inner_rtol, 0.5 * tolv[q] / rn[q]) : 0.0;
    std::fill(beta0.begin(), beta0.end(), -1.0);
    bool inner_done = false, first_cycle = true;
    while (!inner_done && total < max_its) {
      // V0 = rhs - A d (d = 0 on the first cycle); beta_q = |V0_q|
      if (first_cycle) {
        CK(c, cudaMemcpyAsync(S.V, S.t2, sizeof(float) * ld, cudaMemcpyDeviceToDevice, st));
      } else if ((rc = bres<float>(c, M.blk, M.W, S.t6, S.t2, S.V, nullptr, 0, nullptr, st))) {
        return rc;
      }
      bnorm_kernel<<<S.nblk, 256, 0, st>>>(S.V, n, S.part);
      bnorm_finish_kernel<<<1, kNR, 0, st>>>(S.part, S.nblk, S.nrm, S.inv);
      bscale_kernel<<<nblk(ld / 4, 256), 256, 0, st>>>(S.V, S.inv, S.V, ld);
      bump(3);
      CK(c, cudaMemcpyAsync(nrm.data(), S.nrm, sizeof(double) * kNR, cudaMemcpyDeviceToHost, st));
      CK(c, cudaMemsetAsync(S.H, 0, sizeof(double) * kNR * (m + 1) * m, st));
      CK(c, cudaStreamSynchronize(st));
      bool any = false;
      for (int q = 0; q < kNR; ++q) {
        if (!active[q]) continue;
        if (beta0[q] < 0.0) beta0[q] = nrm[q];
        if (nrm[q] > target[q] * beta0[q]) any = true;
      }
      first_cycle = false;
      if (!any) break;
      int k = 0;
      // host checks of the least-squares residuals: every 5 steps, and
      // (adaptive) at the step where the slowest active RHS is predicted to
      // reach its target from its observed convergence rate
      int next_check = std::min(5, m);
      for (int j = 0; j < m && total < max_its; ++j) {
        if ((rc = run_bstep(c, j, m, st))) return rc;
        ++total;
        k = j + 1;
        for (int q = 0; q < kNR; ++q)
          if (active[q]) ++its[q];
        if (k >= next_check || k == m) {
          CK(c, cudaMemcpyAsync(Hh.data(), S.H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
          CK(c, cudaStreamSynchronize(st));
          bool all = true;
          int need_max = 0;
          for (int q = 0; q < kNR; ++q) {
            if (!active[q] || nrm[q] <= target[q] * beta0[q]) continue;
            std::vector<double> Hq(Hh.begin() + (size_t)q * (m + 1) * m, Hh.begin() + (size_t)(q + 1) * (m + 1) * m);
            std::vector<double> yq;
            bool ok = true;
            const double est = hessenberg_ls(Hq, m, k, nrm[q], yq, ok);
            if (!ok || !(est <= target[q] * beta0[q])) {
              all = false;
              int need = 5;
              const double rate = std::pow(est / nrm[q], 1.0 / k);
              if (ok && rate > 0.0 && rate < 1.0)
                need = (int)std::ceil(std::log(target[q] * beta0[q] / est) / std::log(rate));
              need_max = std::max(need_max, std::max(need, 1));
            }
          }
          if (all) break;
          next_check = c->adaptive_chunk ? k + std::min(need_max, 5) : k + 5;
        }
      }
      // per-RHS least squares over the k steps, d += Z y
      CK(c, cudaMemcpyAsync(Hh.data(), S.H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      std::fill(ybuf.begin(), ybuf.end(), 0.0);
      bool alld = true;
      for (int q = 0; q < kNR; ++q) {
        if (!active[q] || nrm[q] <= target[q] * beta0[q]) continue;
        std::vector<double> Hq(Hh.begin() + (size_t)q * (m + 1) * m, Hh.begin() + (size_t)(q + 1) * (m + 1) * m);
        std::vector<double> yq;
        bool ok = true;
        const double est = hessenberg_ls(Hq, m, k, nrm[q], yq, ok);
        if (!ok) {
          active[q] = 0;   // breakdown of this RHS: keep its current iterate
          continue;
        }
        for (int i = 0; i < k; ++i) ybuf[(size_t)i * kNR + q] = yq[i];
        if (!(est <= target[q] * beta0[q])) alld = false;
      }
      CK(c, cudaMemcpyAsync(S.y, ybuf.data(), sizeof(double) * 32 * kNR, cudaMemcpyHostToDevice, st));
      bcombine_kernel<<<nblk(ld, 256), 256, 0, st>>>(S.Z, ld, k, S.y, S.t6, ld);
      bump();
      CKL(c);
      inner_done = alld;
    }
    // x_q += |r_q| d_q for the active RHS
    for (int q = 0; q < kNR; ++q) a[q] = active[q] ? rn[q] : 0.0;
    CK(c, cudaMemcpyAsync(S.scl, a.data(), sizeof(double) * kNR, cudaMemcpyHostToDevice, st));
    bupdate_kernel<<<tgrid, tblock, 0, st>>>(x, n, nrhs, S.scl, S.t6);
    bump();
    CKL(c);
    for (int q = 0; q < nrhs; ++q) redo[q] = active[q] ? 1 : 0;
    if ((rc = outer_residuals())) return rc;
  }
  {
    int herr = 0;
    CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (herr == 3) {
      c->err = "batched solve: a bulk-copy wait of the preconditioner timed out";
      return DG_ERR_CUDA;
    }
  }
  bool all_conv = true;
  for (int q = 0; q < nrhs; ++q) {
    if (its_out) its_out[q] = its[q];
    if (res_out) res_out[q] = rn[q];
    if (!(rn[q] <= tolv[q])) all_conv = false;
  }
  if (status) {
    c->err = "batched solve: non-finite residual";
    return status;
  }
  if (!all_conv) {
    c->err = "batched solve reached the iteration limit";
    return DG_ERR_NOCONV;
  }
  return DG_OK;
}

// ---------------------------------------------------------------------------
// Multi-RHS operator stages on RHS-interleaved FP32 vectors (kNR = 64 right-
// hand sides, x[(e * 20 + n) * 64 + q]), P3 tetrahedra.

namespace {

int batched_prep(dg_ctx* c, const char* name, cudaStream_t st) {
  if (!c->built) return fail(c, DG_ERR_STATE, std::string(name) + ": operator not built");
  if (c->D != 3) return fail(c, DG_ERR_ARG, std::string(name) + ": P3 tetrahedra only");
  CK(c, cudaSetDevice(c->dev));
  Mixed& M = mixed_of(c);
  int rc;
  if (!M.built || c->mixed_version != c->build_version) {
    if ((rc = build_mixed(c, st))) return rc;
    c->mixed_version = c->build_version;
  }
  if (!M.has5 && (rc = build_blk5(c, st))) return rc;
  if ((rc = ensure_batch(c, 1))) return rc;
  CK(c, cudaFuncSetAttribute(bres_mma_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBDyn));
  CK(c, cudaFuncSetAttribute(bres_tc05_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcDyn));
  CK(c, cudaFuncSetAttribute(bres_tcs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTsDyn));
  CK(c, cudaFuncSetAttribute(bres_tcw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTwDyn));
  CK(c, cudaFuncSetAttribute(bdense2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDnSmem));
  return DG_OK;
}

}  // namespace

// Y = A X for 64 right-hand sides with the FP32 operator copy (CUDA cores).
extern "C" int dg_apply_batched(dg_ctx* c, const float* x, float* y, void* stream) {
  if (!c || !x || !y) return set_thread_error(DG_ERR_ARG, "dg_apply_batched: null argument");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int rc;
  if ((rc = batched_prep(c, "dg_apply_batched", st))) return rc;
  Mixed& M = mixed_of(c);
  return bres<float>(c, M.blk, M.W, x, nullptr, y, nullptr, RF_NEG, nullptr, st);
}

// One smoothing step of the batched preconditioner with its BF16 copies:
// X_out = X + W (B - A X) for 64 right-hand sides (X NULL = zero guess),
// through the batched kernel variant in use (dg_set_batched_kernel).
extern "C" int dg_smooth_pc_batched(dg_ctx* c, const float* x, const float* b, float* x_out, void* stream) {
  if (!c || !b || !x_out) return set_thread_error(DG_ERR_ARG, "dg_smooth_pc_batched: null argument");
  if (x_out == x) return fail(c, DG_ERR_ARG, "dg_smooth_pc_batched: x_out must not alias x");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int rc;
  if ((rc = batched_prep(c, "dg_smooth_pc_batched", st))) return rc;
  if (!c->precond_bf16) return fail(c, DG_ERR_STATE, "dg_smooth_pc_batched: needs the BF16 preconditioner copies");
  Mixed& M = mixed_of(c);
  CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
  return bsmooth(c, M, batch_of(M), c->batched_kernel, x, b, x_out, x ? RF_SMOOTH : (RF_SMOOTH | RF_ZEROX), nullptr,
                 nullptr, st);
}

// X_out = X + (C - w X - sum_f S_ef X_nb(f)) for 64 right-hand sides on the
// scaled face blocks (the batched preconditioner's steps after its zero-start
// one, bsc_mma_kernel); DG_ERR_STATE when the scaled form is not in use.
extern "C" int dg_smooth_scaled_batched(dg_ctx* c, const float* x, const float* cv, float* x_out, void* stream) {
  if (!c || !x || !cv || !x_out) return set_thread_error(DG_ERR_ARG, "dg_smooth_scaled_batched: null argument");
  if (x_out == x) return fail(c, DG_ERR_ARG, "dg_smooth_scaled_batched: x_out must not alias x");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int rc;
  if ((rc = batched_prep(c, "dg_smooth_scaled_batched", st))) return rc;
  Mixed& M = mixed_of(c);
  if (!M.sc || !c->precond_bf16)
    return fail(c, DG_ERR_STATE, "dg_smooth_scaled_batched: the scaled face blocks are not in use");
  return bsmooth_scaled(c, M, x, cv, x_out, nullptr, st);
}

// Batched smoothing kernel variant: -1 = timed choice at the next batched
// solve (default), 0 CUDA cores, 1 / 2 mma.sync per element (4 / 8 warps),
// 3 mma.sync persistent bulk-copy, 4 tcgen05 persistent bulk-copy.
// tune_us (may be NULL) receives the last timing per variant (us, -1 = not
// timed) and *chosen the variant in use.
extern "C" int dg_set_batched_kernel(dg_ctx* c, int32_t variant) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_batched_kernel: null context");
  if (variant < -1 || variant >= kBatchedVariants)
    return fail(c, DG_ERR_ARG, "dg_set_batched_kernel: variant must be -1 .. 6");
  if (variant < 0) {
    c->batched_pinned = false;
    batch_of(mixed_of(c)).tune_version = -1;
  } else {
    c->batched_kernel = variant;
    c->batched_pinned = true;
  }
  Mixed& M = mixed_of(c);
  for (auto& g : M.graphs)
    if (g) cudaGraphExecDestroy(g);
  M.graphs.clear();
  M.g_m = 0;
  return DG_OK;
}

extern "C" int dg_batched_tuning(const dg_ctx* c, float* tune_us, int32_t n, int32_t* chosen) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_batched_tuning: null context");
  const Mixed& M = mixed_of(const_cast<dg_ctx*>(c));
  const BatchState* S = static_cast<const BatchState*>(M.batch);
  for (int v = 0; tune_us && v < n && v < kBatchedVariants; ++v) tune_us[v] = S ? S->tune_us[v] : -1.0f;
  if (chosen) *chosen = c->batched_kernel;
  return DG_OK;
}
