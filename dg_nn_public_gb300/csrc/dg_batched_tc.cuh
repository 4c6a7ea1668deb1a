// Batched BF16 smoothing / residual step of the multi-RHS preconditioner on
// the fifth-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory), with the element's operator data streamed by bulk copies.
// Included into dg_solver.cu after dg_batched.cuh (it uses kNR, the flags,
// the bulk-copy / mbarrier helpers and the context).
//
// One element e, kNR = 64 right-hand sides, x RHS-interleaved
// (x[(e*20 + n)*64 + q]).  The product Y(q, m) = sum_k X(q, k) A_stack(m, k)
// runs as D (128 x 24) = Aop (128 x K) * Bop (K x 24):
//   * rows of D / Aop are r = 2q + part: the x value of RHS q split into a
//     BF16 high part (part 0) and the BF16 rounding of the remainder (part
//     1), so x keeps ~16 bits through the product; the two rows are summed
//     in the epilogue (two neighbouring TMEM lanes);
//   * K stacks the element's five blocks (own + four face neighbours), 24
//     slots per block (nodes 20..23 zero) and one zero slot group: K = 128;
//   * N = 24 covers the 20 block rows m (columns 20..23 of D are unused).
// Aop is built in shared memory from the gathered FP32 x slabs ("MN-major":
// eight consecutive rows r, i.e. four RHS x hi/lo, are one 16-byte row of a
// core matrix, so one float4 of x becomes one 16-byte store).  Bop is the
// element's BF16 blocks in a padded chunk layout that is already the
// canonical K-major core-matrix layout, so it goes from global memory to
// shared memory by one bulk copy and straight into the MMA.  The smoothing
// product W res uses the same path with the residual as a K-major operand.
//
// Every CTA runs kTcT = 128 threads; thread r reads TMEM lane r, i.e. row
// r = 2q + part of D, and the pair (2q, 2q+1) owns RHS q in the epilogue.
// Waits on mbarriers are bounded: on a time-out the kernel sets the
// context's error word to 3, waits (bounded) for its own copies in flight,
// frees its tensor memory and returns.
#pragma once

namespace {

// ---- tensor-core (tcgen05) primitives -------------------------------------

// shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (stride between core matrices along K), stride byte offset (along
// M / N), version 1 in bits 46-47
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: BF16 x BF16 -> FP32, M x N, A
// K-major (a_mn = 0) or MN-major (1), B K-major
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int m, int n, int a_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- layout and sizes -----------------------------------------------------

constexpr int kTcT = 128;                        // threads per CTA (one per TMEM lane)
constexpr int kTcStages = 2;                     // bulk-copy ring depth
constexpr int kTcCTA = 3;                        // CTAs per SM
constexpr int kTcChunk = 320;                    // 20 rows x 16 bytes (8 BF16 columns)
constexpr int kTcWBytes = 3 * kTcChunk;          // W: 3 chunks
constexpr int kTcABytes = 15 * kTcChunk;         // 5 blocks x 3 chunks
constexpr int kTcElem = kTcWBytes + kTcABytes;   // 5,760 bytes per element (padded layout)
// stage: [W | A blocks | zero chunk | b slab]; the zero chunk is K slots
// 120..127 of the block product (Aop is zero there as well) and is never
// overwritten by a copy
constexpr int kTcStW = 0, kTcStA = kTcWBytes, kTcStZ = kTcElem, kTcStB = kTcElem + kTcChunk;
constexpr int kTcStage = kTcStB + 20 * kNR * 4;  // 11,200 bytes
constexpr int kTcLBO = 2048;                     // K-direction core-matrix stride of Aop / Rop
constexpr int kTcAop = 16 * kTcLBO;              // 128 rows x 128 K slots (BF16): 32 KiB
constexpr int kTcRop = 4 * kTcLBO;               // 128 rows x 32 K slots: 8 KiB
constexpr int kTcDyn = kTcStages * kTcStage + kTcAop + kTcRop;
constexpr uint32_t kTcCols = 64;                 // TMEM columns: D1 at 0, D2 at 32
constexpr uint32_t kTcIdescA = tc_idesc_bf16(128, 24, 1);   // Aop MN-major
constexpr uint32_t kTcIdescR = tc_idesc_bf16(128, 24, 0);   // Rop K-major

// element tc layout: [W chunks 0..2][block 0 chunks 0..2] ... [block 4 ...];
// chunk c = rows m 0..19 x BF16 columns 8c .. 8c+7 (columns >= 20 zero);
// built from the chunked BF16 copies (same values)
__global__ void tc_layout_kernel(const __nv_bfloat16* __restrict__ blk16, const __nv_bfloat16* __restrict__ W16,
                                 const int* __restrict__ nbe, __nv_bfloat16* __restrict__ tc, int64_t B) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * (kTcElem / 2)) return;
  const int64_t e = i / (kTcElem / 2);
  const int rem = (int)(i - e * (kTcElem / 2));
  const int j = rem / 480, w = rem % 480;        // slot j (0 = W, 1 + b = block b)
  const int ch = w / 160, m = (w % 160) / 8, n = 8 * ch + (w % 8);
  __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
  // boundary faces have no neighbour block: the slot is stored as zeros, so
  // that a stale x slab in its place contributes nothing
  if (n < 20 && (j <= 1 || nbe[e * 4 + j - 2] >= 0)) {
    const __nv_bfloat16* src = j == 0 ? W16 + e * 400 : blk16 + (e * 5 + (j - 1)) * 400;
    v = src[chunk20_index(m, n)];
  }
  tc[i] = v;
}

// two FP32 values -> packed BF16 (lo half = first)
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

// x (4 RHS) -> 16 bytes: hi, lo of RHS 0, then RHS 1, 2, 3 (rows 2q, 2q+1)
__device__ __forceinline__ uint4 split_hilo4(float4 v) {
  const float h0 = __bfloat162float(__float2bfloat16_rn(v.x)), h1 = __bfloat162float(__float2bfloat16_rn(v.y)),
              h2 = __bfloat162float(__float2bfloat16_rn(v.z)), h3 = __bfloat162float(__float2bfloat16_rn(v.w));
  uint4 o;
  o.x = pack_bf16x2(h0, v.x - h0);
  o.y = pack_bf16x2(h1, v.y - h1);
  o.z = pack_bf16x2(h2, v.z - h2);
  o.w = pack_bf16x2(h3, v.w - h3);
  return o;
}

__global__ void __launch_bounds__(kTcT, kTcCTA) bres_tc05_kernel(
    const __nv_bfloat16* __restrict__ tcblk, const int* __restrict__ nbe, const float* __restrict__ x,
    const float* __restrict__ b, float* __restrict__ r, float* __restrict__ x_out, int64_t B, int flags,
    const float* __restrict__ P, float* __restrict__ r1, int* __restrict__ err, const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4;
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* stages = tsm;
  unsigned char* Aop = tsm + kTcStages * kTcStage;
  unsigned char* Rop = Aop + kTcAop;
  __shared__ __align__(8) uint64_t full[kTcStages];
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int nbs[kTcStages][F];
  __shared__ float Ps[N][F];
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  const bool restrict_ = flags & RF_RESTRICT;
  const float ws = wsp ? *wsp : 1.0f;
  const float sgn = (flags & RF_NEG) ? -1.0f : 1.0f;
  const int64_t stride = gridDim.x;
  // everything the MMAs may read starts finite: zero the stages and operands
  for (int i = tid; i < kTcDyn / 16; i += kTcT) reinterpret_cast<uint4*>(tsm)[i] = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < N * F; i += kTcT) Ps[i / F][i % F] = (float)P[i];
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < kTcStages; ++s) mbar_init(&full[s], 1);
    mbar_init(&mma_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTcCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);

  // thread 0 issues the copies of the CTA's k-th element into stage k % S
  auto issue = [&](int64_t k) {
    const int64_t e = blockIdx.x + k * stride;
    if (e >= B) return;
    const int s = (int)(k % kTcStages);
    unsigned char* st = stages + (size_t)s * kTcStage;
    const int4 nb = reinterpret_cast<const int4*>(nbe)[e];
    nbs[s][0] = nb.x;
    nbs[s][1] = nb.y;
    nbs[s][2] = nb.z;
    nbs[s][3] = nb.w;
    const unsigned char* src = reinterpret_cast<const unsigned char*>(tcblk) + (size_t)e * kTcElem;
    uint32_t bytes = 0;
    if (smooth) bytes += kTcWBytes;
    if (!zerox) bytes += kTcABytes;
    if (b) bytes += 20 * kNR * 4;
    mbar_expect_tx(&full[s], bytes);
    if (smooth && !zerox) {
      bulk_copy_g2s(st + kTcStW, src, kTcElem, &full[s]);
    } else if (smooth) {
      bulk_copy_g2s(st + kTcStW, src, kTcWBytes, &full[s]);
    } else if (!zerox) {
      bulk_copy_g2s(st + kTcStA, src + kTcWBytes, kTcABytes, &full[s]);
    }
    if (b) bulk_copy_g2s(st + kTcStB, b + e * (int64_t)N * kNR, 20 * kNR * 4, &full[s]);
  };
  if (tid == 0)
    for (int k = 0; k < kTcStages; ++k) issue(k);

  // thread roles in the epilogue: lane pair (2q, 2q+1) = RHS q
  const int q = tid >> 1, part = tid & 1;
  uint32_t mma_phase = 0;
  int64_t k = 0;
  for (int64_t e = blockIdx.x; e < B; e += stride, ++k) {
    const int s = (int)(k % kTcStages);
    unsigned char* st = stages + (size_t)s * kTcStage;
    if (tid == 0 && !mbar_wait_bounded(&full[s], (uint32_t)((k / kTcStages) & 1))) {
      atomicExch(err, 3);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    float v[24];
#pragma unroll
    for (int i = 0; i < 24; ++i) v[i] = 0.0f;
    if (!zerox) {
      // gather x of the element and its face neighbours into Aop: item i =
      // (slab j, node n, RHS quad q4); a warp covers 8 nodes x 4 quads, i.e.
      // four whole core matrices (conflict-free 16-byte stores)
      float4 xv[15];
#pragma unroll
      for (int u = 0; u < 15; ++u) {
        const int i = tid + u * kTcT;
        const int nn = i & 7, q4lo = (i >> 3) & 3, g = (i >> 5) % 3, q4hi = (i / 96) & 3, j = i / 384;
        const int n = 8 * g + nn, q4 = 4 * q4hi + q4lo;
        const int64_t src = j == 0 ? e : (int64_t)nbs[s][j - 1];
        xv[u] = (n < N && src >= 0) ? reinterpret_cast<const float4*>(x + (src * N + n) * kNR)[q4]
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 15; ++u) {
        const int i = tid + u * kTcT;
        const int nn = i & 7, q4lo = (i >> 3) & 3, g = (i >> 5) % 3, q4hi = (i / 96) & 3, j = i / 384;
        const int n = 8 * g + nn, q4 = 4 * q4hi + q4lo;
        if (n < N)   // core matrix (rows 8 q4 .., K group 3 j + g), K row nn
          *reinterpret_cast<uint4*>(Aop + (3 * j + g) * kTcLBO + q4 * 128 + nn * 16) = split_hilo4(xv[u]);
      }
      fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_addr(Aop), b0 = smem_addr(st + kTcStA);
#pragma unroll
        for (int ks = 0; ks < 8; ++ks)
          tc_mma(tmem, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128), tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128),
                 kTcIdescA, ks > 0 ? 1u : 0u);
        tc_commit(&mma_bar);
        if (!mbar_wait_bounded(&mma_bar, mma_phase)) {
          atomicExch(err, 3);
          abort_flag = 1;
        }
      }
      mma_phase ^= 1u;
      __syncthreads();   // one waiter, so that every warp takes the same branch below
      tc_fence_after();
      if (!abort_flag) {
        float t8[8];
#pragma unroll
        for (int c8 = 0; c8 < 3; ++c8) {
          tc_ld8(lane_base + 8 * c8, t8);
          tc_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) v[8 * c8 + i] = t8[i];
        }
      }
    }
    // hi + lo rows: both threads of the pair hold the sum of RHS q
#pragma unroll
    for (int n = 0; n < N; ++n) v[n] += __shfl_xor_sync(0xffffffffu, v[n], 1);
    const float* bst = reinterpret_cast<const float*>(st + kTcStB);
    float res[N];
#pragma unroll
    for (int n = 0; n < N; ++n) res[n] = (b ? bst[n * kNR + q] : 0.0f) - v[n];
    if (r) {
#pragma unroll
      for (int n0 = 0; n0 < N; n0 += 2)   // the pair splits the rows: part 0 even, part 1 odd
        r[(e * N + n0 + part) * kNR + q] = sgn * (part ? res[n0 + 1] : res[n0]);
    }
    if (restrict_) {
      float p0 = 0.f, p1 = 0.f;
      const int c0 = 2 * part;
#pragma unroll
      for (int n = 0; n < N; ++n) {
        p0 = fmaf(Ps[n][c0], res[n], p0);
        p1 = fmaf(Ps[n][c0 + 1], res[n], p1);
      }
      r1[(e * F + c0) * kNR + q] = p0;
      r1[(e * F + c0 + 1) * kNR + q] = p1;
    }
    if (smooth && !abort_flag) {   // abort_flag is uniform here (read after a barrier)
      // residual rows of the K-major operand: row 2q (hi) or 2q+1 (lo),
      // K slots n = 0..19 in groups of 8 (slots 20..31 stay zero)
#pragma unroll
      for (int g = 0; g < 3; ++g) {
        uint32_t wv[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int n0 = 8 * g + 2 * h;
          float a0 = n0 < N ? res[n0] : 0.0f, a1 = n0 + 1 < N ? res[n0 + 1] : 0.0f;
          if (part) {
            a0 -= __bfloat162float(__float2bfloat16_rn(a0));
            a1 -= __bfloat162float(__float2bfloat16_rn(a1));
          }
          wv[h] = pack_bf16x2(a0, a1);
        }
        *reinterpret_cast<uint4*>(Rop + g * kTcLBO + (tid >> 3) * 128 + (tid & 7) * 16) =
            make_uint4(wv[0], wv[1], wv[2], wv[3]);
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_addr(Rop), b0 = smem_addr(st + kTcStW);
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
          tc_mma(tmem + 32, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128),
                 tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128), kTcIdescR, ks > 0 ? 1u : 0u);
        tc_commit(&mma_bar);
        if (!mbar_wait_bounded(&mma_bar, mma_phase)) {
          atomicExch(err, 3);
          abort_flag = 1;
        }
      }
      mma_phase ^= 1u;
      __syncthreads();
      tc_fence_after();
      if (!abort_flag) {
        float c[24], t8[8];
#pragma unroll
        for (int c8 = 0; c8 < 3; ++c8) {
          tc_ld8(lane_base + 32 + 8 * c8, t8);
          tc_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) c[8 * c8 + i] = t8[i];
        }
#pragma unroll
        for (int n = 0; n < N; ++n) c[n] += __shfl_xor_sync(0xffffffffu, c[n], 1);
#pragma unroll
        for (int n0 = 0; n0 < N; n0 += 2) {
          const int64_t o = (e * N + n0 + part) * kNR + q;
          x_out[o] = ws * (part ? c[n0 + 1] : c[n0]) + (zerox ? 0.0f : x[o]);
        }
      }
    }
    tc_fence_before();
    __syncthreads();   // stage s, Aop, Rop and the accumulators are free again
    if (abort_flag) break;
    if (tid == 0) {
      fence_async_smem();
      issue(k + kTcStages);
    }
  }
  if (abort_flag && tid == 0) {
    // copies this CTA issued and did not consume
    for (int64_t j = k; j < k + kTcStages; ++j) {
      if (blockIdx.x + j * stride >= B) break;
      (void)mbar_wait_bounded(&full[j % kTcStages], (uint32_t)((j / kTcStages) & 1));
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
}


// ---------------------------------------------------------------------------
// Split-x pipeline: the preconditioner's iterate is kept in global memory in
// the tensor-core operand layout itself, so the smoothing kernel moves it to
// shared memory with bulk copies and multiplies without converting.
//
// Split layout of one element's x (64 RHS, 20 nodes padded to 24), 6,144
// bytes: K group kg = n / 8 (2,048 bytes) x M group mi = q / 4 (128 bytes) x
// node row n % 8 (16 bytes) x (RHS q % 4) x (BF16 high part, BF16 rounding
// of the remainder); nodes 20..23 are zero.  It is exactly one element's
// three K groups of the MN-major operand, so the five slabs of an element
// and its face neighbours, copied back to back, form the whole A operand.
constexpr int kSplit = 6144;
constexpr int RF_OUT_SPLIT = 32;                  // x_out in the split layout (else FP32 interleaved)
constexpr int kTsStages = 2;
constexpr int kTsCTA = 2;
// stage: [W | blocks | zero chunk | x slabs (own, 4 faces) | zero K group | b slab]
constexpr int kTsW = 0, kTsA = kTcWBytes, kTsZ = kTcElem, kTsX = kTcElem + kTcChunk;
constexpr int kTsXZ = kTsX + 5 * kSplit, kTsB = kTsXZ + kTcLBO;
constexpr int kTsStage = kTsB + 20 * kNR * 4;     // 43,968 bytes
constexpr int kTsDyn = kTsStages * kTsStage + kTcRop + kSplit;

__device__ __forceinline__ int split_off(int n, int q) {
  return (n >> 3) * kTcLBO + (q >> 2) * 128 + (n & 7) * 16 + (q & 3) * 4;
}

__device__ __forceinline__ uint32_t split_pack(float v) {
  const float h = __bfloat162float(__float2bfloat16_rn(v));
  return pack_bf16x2(h, v - h);
}

__device__ __forceinline__ float split_value(uint32_t w) {
  return __uint_as_float(w << 16) + __uint_as_float(w & 0xFFFF0000u);
}

__device__ __forceinline__ void bulk_store_s2g(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// FP32 interleaved -> split (one thread per (element, node, 4 RHS))
__global__ void to_split_kernel(const float* __restrict__ x, unsigned char* __restrict__ xs, int64_t B) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * 20 * (kNR / 4)) return;
  const int64_t e = t / (20 * (kNR / 4));
  const int rem = (int)(t - e * (20 * (kNR / 4)));
  const int n = rem / (kNR / 4), q4 = rem % (kNR / 4);
  const float4 v = reinterpret_cast<const float4*>(x + (e * 20 + n) * kNR)[q4];
  *reinterpret_cast<uint4*>(xs + e * kSplit + split_off(n, 4 * q4)) = split_hilo4(v);
}

// x (split) += P (w * ecg) at the element's corners: the P1 -> P3 coarse
// correction of bprolong_kernel on the split layout
__global__ void __launch_bounds__(320) bprolong_split_kernel(unsigned char* __restrict__ xs,
                                                             const float* __restrict__ ecg, const int* __restrict__ pos,
                                                             const int* __restrict__ p1cg,
                                                             const float* __restrict__ wdg,
                                                             const float* __restrict__ P, int64_t B) {
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
  uint4* p = reinterpret_cast<uint4*>(xs + e * kSplit + split_off(n, 4 * q4));
  const uint4 w = *p;
  const float4 xv = make_float4(split_value(w.x) + v.x, split_value(w.y) + v.y, split_value(w.z) + v.z,
                                split_value(w.w) + v.w);
  *p = split_hilo4(xv);
}

// The batched smoothing / residual step on split x: flags as bres_kernel
// plus RF_OUT_SPLIT; x (split) of the element and its face neighbours, its
// blocks, smoother matrix and b slab arrive by bulk copies into a ring of
// kTsStages stages; D = Aop * Bop on the tensor cores (Aop = the copied x
// slabs, no conversion); epilogue as bres_tc05_kernel, with x_out written in
// the split layout through a staging buffer and one bulk store per element,
// or as FP32.
__global__ void __launch_bounds__(kTcT, kTsCTA) bres_tcs_kernel(
    const __nv_bfloat16* __restrict__ tcblk, const int* __restrict__ nbe, const unsigned char* __restrict__ xs,
    const float* __restrict__ b, float* __restrict__ r, void* __restrict__ x_out, int64_t B, int flags,
    const float* __restrict__ P, float* __restrict__ r1, int* __restrict__ err, const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4;
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* stages = tsm;
  unsigned char* Rop = tsm + kTsStages * kTsStage;
  unsigned char* Out = Rop + kTcRop;
  __shared__ __align__(8) uint64_t full[kTsStages];
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ float Ps[N][F];
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  const bool restrict_ = flags & RF_RESTRICT;
  const bool out_split = flags & RF_OUT_SPLIT;
  const float ws = wsp ? *wsp : 1.0f;
  const float sgn = (flags & RF_NEG) ? -1.0f : 1.0f;
  const int64_t stride = gridDim.x;
  for (int i = tid; i < kTsDyn / 16; i += kTcT) reinterpret_cast<uint4*>(tsm)[i] = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < N * F; i += kTcT) Ps[i / F][i % F] = (float)P[i];
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < kTsStages; ++s) mbar_init(&full[s], 1);
    mbar_init(&mma_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTcCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);

  auto issue = [&](int64_t k) {
    const int64_t e = blockIdx.x + k * stride;
    if (e >= B) return;
    const int s = (int)(k % kTsStages);
    unsigned char* st = stages + (size_t)s * kTsStage;
    const unsigned char* src = reinterpret_cast<const unsigned char*>(tcblk) + (size_t)e * kTcElem;
    int nb[F] = {-1, -1, -1, -1};
    uint32_t bytes = 0;
    if (smooth) bytes += kTcWBytes;
    if (!zerox) {
      const int4 n4 = reinterpret_cast<const int4*>(nbe)[e];
      nb[0] = n4.x;
      nb[1] = n4.y;
      nb[2] = n4.z;
      nb[3] = n4.w;
      bytes += kTcABytes + kSplit;
      for (int f = 0; f < F; ++f)
        if (nb[f] >= 0) bytes += kSplit;
    }
    if (b) bytes += 20 * kNR * 4;
    mbar_expect_tx(&full[s], bytes);
    if (smooth && !zerox)
      bulk_copy_g2s(st + kTsW, src, kTcElem, &full[s]);
    else if (smooth)
      bulk_copy_g2s(st + kTsW, src, kTcWBytes, &full[s]);
    else if (!zerox)
      bulk_copy_g2s(st + kTsA, src + kTcWBytes, kTcABytes, &full[s]);
    if (!zerox) {
      bulk_copy_g2s(st + kTsX, xs + e * kSplit, kSplit, &full[s]);
      for (int f = 0; f < F; ++f)   // a boundary face keeps a stale slab: its block is zero
        if (nb[f] >= 0) bulk_copy_g2s(st + kTsX + (1 + f) * kSplit, xs + (int64_t)nb[f] * kSplit, kSplit, &full[s]);
    }
    if (b) bulk_copy_g2s(st + kTsB, b + e * (int64_t)N * kNR, 20 * kNR * 4, &full[s]);
  };
  if (tid == 0)
    for (int k = 0; k < kTsStages; ++k) issue(k);

  const int q = tid >> 1, part = tid & 1;
  uint32_t mma_phase = 0;
  int64_t k = 0;
  for (int64_t e = blockIdx.x; e < B; e += stride, ++k) {
    const int s = (int)(k % kTsStages);
    unsigned char* st = stages + (size_t)s * kTsStage;
    if (!mbar_wait_bounded(&full[s], (uint32_t)((k / kTsStages) & 1))) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      if (tid == 0) atomicExch(err, 3);
      break;
    }
    float v[24];
#pragma unroll
    for (int i = 0; i < 24; ++i) v[i] = 0.0f;
    if (!zerox) {
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_addr(st + kTsX), b0 = smem_addr(st + kTsA);
#pragma unroll
        for (int ks = 0; ks < 8; ++ks)
          tc_mma(tmem, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128), tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128),
                 kTcIdescA, ks > 0 ? 1u : 0u);
        tc_commit(&mma_bar);
        if (!mbar_wait_bounded(&mma_bar, mma_phase)) {
          atomicExch(err, 3);
          abort_flag = 1;
        }
      }
      mma_phase ^= 1u;
      __syncthreads();
      tc_fence_after();
      if (!abort_flag) {
        float t8[8];
#pragma unroll
        for (int c8 = 0; c8 < 3; ++c8) {
          tc_ld8(lane_base + 8 * c8, t8);
          tc_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) v[8 * c8 + i] = t8[i];
        }
      }
    }
#pragma unroll
    for (int n = 0; n < N; ++n) v[n] += __shfl_xor_sync(0xffffffffu, v[n], 1);
    const float* bst = reinterpret_cast<const float*>(st + kTsB);
    float res[N];
#pragma unroll
    for (int n = 0; n < N; ++n) res[n] = (b ? bst[n * kNR + q] : 0.0f) - v[n];
    if (r) {
#pragma unroll
      for (int n0 = 0; n0 < N; n0 += 2) r[(e * N + n0 + part) * kNR + q] = sgn * (part ? res[n0 + 1] : res[n0]);
    }
    if (restrict_) {
      float p0 = 0.f, p1 = 0.f;
      const int c0 = 2 * part;
#pragma unroll
      for (int n = 0; n < N; ++n) {
        p0 = fmaf(Ps[n][c0], res[n], p0);
        p1 = fmaf(Ps[n][c0 + 1], res[n], p1);
      }
      r1[(e * F + c0) * kNR + q] = p0;
      r1[(e * F + c0 + 1) * kNR + q] = p1;
    }
    if (smooth && !abort_flag) {   // abort_flag is uniform here (read after a barrier)
#pragma unroll
      for (int g = 0; g < 3; ++g) {
        uint32_t wv[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int n0 = 8 * g + 2 * h;
          float a0 = n0 < N ? res[n0] : 0.0f, a1 = n0 + 1 < N ? res[n0 + 1] : 0.0f;
          if (part) {
            a0 -= __bfloat162float(__float2bfloat16_rn(a0));
            a1 -= __bfloat162float(__float2bfloat16_rn(a1));
          }
          wv[h] = pack_bf16x2(a0, a1);
        }
        *reinterpret_cast<uint4*>(Rop + g * kTcLBO + (tid >> 3) * 128 + (tid & 7) * 16) =
            make_uint4(wv[0], wv[1], wv[2], wv[3]);
      }
      if (tid == 0 && out_split) bulk_wait_read();   // the staging buffer's previous store has been read
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_addr(Rop), b0 = smem_addr(st + kTsW);
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
          tc_mma(tmem + 32, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128),
                 tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128), kTcIdescR, ks > 0 ? 1u : 0u);
        tc_commit(&mma_bar);
        if (!mbar_wait_bounded(&mma_bar, mma_phase)) {
          atomicExch(err, 3);
          abort_flag = 1;
        }
      }
      mma_phase ^= 1u;
      __syncthreads();
      tc_fence_after();
      if (!abort_flag) {
        float c[24], t8[8];
#pragma unroll
        for (int c8 = 0; c8 < 3; ++c8) {
          tc_ld8(lane_base + 32 + 8 * c8, t8);
          tc_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) c[8 * c8 + i] = t8[i];
        }
#pragma unroll
        for (int n = 0; n < N; ++n) c[n] += __shfl_xor_sync(0xffffffffu, c[n], 1);
        const unsigned char* xo_own = st + kTsX;
#pragma unroll
        for (int n0 = 0; n0 < N; n0 += 2) {
          const int n = n0 + part;
          const float xv = zerox ? 0.0f : split_value(*reinterpret_cast<const uint32_t*>(xo_own + split_off(n, q)));
          const float xo = xv + ws * (part ? c[n0 + 1] : c[n0]);
          if (out_split)
            *reinterpret_cast<uint32_t*>(Out + split_off(n, q)) = split_pack(xo);
          else
            reinterpret_cast<float*>(x_out)[(e * N + n) * kNR + q] = xo;
        }
        if (out_split) {
          fence_async_smem();
          __syncthreads();
          if (tid == 0) bulk_store_s2g(reinterpret_cast<unsigned char*>(x_out) + e * kSplit, Out, kSplit);
        }
      }
    }
    tc_fence_before();
    __syncthreads();   // stage s, Rop and the accumulators are free again
    if (abort_flag) break;
    if (tid == 0) {
      fence_async_smem();
      issue(k + kTsStages);
    }
  }
  if (abort_flag && tid == 0) {
    for (int64_t j = k; j < k + kTsStages; ++j) {
      if (blockIdx.x + j * stride >= B) break;
      (void)mbar_wait_bounded(&full[j % kTsStages], (uint32_t)((j / kTsStages) & 1));
    }
  }
  if (tid == 0) bulk_wait_all();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
}


// ---------------------------------------------------------------------------
// Warp-specialized form of bres_tcs_kernel (same arithmetic, one CTA per SM):
//   warp 0      bulk copies of the next elements into a ring of kTwStages
//               stages (waits for a stage to be released);
//   warp 1      one thread issues the MMAs, software-pipelined: the block
//               product D1 of element k, then the smoothing product D2 of
//               element k - 1 (whose residual operand Rop the epilogue has
//               written meanwhile);
//   warps 2..9  the epilogue on TMEM lane quadrant (warp % 4) and half of the
//               block rows (warps 2..5 rows 0..9, warps 6..9 rows 10..19),
//               also pipelined: the residual half of element k (D1 -> res ->
//               Rop), then the update half of element k - 1 (D2 -> x_out).
// Three accumulator sets (t = k % 3) and three Rop buffers let the MMAs of
// one element run while the epilogue works on the two before it.  The roles
// meet only at mbarriers; every wait is bounded (on a time-out the kernel
// records error 3 and every role leaves its loop).
constexpr int kTwT = 320;
constexpr int kTwStages = 4;
constexpr int kTwNT = 3;                          // accumulator sets / Rop buffers
constexpr int kTwDyn = kTwStages * kTsStage + kTwNT * kTcRop + 2 * kSplit;
constexpr uint32_t kTwCols = 256;                 // set t: D1 at 64 t, D2 at 64 t + 32

__device__ __forceinline__ void mbar_arrive1(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }

__global__ void __launch_bounds__(kTwT, 1) bres_tcw_kernel(
    const __nv_bfloat16* __restrict__ tcblk, const int* __restrict__ nbe, const unsigned char* __restrict__ xs,
    const float* __restrict__ b, void* __restrict__ x_out, int64_t B, int flags, const float* __restrict__ P,
    float* __restrict__ r1, int* __restrict__ err, const float* __restrict__ wsp) {
  constexpr int N = 20, F = 4, S = kTwStages, NT = kTwNT;
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* stages = tsm;
  unsigned char* Rop = tsm + S * kTsStage;           // NT buffers
  unsigned char* Out = Rop + NT * kTcRop;            // two buffers
  __shared__ __align__(8) uint64_t full[S], empty[S], d1full[NT], ropfull[NT], d2full[NT], tfree[NT];
  __shared__ uint32_t tmem_slot;
  __shared__ float Ps[N][F];
  __shared__ float red1[2][F][kNR];
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool zerox = flags & RF_ZEROX;
  const bool smooth = flags & RF_SMOOTH;
  const bool restrict_ = flags & RF_RESTRICT;
  const bool out_split = flags & RF_OUT_SPLIT;
  const int64_t stride = gridDim.x;
  const int64_t nmine = blockIdx.x < B ? (B - 1 - blockIdx.x) / stride + 1 : 0;
  for (int i = tid; i < kTwDyn / 16; i += kTwT) reinterpret_cast<uint4*>(tsm)[i] = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < N * F; i += kTwT) Ps[i / F][i % F] = (float)P[i];
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < NT; ++i) {
      mbar_init(&d1full[i], 1);
      mbar_init(&ropfull[i], 1);
      mbar_init(&d2full[i], 1);
      mbar_init(&tfree[i], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTwCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  auto wait = [&](uint64_t* bar, uint32_t parity) -> bool {
    for (uint32_t it = 0; it < kTmaSpinLimit; ++it) {
      if (mbar_try_wait(bar, parity)) return true;
      if (abort_flag) return false;
    }
    abort_flag = 1;
    atomicExch(err, 3);
    return false;
  };
  // the u-th use of a ring slot completes phase u: parity u & 1
  auto par = [](int64_t use) -> uint32_t { return (uint32_t)(use & 1); };
  int64_t issued = 0;

  if (warp == 0) {
    if (lane == 0) {
      // ---- producer ----
      for (int64_t k = 0; k < nmine && !abort_flag; ++k) {
        const int s = (int)(k % S);
        if (k >= S && !wait(&empty[s], par(k / S - 1))) break;
        const int64_t e = blockIdx.x + k * stride;
        unsigned char* st = stages + (size_t)s * kTsStage;
        const unsigned char* src = reinterpret_cast<const unsigned char*>(tcblk) + (size_t)e * kTcElem;
        int nb[F] = {-1, -1, -1, -1};
        uint32_t bytes = 0;
        if (smooth) bytes += kTcWBytes;
        if (!zerox) {
          const int4 n4 = reinterpret_cast<const int4*>(nbe)[e];
          nb[0] = n4.x;
          nb[1] = n4.y;
          nb[2] = n4.z;
          nb[3] = n4.w;
          bytes += kTcABytes + kSplit;
          for (int f = 0; f < F; ++f)
            if (nb[f] >= 0) bytes += kSplit;
        }
        if (b) bytes += 20 * kNR * 4;
        mbar_expect_tx(&full[s], bytes);
        if (smooth && !zerox)
          bulk_copy_g2s(st + kTsW, src, kTcElem, &full[s]);
        else if (smooth)
          bulk_copy_g2s(st + kTsW, src, kTcWBytes, &full[s]);
        else if (!zerox)
          bulk_copy_g2s(st + kTsA, src + kTcWBytes, kTcABytes, &full[s]);
        if (!zerox) {
          bulk_copy_g2s(st + kTsX, xs + e * kSplit, kSplit, &full[s]);
          for (int f = 0; f < F; ++f)   // a boundary face keeps a stale slab: its block is zero
            if (nb[f] >= 0)
              bulk_copy_g2s(st + kTsX + (1 + f) * kSplit, xs + (int64_t)nb[f] * kSplit, kSplit, &full[s]);
        }
        if (b) bulk_copy_g2s(st + kTsB, b + e * (int64_t)N * kNR, 20 * kNR * 4, &full[s]);
        issued = k + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: D1(k), then D2(k - 1) ----
      auto mma2 = [&](int64_t j) -> bool {
        const int tj = (int)(j % NT);
        if (!wait(&ropfull[tj], par(j / NT))) return false;
        tc_fence_after();
        const uint32_t a0 = smem_addr(Rop + tj * kTcRop), b0 = smem_addr(stages + (size_t)(j % S) * kTsStage + kTsW);
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
          tc_mma(tmem + 64u * tj + 32u, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128),
                 tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128), kTcIdescR, ks > 0 ? 1u : 0u);
        tc_commit(&d2full[tj]);
        return true;
      };
      bool ok = true;
      for (int64_t k = 0; k < nmine && ok && !abort_flag; ++k) {
        const int s = (int)(k % S), t = (int)(k % NT);
        if (!wait(&full[s], par(k / S))) break;
        if (k >= NT && !wait(&tfree[t], par(k / NT - 1))) break;
        tc_fence_after();
        if (!zerox) {
          unsigned char* st = stages + (size_t)s * kTsStage;
          const uint32_t a0 = smem_addr(st + kTsX), b0 = smem_addr(st + kTsA);
#pragma unroll
          for (int ks = 0; ks < 8; ++ks)
            tc_mma(tmem + 64u * t, tc_sdesc(a0 + ks * 2 * kTcLBO, kTcLBO, 128),
                   tc_sdesc(b0 + ks * 2 * kTcChunk, kTcChunk, 128), kTcIdescA, ks > 0 ? 1u : 0u);
        }
        tc_commit(&d1full[t]);
        if (smooth && k >= 1) ok = mma2(k - 1);
      }
      if (ok && smooth && nmine > 0 && !abort_flag) (void)mma2(nmine - 1);
    }
  } else {
    // ---- epilogue: 8 warps, residual half of k then update half of k - 1 ----
    const int lq = warp & 3;                          // TMEM lane quadrant of this warp
    const int half = (warp - 2) >> 2;                 // block rows 0..9 or 10..19
    const int r = 32 * lq + lane, q = r >> 1, part = r & 1;
    const int n0 = 10 * half;
    const bool elected = warp == 2 && lane == 0;
    const float ws = wsp ? *wsp : 1.0f;
    const uint32_t lane_off = (uint32_t)(32 * lq) << 16;
    // 10 rows n0 .. n0+9 of accumulator column base col0 (columns 8 half ..)
    auto ld10 = [&](uint32_t col0, float (&v)[10]) {
      float a[8], c8[8];
      tc_ld8(tmem + lane_off + col0 + 8 * half, a);
      tc_ld8(tmem + lane_off + col0 + 8 * half + 8, c8);
      tc_wait_ld();
#pragma unroll
      for (int i = 0; i < 10; ++i) {   // row n0 + i sits at column offset i + 2 half
        const float lo = i < 8 ? a[i] : c8[i - 8];
        const float hi = i + 2 < 8 ? a[i + 2] : c8[i - 6];
        v[i] = half ? hi : lo;
      }
#pragma unroll
      for (int i = 0; i < 10; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], 1);
    };
    // residual half of element k: D1 -> res -> (r1) -> Rop[t]
    auto first = [&](int64_t k) -> bool {
      const int s = (int)(k % S), t = (int)(k % NT);
      const int64_t e = blockIdx.x + k * stride;
      unsigned char* st = stages + (size_t)s * kTsStage;
      wait(&full[s], par(k / S));
      wait(&d1full[t], par(k / NT));
      epi_sync();   // every epilogue thread sees the same abort_flag
      if (abort_flag) return false;
      tc_fence_after();
      float v[10];
      if (zerox) {
#pragma unroll
        for (int i = 0; i < 10; ++i) v[i] = 0.0f;
      } else {
        ld10(64u * t, v);
      }
      const float* bst = reinterpret_cast<const float*>(st + kTsB);
      float res[10];
#pragma unroll
      for (int i = 0; i < 10; ++i) res[i] = (b ? bst[(n0 + i) * kNR + q] : 0.0f) - v[i];
      if (restrict_) {
        if (part == 0) {
#pragma unroll
          for (int c = 0; c < F; ++c) {
            float p = 0.0f;
#pragma unroll
            for (int i = 0; i < 10; ++i) p = fmaf(Ps[n0 + i][c], res[i], p);
            red1[half][c][q] = p;
          }
        }
        epi_sync();
        if (half == 0 && part == 0)
#pragma unroll
          for (int c = 0; c < F; ++c) r1[(e * F + c) * kNR + q] = red1[0][c][q] + red1[1][c][q];
      }
      if (smooth) {
        // rows of the K-major residual operand: high (part 0) or low
        // (part 1) BF16 part of res[q][n] in K slot n
        uint32_t w[5];
#pragma unroll
        for (int h = 0; h < 5; ++h) {
          float a0 = res[2 * h], a1 = res[2 * h + 1];
          if (part) {
            a0 -= __bfloat162float(__float2bfloat16_rn(a0));
            a1 -= __bfloat162float(__float2bfloat16_rn(a1));
          }
          w[h] = pack_bf16x2(a0, a1);
        }
        unsigned char* row = Rop + t * kTcRop + (r >> 3) * 128 + (r & 7) * 16;
        if (half == 0) {   // slots 0..9: group 0 (0..7), group 1 (8, 9)
          *reinterpret_cast<uint4*>(row) = make_uint4(w[0], w[1], w[2], w[3]);
          *reinterpret_cast<uint32_t*>(row + kTcLBO) = w[4];
        } else {           // slots 10..19: group 1 (10..15), group 2 (16..19)
          *reinterpret_cast<uint32_t*>(row + kTcLBO + 4) = w[0];
          *reinterpret_cast<uint2*>(row + kTcLBO + 8) = make_uint2(w[1], w[2]);
          *reinterpret_cast<uint2*>(row + 2 * kTcLBO) = make_uint2(w[3], w[4]);
        }
        fence_async_smem();
        tc_fence_before();
        epi_sync();
        if (elected) mbar_arrive1(&ropfull[t]);
      } else {
        tc_fence_before();
        epi_sync();   // res read from D1 and the stage: release both
        if (elected) {
          mbar_arrive1(&tfree[t]);
          mbar_arrive1(&empty[s]);
        }
      }
      return true;
    };
    // update half of element j: D2 -> x_out; releases its stage and set
    auto second = [&](int64_t j) -> bool {
      const int s = (int)(j % S), t = (int)(j % NT);
      const int64_t e = blockIdx.x + j * stride;
      unsigned char* st = stages + (size_t)s * kTsStage;
      unsigned char* ob = Out + (int)(j & 1) * kSplit;
      if (elected && out_split) bulk_wait_read1();   // this buffer's store of element j - 2 has been read
      wait(&d2full[t], par(j / NT));
      epi_sync();
      if (abort_flag) return false;
      tc_fence_after();
      float c[10];
      ld10(64u * t + 32u, c);
      const unsigned char* xo_own = st + kTsX;
#pragma unroll
      for (int i0 = 0; i0 < 10; i0 += 2) {   // the pair splits the rows: part 0 even, part 1 odd
        const int n = n0 + i0 + part;
        const float cv = part ? c[i0 + 1] : c[i0];
        const float xv = zerox ? 0.0f : split_value(*reinterpret_cast<const uint32_t*>(xo_own + split_off(n, q)));
        const float xo = xv + ws * cv;
        if (out_split)
          *reinterpret_cast<uint32_t*>(ob + split_off(n, q)) = split_pack(xo);
        else
          reinterpret_cast<float*>(x_out)[(e * N + n) * kNR + q] = xo;
      }
      if (out_split) fence_async_smem();
      tc_fence_before();
      epi_sync();
      if (elected) {
        if (out_split) bulk_store_s2g(reinterpret_cast<unsigned char*>(x_out) + e * kSplit, ob, kSplit);
        mbar_arrive1(&tfree[t]);
        mbar_arrive1(&empty[s]);
      }
      return true;
    };
    bool ok = true;
    for (int64_t k = 0; k < nmine && ok; ++k) {
      ok = first(k);
      if (ok && smooth && k >= 1) ok = second(k - 1);
    }
    if (ok && smooth && nmine > 0) (void)second(nmine - 1);
    if (elected) bulk_wait_all();
  }
  __syncthreads();
  if (warp == 0 && lane == 0 && abort_flag) {
    // copies issued and possibly still in flight: wait (bounded) for each
    // stage's outstanding phase
    for (int64_t k = issued > S ? issued - S : 0; k < issued; ++k)
      (void)mbar_wait_bounded(&full[k % S], par(k / S));
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTwCols));
}

}  // namespace
