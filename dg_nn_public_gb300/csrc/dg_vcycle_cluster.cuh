// FP32 SFC V-cycle of the mixed preconditioner on one thread-block cluster.
//
// The levels above the dense coarse level are small (c2: 9,261 and 4,631
// rows), so the launch chain of the V-cycle (vertex gather, 3 + 3 Jacobi
// sweeps and 2 pair-sum restrictions down, 2 prolongations and 2 + 2 sweeps
// up: 17 launches of a few microseconds each) is bound by launch and
// dependency latency, not by bytes.  Here the down leg and the up leg each
// run as ONE launch of a cluster of up to 16 CTAs.  Each CTA owns a
// contiguous slice of every level's rows and holds in its shared memory
//   * the slice of the level vectors (e in two buffers, r, rr), which the
//     other CTAs read as distributed shared memory (mapa +
//     ld.shared::cluster);
//   * an image of its rows of the level matrix, copied in before the
//     programmatic-launch wait: row offsets, diagonal, and per entry the
//     value with the owner CTA and slice index of its column.
// A cluster barrier (barrier.cluster arrive.release / wait.acquire)
// separates the phases.  The dense coarse mat-vec stays a full-GPU launch
// between the two legs: the down leg leaves each level's e and r in global
// memory and the dense level's r, the up leg starts from them and leaves
// level 0's e.
//
// The arithmetic is that of the launch chain, operation for operation, so
// both give the same bits:
//   * gather_cg32_kernel: per vertex, 32 lane-strided FMA partial sums over
//     its DG copies, combined in the shuffle-down tree order (here 8 lanes
//     per vertex, each holding 4 of the 32 partial sums: the tree's first
//     two levels are formed in the lane, the last three by xor shuffles);
//   * lev_jacobi_kernel: 8 lanes per row, lane-strided FMA partial sums
//     combined by xor shuffles, then e_out = fma(rr / diag, w, e_in);
//   * lev_restrict_kernel / lev_prolong_kernel: the same pair sums and adds.
//
// Every CTA runs the same sequence of cluster barriers (the phase loops
// depend on the launch parameters only, and no thread returns early), so
// every barrier completes.  A barrier precedes the first access to another
// CTA's shared memory (all CTAs have started) and follows the last one (no
// CTA exits while another still reads its slice).
//
// Reference: multigrid_linearelastic.py:33-38 (level Jacobi), :147-153
// (restriction), :163-164 (prolongation); the DG -> P1CG gather of
// volume_mf_diff.py's restrictor.

constexpr int kVcMaxLev = 6;       // levels above the dense coarse level
constexpr int kVcThreads = 1024;
constexpr int kVcSmemMax = 200 * 1024;
constexpr int kVcLocalBits = 20;   // matrix image: column = owner << 20 | slice index

struct VcLevel {
  const int* up;   // global: prolongation source of each row
  float* e;        // global: e after the down leg (level 0: the V-cycle result)
  float* r;        // global: r of the level (the dense level: its input)
  int n;
  int ch;          // rows per CTA slice
  int off;         // shared-memory word offset of the slice vectors e0, e1, r, rr
  int rp_off;      // shared-memory word offsets of the matrix image: row offsets,
  int dg_off;      //   diagonal,
  int ent_off;     //   entries (column code, value bits)
  float inv_ch;    // 1 / ch, for the owner of a row
};

struct VcParams {
  VcLevel lev[kVcMaxLev + 1];   // levels 0 .. lc (lc = the dense level)
  int lc, npre, npost;
  float w;
  // matrix images of all CTAs: CTA r's image is img[r * img_words ..), copied
  // to shared-memory word img_off
  const int4* img;
  int img_words;
  int img_off;
  // vertex gather of the element P1 restrictions into level 0's r
  const float* r1;
  const int* gptr;
  const int* gent;
  const float* wdg;
  const int* pos;
  int ncg;
};

__device__ __forceinline__ unsigned vc_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned vc_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

// all threads of all CTAs of the cluster; writes before it (shared memory
// of any CTA, global memory) are visible to reads after it in the cluster
__device__ __forceinline__ void vc_sync() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ void vc_slice(int n, int ch, unsigned rank, int& r0, int& r1) {
  r0 = min(n, (int)rank * ch);
  r1 = min(n, r0 + ch);
}

// owner CTA of row j and its index there
__device__ __forceinline__ void vc_owner(const VcLevel& L, int j, unsigned& owner, int& local) {
  int o = (int)((float)j * L.inv_ch);
  if (o * L.ch > j) --o;
  else if ((o + 1) * L.ch <= j) ++o;
  owner = (unsigned)o;
  local = j - o * L.ch;
}

// the shared::cluster address in CTA `rank` of a shared::cta address
__device__ __forceinline__ uint32_t vc_map(uint32_t a, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__device__ __forceinline__ float vc_ld(uint32_t addr) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}

__device__ __forceinline__ void vc_st(uint32_t addr, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// element j of slice vector `buf` (0 = e0, 1 = e1, 2 = r, 3 = rr) of level L,
// wherever its owner is
__device__ __forceinline__ float vc_get(float* sm, const VcLevel& L, int buf, int j) {
  unsigned o;
  int loc;
  vc_owner(L, j, o, loc);
  return vc_ld(vc_map(smem_addr(sm + L.off + buf * L.ch + loc), o));
}

// this CTA's matrix image into shared memory (before the programmatic-
// launch wait: fixed data)
__device__ __forceinline__ void vc_load_image(const VcParams& p, float* sm, unsigned rank) {
  const int4* src = p.img + (size_t)rank * (p.img_words / 4);
  int4* dst = reinterpret_cast<int4*>(sm + p.img_off);
  for (int i = threadIdx.x; i < p.img_words / 4; i += blockDim.x) dst[i] = __ldg(src + i);
}

// level 0's r[pos[v]] = sum over the DG copies of vertex v of wdg * r1;
// 8 lanes per vertex, lane l holding the partial sums P(l + 8 jj), jj < 4,
// of the 32-lane order
__device__ void vc_gather(const VcParams& p, float* sm, unsigned rank, unsigned cs) {
  const VcLevel& L0 = p.lev[0];
  const int chv = (p.ncg + (int)cs - 1) / (int)cs;
  int s0, s1;
  vc_slice(p.ncg, chv, rank, s0, s1);
  const int ntask = (s1 - s0) * 8;
  for (int t0 = 0; t0 < ntask; t0 += blockDim.x) {
    const int t = t0 + (int)threadIdx.x;
    const bool act = t < ntask;
    const int v = s0 + (t >> 3), lane = t & 7;
    float P[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (act) {
      const int k0 = p.gptr[v], k1 = p.gptr[v + 1];
      for (int kb = k0 + lane; kb < k1; kb += 32) {
        int ent[4];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) ent[jj] = kb + 8 * jj < k1 ? p.gent[kb + 8 * jj] : -1;
        float wv[4], rv[4];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          wv[jj] = ent[jj] >= 0 ? (float)p.wdg[ent[jj]] : 0.0f;
          rv[jj] = ent[jj] >= 0 ? p.r1[ent[jj]] : 0.0f;
        }
#pragma unroll
        for (int jj = 0; jj < 4; ++jj)
          if (ent[jj] >= 0) P[jj] = __fmaf_rn(wv[jj], rv[jj], P[jj]);
      }
    }
    // (P(l) + P(l + 16)) + (P(l + 8) + P(l + 24)), then lanes l, l ^ 4, ...
    float a = (P[0] + P[2]) + (P[1] + P[3]);
    a += __shfl_xor_sync(0xffffffffu, a, 4, 8);
    a += __shfl_xor_sync(0xffffffffu, a, 2, 8);
    a += __shfl_xor_sync(0xffffffffu, a, 1, 8);
    if (act && lane == 0) {
      unsigned o;
      int loc;
      vc_owner(L0, p.pos[v], o, loc);
      vc_st(vc_map(smem_addr(sm + L0.off + 2 * L0.ch + loc), o), a);
    }
  }
}

// one Jacobi sweep over the CTA's rows, 8 lanes per row: rr = r - A e_in,
// e_out = e_in + rr / diag * w; ein / eout select the slice buffers
// (ein < 0: zero guess), keep_rr stores rr
__device__ void vc_sweep(const VcLevel& L, float* sm, int ein, int eout, bool keep_rr, float w, unsigned rank) {
  int s0, s1;
  vc_slice(L.n, L.ch, rank, s0, s1);
  const int ntask = (s1 - s0) * 8;
  const int* rp = reinterpret_cast<const int*>(sm + L.rp_off);
  const float* dg = sm + L.dg_off;
  const int2* ent = reinterpret_cast<const int2*>(sm + L.ent_off);
  float* my = sm + L.off;
  const uint32_t ebase = smem_addr(sm + L.off + (ein >= 0 ? ein : 0) * L.ch);
  for (int t0 = 0; t0 < ntask; t0 += blockDim.x) {
    const int t = t0 + (int)threadIdx.x;
    const bool act = t < ntask;
    const int li = t >> 3, lane = t & 7;
    float s = 0.0f;
    if (act && ein >= 0) {
      const int k1 = rp[li + 1];
      for (int kb = rp[li] + lane; kb < k1; kb += 32) {
        float x[4], v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const bool ok = kb + 8 * q < k1;
          const int2 c = ent[ok ? kb + 8 * q : kb];
          v[q] = __int_as_float(c.y);
          const uint32_t loc = (uint32_t)c.x & ((1u << kVcLocalBits) - 1u);
          x[q] = ok ? vc_ld(vc_map(ebase + 4u * loc, (uint32_t)c.x >> kVcLocalBits)) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (kb + 8 * q < k1) s = __fmaf_rn(v[q], x[q], s);
      }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 4, 8);
    s += __shfl_xor_sync(0xffffffffu, s, 2, 8);
    s += __shfl_xor_sync(0xffffffffu, s, 1, 8);
    if (act && lane == 0) {
      const float rr = my[2 * L.ch + li] - s;
      const float e0 = ein >= 0 ? my[ein * L.ch + li] : 0.0f;
      my[eout * L.ch + li] = __fmaf_rn(rr / dg[li], w, e0);
      if (keep_rr) my[3 * L.ch + li] = rr;
    }
  }
}

// down leg: gather, then per level npre + 1 sweeps (the last one keeps its
// residual) and the restriction to the next level (the dense level's r to
// global memory); each level's e and r are left in global memory
__global__ void __launch_bounds__(kVcThreads, 1) vcycle_down_kernel(const VcParams p) {
  extern __shared__ __align__(16) float vc_smem[];
  const unsigned rank = vc_rank();
  vc_load_image(p, vc_smem, rank);
  vc_sync();   // images in place, every CTA of the cluster running
  pdl_wait_then_trigger();
  vc_gather(p, vc_smem, rank, vc_size());
  vc_sync();
  for (int l = 0; l < p.lc; ++l) {
    const VcLevel& L = p.lev[l];
    int cur = 0;
    for (int it = 0; it <= p.npre; ++it) {
      const int ein = (l == 0 && it == 0) ? -1 : cur;
      vc_sweep(L, vc_smem, ein, cur ^ 1, it == p.npre, p.w, rank);
      cur ^= 1;
      vc_sync();
    }
    // the next level: r_next[i] = rr[2i] + rr[2i+1], e_next[i] = e[2i] + e[2i+1]
    const VcLevel& N = p.lev[l + 1];
    const bool dense = l + 1 == p.lc;
    int t0, t1;
    vc_slice(N.n, N.ch, rank, t0, t1);
    for (int i = t0 + (int)threadIdx.x; i < t1; i += blockDim.x) {
      const int a = 2 * i, b = 2 * i + 1;
      const float rn = vc_get(vc_smem, L, 3, a) + (b < L.n ? vc_get(vc_smem, L, 3, b) : 0.0f);
      if (dense) {
        N.r[i] = rn;
      } else {
        const float en = vc_get(vc_smem, L, cur, a) + (b < L.n ? vc_get(vc_smem, L, cur, b) : 0.0f);
        vc_smem[N.off + 2 * N.ch + (i - t0)] = rn;
        vc_smem[N.off + (i - t0)] = en;   // e0 of the next level
      }
    }
    // this level's e and r for the up leg
    int s0, s1;
    vc_slice(L.n, L.ch, rank, s0, s1);
    for (int i = s0 + (int)threadIdx.x; i < s1; i += blockDim.x) {
      L.e[i] = vc_smem[L.off + cur * L.ch + (i - s0)];
      L.r[i] = vc_smem[L.off + 2 * L.ch + (i - s0)];
    }
    vc_sync();
  }
}

// up leg: the levels' e and r as the down leg left them, then per level
// (coarse to fine) the prolongation of the coarser correction and npost
// sweeps; level 0's e to global memory
__global__ void __launch_bounds__(kVcThreads, 1) vcycle_up_kernel(const VcParams p) {
  extern __shared__ __align__(16) float vc_smem[];
  const unsigned rank = vc_rank();
  vc_load_image(p, vc_smem, rank);
  pdl_wait_then_trigger();
  for (int l = 0; l < p.lc; ++l) {
    const VcLevel& L = p.lev[l];
    int s0, s1;
    vc_slice(L.n, L.ch, rank, s0, s1);
    for (int i = s0 + (int)threadIdx.x; i < s1; i += blockDim.x) {
      vc_smem[L.off + (i - s0)] = __ldcg(L.e + i);
      vc_smem[L.off + 2 * L.ch + (i - s0)] = __ldcg(L.r + i);
    }
  }
  vc_sync();
  int cur_next = 0;   // buffer of the next coarser level's current e
  for (int l = p.lc - 1; l >= 0; --l) {
    const VcLevel& L = p.lev[l];
    const VcLevel& N = p.lev[l + 1];
    const bool from_dense = l + 1 == p.lc;
    int s0, s1;
    vc_slice(L.n, L.ch, rank, s0, s1);
    for (int i = s0 + (int)threadIdx.x; i < s1; i += blockDim.x) {
      const int j = L.up[i];
      const float en = from_dense ? __ldcg(N.e + j) : vc_get(vc_smem, N, cur_next, j);
      vc_smem[L.off + (i - s0)] += en;
    }
    vc_sync();
    int cur = 0;
    for (int it = 0; it < p.npost; ++it) {
      vc_sweep(L, vc_smem, cur, cur ^ 1, false, p.w, rank);
      cur ^= 1;
      vc_sync();
    }
    cur_next = cur;
    if (l == 0)
      for (int i = s0 + (int)threadIdx.x; i < s1; i += blockDim.x) L.e[i] = vc_smem[L.off + cur * L.ch + (i - s0)];
  }
}
