// Device kernels of libdgsip, part 2: right-hand side, DG<->CG transfers,
// SFC-level multigrid and the Krylov vector kernels (FP64).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dg_kernels.cuh"

namespace dg {

// ---------------------------------------------------------------------------
// boundary-face geometry for the right-hand side (Dirichlet / Neumann faces)
struct BFaceParams {
  Tables T;
  const double* x;       // (B, D, N)
  const int* elem;       // (nbf) element of each boundary face
  const int* face;       // (nbf) local face index
  double* sw;            // (nbf, SG) sdet * sweight
  double* gn;            // (nbf, N, SG) grad(phi).n
  double* gam;           // (nbf) eta / h
  double eta;
  int nbf;
};

template <int D, int N, int F, int SG>
__global__ void bface_geom_kernel(BFaceParams p) {
  const int k = blockIdx.x;       // boundary face
  const int tid = threadIdx.x;
  __shared__ double xe[D * N];
  __shared__ double ivs[SG][D * D];
  __shared__ double nrm[SG][D];
  __shared__ double swl[SG];
  const int e = p.elem[k], f = p.face[k];
  for (int i = tid; i < D * N; i += blockDim.x) xe[i] = p.x[(int64_t)e * D * N + i];
  __syncthreads();
  const double* snlx_f = p.T.snlx + (size_t)f * D * N * SG;
  for (int g = tid; g < SG; g += blockDim.x) {
    double j[D * D];
    jacobian<D, N>(snlx_f, SG, g, xe, j);
    inv_det<D>(j, ivs[g]);
    double sdet = face_normal<D>(j, p.T.drst + f * D * (D - 1), nrm[g]);
    swl[g] = sdet * p.T.sweight[g];
    p.sw[(int64_t)k * SG + g] = swl[g];
  }
  __syncthreads();
  for (int i = tid; i < N * SG; i += blockDim.x) {
    int n = i / SG, g = i % SG;
    double v = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double gi = 0.0;
#pragma unroll
      for (int b = 0; b < D; ++b) gi += ivs[g][a * D + b] * snlx_f[(b * N + n) * SG + g];
      v += gi * nrm[g][a];
    }
    p.gn[((int64_t)k * N + n) * SG + g] = v;
  }
  if (tid == 0) {
    double h = 0.0;
    for (int g = 0; g < SG; ++g) h += swl[g];
    if (D == 3) h = sqrt(h);
    p.gam[k] = p.eta / h;
  }
}

// b[e] = M_e f[e] (consistent mass, z06/volume_mf_diff.py:195-239)
template <int N, int VG, int EPB>
__global__ void rhs_mass_kernel(const double* __restrict__ nt, const double* __restrict__ detw,
                                const double* __restrict__ f, double* __restrict__ b, int64_t B) {
  __shared__ double fq[EPB][VG];
  __shared__ double fs[EPB][N];
  const int le = threadIdx.x / N, m = threadIdx.x % N;
  const int64_t e = (int64_t)blockIdx.x * EPB + le;
  const bool valid = e < B;
  if (valid) fs[le][m] = f[e * N + m];
  __syncthreads();
  for (int g = m; g < VG; g += N) {
    double s = 0.0;
    if (valid)
      for (int n = 0; n < N; ++n) s += nt[n * VG + g] * fs[le][n];
    fq[le][g] = valid ? s * detw[e * VG + g] : 0.0;
  }
  __syncthreads();
  if (!valid) return;
  double acc = 0.0;
  for (int g = 0; g < VG; ++g) acc += nt[m * VG + g] * fq[le][g];
  b[e * N + m] = acc;
}

// Dirichlet lifting (mode 0) or Neumann flux (mode 1) of the boundary faces
// with local face index fsel (z06/volume_mf_diff.py:242-359).  Faces of one
// local index never share an element, so the updates do not collide.
template <int N, int SG>
__global__ void rhs_bface_kernel(const double* __restrict__ sn_tab, const int* __restrict__ elem,
                                 const int* __restrict__ face, const int* __restrict__ type,
                                 const double* __restrict__ sw, const double* __restrict__ gn,
                                 const double* __restrict__ gam, const double* __restrict__ kappa,
                                 const double* __restrict__ g, double* __restrict__ b, int nbf,
                                 int fsel, int mode, double mu) {
  const int k = blockIdx.x * (blockDim.x / N) + threadIdx.x / N;
  const int m = threadIdx.x % N;
  if (k >= nbf) return;
  const int f = face[k];
  if (f != fsel || type[k] != mode) return;
  const int e = elem[k];
  const double* snf = sn_tab + (size_t)f * N * SG;
  double acc = 0.0;
  for (int q = 0; q < SG; ++q) {
    double gq = 0.0;
    for (int n = 0; n < N; ++n) gq += snf[n * SG + q] * g[(int64_t)e * N + n];
    double w = sw[(int64_t)k * SG + q];
    if (mode == 0)
      acc += (-gn[((int64_t)k * N + m) * SG + q] + gam[k] * snf[m * SG + q]) * gq * w;
    else
      acc += snf[m * SG + q] * gq * w;
  }
  if (mode == 0) acc *= mu * kappa[e];
  b[(int64_t)e * N + m] += acc;
}

// ---------------------------------------------------------------------------
// DG <-> CG P1 transfers (z06/volume_mf_diff.py:1961-1966, 2010-2013;
// multigrid_linearelastic.py:286-297; sparsity.py:125-165)

// out[pos(i)] = sum over DG copies (e, c) of vertex i of w_ec * sum_n P[n][c] r[e][n]
template <int N, int NC, typename T = double>
__global__ void restrict_cg_kernel(const T* __restrict__ r, const double* __restrict__ P,
                                   const int* __restrict__ gptr, const int* __restrict__ gent,
                                   const double* __restrict__ wdg, const int* __restrict__ pos,
                                   T* __restrict__ out, int ncg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncg) return;
  T acc = 0;
  for (int k = gptr[i]; k < gptr[i + 1]; ++k) {
    const int ent = gent[k];
    const int64_t e = ent / NC;
    const int c = ent % NC;
    T v = 0;
#pragma unroll
    for (int n = 0; n < N; ++n) v += (T)P[n * NC + c] * r[e * N + n];
    acc += (T)wdg[ent] * v;
  }
  out[pos ? pos[i] : i] = acc;
}

// out[pos(i)] = sum over DG copies (e, c) of vertex i of w_ec * r1[e][c],
// r1 the P3->P1 element restriction formed by the residual kernel
template <typename T>
__global__ void gather_cg_kernel(const T* __restrict__ r1, const int* __restrict__ gptr,
                                 const int* __restrict__ gent, const double* __restrict__ wdg,
                                 const int* __restrict__ pos, T* __restrict__ out, int ncg) {
  pdl_wait_then_trigger();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncg) return;
  T acc = 0;
  for (int k = gptr[i]; k < gptr[i + 1]; ++k) {
    const int ent = gent[k];
    acc += (T)wdg[ent] * r1[ent];
  }
  out[pos ? pos[i] : i] = acc;
}

// x[e][n] (+)= sum_c P[n][c] * w_ec * ecg[idx(p1cg[e][c])]; with whichc set,
// ecg is the indicator of colour `color` (colour-probe prolongation).
template <int N, int NC, typename T = double>
__global__ void prolong_cg_kernel(T* __restrict__ x, const T* __restrict__ ecg,
                                  const int* __restrict__ pos, const int* __restrict__ p1cg,
                                  const double* __restrict__ wdg, const double* __restrict__ P,
                                  const int* __restrict__ whichc, int color, int64_t B, int add) {
  pdl_wait_then_trigger();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * N) return;
  const int64_t e = t / N;
  const int n = t % N;
  T v = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int vtx = p1cg[e * NC + c];
    T ev;
    if (whichc)
      ev = whichc[vtx] == color ? (T)1 : (T)0;
    else
      ev = ecg[pos ? pos[vtx] : vtx];
    v += (T)P[n * NC + c] * ((T)wdg[e * NC + c] * ev);
  }
  x[t] = add ? x[t] + v : v;
}

// value[spidx[k]] += rarm[colidx[k]] for the probe entries of one colour
__global__ void rar_scatter_kernel(double* __restrict__ value, const double* __restrict__ rarm,
                                   const int* __restrict__ spidx, const int* __restrict__ colidx,
                                   int cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < cnt) value[spidx[k]] += rarm[colidx[k]];
}

// Direct Galerkin P1CG operator (the colour-probe result in one pass).
// G_b = P^T A_b P (NC x NC) for every stored block b, one warp per block:
// lanes m < N form row m of A_b P, then lanes < NC * NC the products with P^T.
template <int N, int NC>
__global__ void __launch_bounds__(128) block_galerkin_kernel(const double* __restrict__ blk,
                                                             const double* __restrict__ P,
                                                             double* __restrict__ G, int64_t nb) {
  constexpr int WPB = 4;
  __shared__ double Q[WPB][N][NC];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int64_t b = (int64_t)blockIdx.x * WPB + wi;
  if (b >= nb) return;   // whole warp
  const double* A = blk + b * N * N;   // A(m, n) at [n * N + m]
  if (lane < N) {
    double q[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) q[c] = 0.0;
    for (int n = 0; n < N; ++n) {
      const double a = A[n * N + lane];
#pragma unroll
      for (int c = 0; c < NC; ++c) q[c] = fma(a, P[n * NC + c], q[c]);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) Q[wi][lane][c] = q[c];
  }
  __syncwarp();
  if (lane < NC * NC) {
    const int a = lane / NC, c = lane % NC;
    double g = 0.0;
    for (int m = 0; m < N; ++m) g = fma(P[m * NC + a], Q[wi][m][c], g);
    G[b * NC * NC + lane] = g;
  }
}

// rar[k] = sum over the contribution list of nonzero k (dg_rap_contributions,
// packed block * 16 + a * 4 + c) of w(e, a) w(nb, c) G_block[a][c], in list
// order (deterministic)
__global__ void rap_gather_kernel(const double* __restrict__ G, const int* __restrict__ ptr,
                                  const int* __restrict__ ent, const double* __restrict__ wdg,
                                  const int* __restrict__ nbe, int F, int NC, double* __restrict__ rar,
                                  int64_t nnz) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  double s = 0.0;
  for (int t = ptr[k]; t < ptr[k + 1]; ++t) {
    const int v = ent[t];
    const int bid = v >> 4, a = (v >> 2) & 3, c = v & 3;
    const int e = bid / (F + 1), sl = bid % (F + 1);
    const int nb = sl == 0 ? e : nbe[e * F + sl - 1];
    s += wdg[e * NC + a] * wdg[nb * NC + c] * G[(int64_t)bid * NC * NC + a * NC + c];
  }
  rar[k] = s;
}

// ---------------------------------------------------------------------------
// SFC levels (multigrid_linearelastic.py:25-172)

// rr = b - A e_in;  e_out = e_in + w * rr / diag   (mg_smooth_one_level);
// e_in = NULL stands for a zero initial guess.
// LPR lanes share a row (strided over its entries, shuffle-reduced) so the
// dependent loads of a row are spread over lanes instead of chained.
constexpr int LPR = 8;
// explicit fused multiply-add (the cluster V-cycle repeats these operations
// bit for bit)
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
template <typename T = double>
__global__ void lev_jacobi_kernel(const int* __restrict__ rowptr, const int* __restrict__ col,
                                  const T* __restrict__ val, const T* __restrict__ diag,
                                  const T* __restrict__ e_in, const T* __restrict__ b,
                                  T* __restrict__ e_out, T* __restrict__ rr_out, int n,
                                  double w) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / LPR, lane = t % LPR;
  // the level matrix is fixed data: the first four entries of this lane are
  // read before the programmatic-launch wait, overlapping the previous kernel
  constexpr int PRE = 4;
  int k0 = 0, k1 = 0;
  int cpre[PRE];
  T vpre[PRE];
  if (i < n) {
    k0 = rowptr[i] + lane;
    k1 = rowptr[i + 1];
  }
#pragma unroll
  for (int q = 0; q < PRE; ++q) {
    const int k = k0 + q * LPR;
    cpre[q] = k < k1 ? col[k] : 0;
    vpre[q] = k < k1 ? val[k] : (T)0;
  }
  pdl_wait_then_trigger();
  T s = 0;
  if (i < n && e_in) {
#pragma unroll
    for (int q = 0; q < PRE; ++q)
      if (k0 + q * LPR < k1) s = fma_t(vpre[q], e_in[cpre[q]], s);
    for (int k = k0 + PRE * LPR; k < k1; k += LPR) s = fma_t(val[k], e_in[col[k]], s);
  }
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
  if (i >= n || lane != 0) return;
  const T rr = b[i] - s;
  e_out[i] = fma_t(rr / diag[i], (T)w, e_in ? e_in[i] : (T)0);
  if (rr_out) rr_out[i] = rr;
}

// pair sums with a zero pad (F.pad + Conv1d([1, 1], stride 2), :147-153)
template <typename T = double>
__global__ void lev_restrict_kernel(const T* __restrict__ rr, const T* __restrict__ e,
                                    T* __restrict__ r_next, T* __restrict__ e_next,
                                    int n, int nn) {
  pdl_wait_then_trigger();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const int a = 2 * i, b = 2 * i + 1;
  r_next[i] = rr[a] + (b < n ? rr[b] : (T)0);
  e_next[i] = e[a] + (b < n ? e[b] : (T)0);
}

// e_l[i] += e_next[up[i]]  (nn.Upsample nearest, :163-164)
template <typename T = double>
__global__ void lev_prolong_kernel(T* __restrict__ e, const T* __restrict__ e_next,
                                   const int* __restrict__ up, int n) {
  pdl_wait_then_trigger();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) e[i] += e_next[up[i]];
}

// coarsest level: one node, e = r / a (scipy spsolve on a 1x1 system, :157-160)
template <typename T = double>
__global__ void lev_coarse_kernel(const T* __restrict__ val, const T* __restrict__ r,
                                  T* __restrict__ e) {
  if (threadIdx.x == 0 && blockIdx.x == 0) e[0] = r[0] / val[0];
}

// ---------------------------------------------------------------------------
// Krylov vector kernels (deterministic fixed-grid reductions)
constexpr int KMAXV = 32;     // maximum number of basis vectors in one pass

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Per-thread accumulation type of the multi-dot / multi-axpy kernels: the
// vectors' own type (each thread sums ~n / (grid * TB) terms; the partial
// sums are combined in FP64).  FP32 vectors thus stay off the FP64 pipe.
template <int TB, typename VT = double>
__global__ void __launch_bounds__(TB) mdot2d_kernel(const VT* __restrict__ V, int64_t ld,
                                                    const VT* __restrict__ z, int64_t n,
                                                    double* __restrict__ partial) {
  __shared__ double red[TB / 32];
  const int i = blockIdx.y;
  const VT* Vi = V + (size_t)i * ld;
  VT acc = 0;
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n; k += (int64_t)gridDim.x * TB)
    acc += Vi[k] * z[k];
  double a = warp_sum((double)acc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += red[w];
    partial[(int64_t)blockIdx.x * KMAXV + i] = s;
  }
}

// z -= sum_i V[i] h[i] (any nv <= 256); with want_norm also partial[bx][0] = slice of |z_new|^2
template <int TB, typename VT = double>
__global__ void __launch_bounds__(TB) axpy_multi_kernel(const VT* __restrict__ V, int64_t ld, int nv,
                                                        const double* __restrict__ h, VT* __restrict__ z,
                                                        int64_t n, double* __restrict__ partial,
                                                        int want_norm) {
  __shared__ VT hs[256];
  __shared__ double red[TB / 32];
  for (int i = threadIdx.x; i < nv; i += TB) hs[i] = (VT)h[i];
  __syncthreads();
  VT acc = 0;
  for (int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x; k < n; k += (int64_t)gridDim.x * TB) {
    VT zk = z[k];
    // groups of 8 independent loads keep enough requests in flight
    for (int i0 = 0; i0 < nv; i0 += 8) {
      VT v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = (i0 + q < nv) ? V[(size_t)(i0 + q) * ld + k] : (VT)0;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (i0 + q < nv) zk -= v[q] * hs[i0 + q];
    }
    z[k] = zk;
    if (want_norm) acc += zk * zk;
  }
  if (!want_norm) return;
  double a = warp_sum((double)acc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TB / 32; ++w) s += red[w];
    partial[(int64_t)blockIdx.x * KMAXV] = s;
  }
}

// out[i] = (accumulate ? out[i] : 0) + sum_blk partial[blk][i]; optional
// sqrt.  One block per vector i (gridDim.x = nv), a fixed-order tree sum.
__global__ void reduce_partial_kernel(const double* __restrict__ partial, int nblk, int nv,
                                      double* __restrict__ out, int accumulate, int take_sqrt) {
  pdl_wait_then_trigger();
  __shared__ double red[32];
  const int i = blockIdx.x;
  if (i >= nv) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[(int64_t)b * KMAXV + i];
  s = warp_sum(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[w];
    if (take_sqrt) t = sqrt(t);
    out[i] = accumulate ? out[i] + t : t;
  }
}

// v = z / (*den): FP64 vectors divide (bitwise like the reference's
// w / h); other types multiply by the reciprocal formed once
template <typename VT = double>
__global__ void scale_kernel(const VT* __restrict__ z, const double* __restrict__ den,
                             VT* __restrict__ v, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  if constexpr (sizeof(VT) == 8) {
    v[k] = z[k] / (VT)(*den);
  } else {
    const VT inv = (VT)(1.0 / *den);
    v[k] = z[k] * inv;
  }
}

// x += alpha * sum_i V[i] y[i]
template <typename VT = double, typename XT = double>
__global__ void combine_kernel(const VT* __restrict__ V, int64_t ld, int nv,
                               const double* __restrict__ y, XT* __restrict__ x, int64_t n,
                               double alpha = 1.0) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s = 0.0;
  for (int i = 0; i < nv; ++i) s += (double)V[i * ld + k] * y[i];
  x[k] = (XT)((double)x[k] + alpha * s);
}

// the same for FP32 vectors in FP32 arithmetic (the inner solve's
// correction): y converted once per CTA, one FMA chain per entry (FP64
// arithmetic per entry would run at the FP64 pipe's rate)
__global__ void combine32_kernel(const float* __restrict__ V, int64_t ld, int nv, const double* __restrict__ y,
                                 float* __restrict__ x, int64_t n) {
  __shared__ float ys[256];   // nv <= 256 (the restart length limit of the mixed solve)
  for (int i = threadIdx.x; i < nv; i += blockDim.x) ys[i] = (float)y[i];
  __syncthreads();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = x[k];
  for (int i = 0; i < nv; ++i) s = fmaf(V[i * ld + k], ys[i], s);
  x[k] = s;
}

}  // namespace dg

namespace dg {

// ---------------------------------------------------------------------------
// Whole SFC V-cycle in one launch on a thread-block cluster.  Each CTA owns
// a contiguous slice of every level's rows; phases are separated by cluster
// barriers (the CTAs of a cluster are co-resident, so the barrier cannot
// wait on an unscheduled block).  Values written by other CTAs of the
// cluster are read with L2-coherent loads.  Semantics are those of
// vcycle() in the host driver (multigrid_linearelastic.py:112-172).
struct VLevel {
  const int* rowptr;
  const int* col;
  const double* val;
  const double* diag;
  const int* up;    // into the next coarser level (levels above the top)
  double* e;
  double* e2;
  double* r;
  double* rr;
  int n;
};

constexpr int VMAXLEV = 40;

struct VCycleParams {
  VLevel lev[VMAXLEV];
  int nlevel;
  int pre, post;
  double w;
  const double* r_in;   // level-0 right-hand side (curve order)
  double* e_out;        // level-0 result
};

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;\n" : "=r"(r));
  return r;
}

// rows [lo, hi) of a level owned by this CTA
__device__ __forceinline__ void slice(int n, unsigned rank, unsigned ncta, int& lo, int& hi) {
  long long per = ((long long)n + ncta - 1) / ncta;
  lo = (int)min((long long)n, per * rank);
  hi = (int)min((long long)n, per * (rank + 1));
}

__device__ __forceinline__ void vjacobi(const VLevel& L, const double* e_in, const double* b, double* e_out,
                                        double* rr_out, int lo, int hi, double w) {
  const int lane = threadIdx.x % LPR;
  const int groups = blockDim.x / LPR;
  // whole warps iterate together so the shuffles see converged lanes
  for (int base = lo; base < hi; base += groups) {
    const int i = base + (int)threadIdx.x / LPR;
    double s = 0.0;
    if (i < hi) {
      const int k1 = __ldg(L.rowptr + i + 1);
      for (int k = __ldg(L.rowptr + i) + lane; k < k1; k += LPR)
        s += __ldg(L.val + k) * __ldcg(e_in + __ldg(L.col + k));
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
    if (i < hi && lane == 0) {
      const double rr = __ldcg(b + i) - s;
      e_out[i] = __ldcg(e_in + i) + rr / __ldg(L.diag + i) * w;
      if (rr_out) rr_out[i] = rr;
    }
  }
}

__global__ void __launch_bounds__(1024) vcycle_cluster_kernel(VCycleParams p) {
  const unsigned rank = cluster_rank(), ncta = cluster_size();
  const int top = p.nlevel - 1;
  int lo, hi;
  // level 0 input, zero initial error
  {
    const VLevel& L = p.lev[0];
    slice(L.n, rank, ncta, lo, hi);
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      L.r[i] = __ldcg(p.r_in + i);
      L.e[i] = 0.0;
    }
  }
  cluster_barrier();
  for (int l = 0; l < top; ++l) {
    const VLevel& L = p.lev[l];
    slice(L.n, rank, ncta, lo, hi);
    double* ea = L.e;
    double* eb = L.e2;
    for (int it = 0; it < p.pre; ++it) {
      vjacobi(L, ea, L.r, eb, nullptr, lo, hi, p.w);
      cluster_barrier();
      double* t = ea; ea = eb; eb = t;
    }
    // the residual-forming smoothing call also updates e (reference quirk)
    vjacobi(L, ea, L.r, eb, L.rr, lo, hi, p.w);
    cluster_barrier();
    // the final error of this level lives in eb; remember it for the way up
    const VLevel& Nx = p.lev[l + 1];
    int clo, chi;
    slice(Nx.n, rank, ncta, clo, chi);
    for (int i = clo + threadIdx.x; i < chi; i += blockDim.x) {
      const int a = 2 * i, b2 = 2 * i + 1;
      Nx.r[i] = __ldcg(L.rr + a) + (b2 < L.n ? __ldcg(L.rr + b2) : 0.0);
      Nx.e[i] = __ldcg(eb + a) + (b2 < L.n ? __ldcg(eb + b2) : 0.0);
    }
    // copy the level's current error into L.e when it sits in e2
    if (eb != L.e)
      for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) L.e[i] = __ldcg(eb + i);
    cluster_barrier();
  }
  if (rank == 0 && threadIdx.x == 0) {
    const VLevel& T = p.lev[top];
    T.e[0] = __ldcg(T.r) / __ldg(T.val);
  }
  cluster_barrier();
  for (int l = top - 1; l >= 0; --l) {
    const VLevel& L = p.lev[l];
    const VLevel& Nx = p.lev[l + 1];
    slice(L.n, rank, ncta, lo, hi);
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) L.e[i] = __ldcg(L.e + i) + __ldcg(Nx.e + __ldg(L.up + i));
    cluster_barrier();
    double* ea = L.e;
    double* eb = L.e2;
    for (int it = 0; it < p.post; ++it) {
      vjacobi(L, ea, L.r, eb, nullptr, lo, hi, p.w);
      cluster_barrier();
      double* t = ea; ea = eb; eb = t;
    }
    if (ea != L.e) {
      for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) L.e[i] = __ldcg(ea + i);
      cluster_barrier();
    }
  }
  if (p.e_out) {
    const VLevel& L = p.lev[0];
    slice(L.n, rank, ncta, lo, hi);
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) p.e_out[i] = __ldcg(L.e + i);
  }
}

}  // namespace dg

namespace dg {

// ---------------------------------------------------------------------------
// Coarse tail of the SFC V-cycle in one CTA: levels l0 .. top (down sweeps,
// pair-sum restriction, the one-node solve, prolongation and up sweeps),
// separated by __syncthreads instead of kernel boundaries.  On entry level
// l0 holds its right-hand side r and initial error e (restricted from the
// level above); on exit its final error is in lev[l0].e.  All data stays in
// the L1/L2 of one SM, which is fast for the small levels (n <= a few
// thousand rows).  Same arithmetic as the per-level kernels.
template <typename T>
struct TLevel {
  const int* rowptr;
  const int* col;
  const T* val;
  const T* diag;
  const int* up;
  T* e;
  T* e2;
  T* r;
  T* rr;
  int n;
};

template <typename T>
struct TailParams {
  TLevel<T> lev[VMAXLEV];
  int l0, top;
  int pre, post;
  double w;
};

template <typename T>
__device__ __forceinline__ void tail_jacobi(const TLevel<T>& L, const T* e_in, T* e_out, T* rr_out, T w) {
  constexpr int TL = 4;   // lanes per row
  const int lane = threadIdx.x % TL;
  const int groups = blockDim.x / TL;
  for (int base = 0; base < L.n; base += groups) {
    const int i = base + (int)threadIdx.x / TL;
    T s = 0;
    if (i < L.n)
      for (int k = L.rowptr[i] + lane; k < L.rowptr[i + 1]; k += TL) s += L.val[k] * e_in[L.col[k]];
#pragma unroll
    for (int o = TL / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, TL);
    if (i < L.n && lane == 0) {
      const T rr = L.r[i] - s;
      e_out[i] = e_in[i] + rr / L.diag[i] * w;
      if (rr_out) rr_out[i] = rr;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) vcycle_tail_kernel(TailParams<T> p) {
  const T w = (T)p.w;
  for (int l = p.l0; l < p.top; ++l) {
    const TLevel<T>& L = p.lev[l];
    T* ea = L.e;
    T* eb = L.e2;
    for (int it = 0; it < p.pre; ++it) {
      tail_jacobi(L, ea, eb, (T*)nullptr, w);
      __syncthreads();
      T* t = ea; ea = eb; eb = t;
    }
    tail_jacobi(L, ea, eb, L.rr, w);     // the residual-forming call also updates e
    __syncthreads();
    const TLevel<T>& Nx = p.lev[l + 1];
    for (int i = threadIdx.x; i < Nx.n; i += blockDim.x) {
      const int a = 2 * i, b2 = 2 * i + 1;
      Nx.r[i] = L.rr[a] + (b2 < L.n ? L.rr[b2] : (T)0);
      Nx.e[i] = eb[a] + (b2 < L.n ? eb[b2] : (T)0);
    }
    if (eb != L.e)
      for (int i = threadIdx.x; i < L.n; i += blockDim.x) L.e[i] = eb[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const TLevel<T>& Tp = p.lev[p.top];
    Tp.e[0] = Tp.r[0] / Tp.val[0];
  }
  __syncthreads();
  for (int l = p.top - 1; l >= p.l0; --l) {
    const TLevel<T>& L = p.lev[l];
    const TLevel<T>& Nx = p.lev[l + 1];
    for (int i = threadIdx.x; i < L.n; i += blockDim.x) L.e[i] = L.e[i] + Nx.e[L.up[i]];
    __syncthreads();
    T* ea = L.e;
    T* eb = L.e2;
    for (int it = 0; it < p.post; ++it) {
      tail_jacobi(L, ea, eb, (T*)nullptr, w);
      __syncthreads();
      T* t = ea; ea = eb; eb = t;
    }
    if (ea != L.e) {
      for (int i = threadIdx.x; i < L.n; i += blockDim.x) L.e[i] = ea[i];
      __syncthreads();
    }
  }
}

}  // namespace dg
