// libdgsip: context, operator assembly, preconditioner and GMRES drivers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "dg_internal.h"
#include "dg_kernels.cuh"
#include "dg_kernels2.cuh"

using namespace dg;

namespace {

constexpr int RED_TB = 256;
constexpr int kBatchedVariants = 7;   // batched smoothing kernel variants (see dg_ctx::batched_kernel)
std::atomic<long long> g_launches{0};   // kernels launched by this library
inline void bump(long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

struct DevLevel {
  int n = 0;
  // fixed summation lists of the level values (after the first build): entry
  // d = sum of rar[vk[j]] over j in [vptr[d], vptr[d+1]) in that order;
  // didx[i] = entry of row i's diagonal or -1
  int nnz = 0;
  int* vptr = nullptr;
  int* vk = nullptr;
  int* didx = nullptr;
  // coarse levels (long lists: one device thread would sum thousands of
  // values in sequence) keep their lists on the host and are summed there
  bool host_sum = false;
  std::vector<int> h_vptr, h_vk, h_didx;
  int* rowptr = nullptr;
  int* col = nullptr;
  double* val = nullptr;
  double* diag = nullptr;
  int* up = nullptr;        // for levels below the top: index into the next level
  double* e = nullptr;      // error
  double* e2 = nullptr;     // ping-pong buffer
  double* r = nullptr;      // right-hand side on this level
  double* rr = nullptr;     // residual scratch
};

}  // namespace

// most DG-level smoothing steps per leg of the mixed preconditioner with
// their own damping factor (Chebyshev roots or DG_MIXED_OMEGAS)
constexpr int kMaxSmoothSteps = 8;
// default smoothing steps per leg of the mixed preconditioner (c2: 2 / 3 / 4
// / 5 / 6 / 8 steps with their best Chebyshev interval took 20.6 / 17.0 /
// 14.0 / 13.8 / 14.1 / 15.3 ms at 78 / 54 / 38 / 33 / 30 / 27 inner steps;
// c3: 2 / 4 / 5 / 6 steps 161 / 114 / 107 / 115 ms)
constexpr int kMixedChebSteps = 5;
// ... and of the batched preconditioner, whose inner steps carry more fixed
// work (per-RHS Gram-Schmidt, FP32 apply on CUDA cores, FP64 residuals):
// c4 with 4 / 5 / 6 steps and ratio 32 / 64 / 128 took 213 / 196 / 166 ms
// per 64 solves at 40 / 33 / 25 inner steps
constexpr int kBatchedChebSteps = 6;

struct dg_ctx {
  int dev = 0;
  int D = 0, N = 0, F = 0, NC = 0, VG = 0, SG = 0;
  int64_t B = 0, nonods = 0, ncg = 0;
  dg_config cfg{};
  std::string err;
  int nsm = 0;
  // host copies
  std::vector<int64_t> p1cg, sfc;      // (B*NC), (ncg) 1-based
  std::vector<double> kappa;
  int face_kappa = 0;   // interior-face kappa: 0 arithmetic mean (reference), 1 harmonic mean
  std::vector<int> bf_elem, bf_face, bf_type;
  // device allocations (released in dg_destroy)
  std::vector<void*> allocs;
  int64_t dev_bytes = 0;   // sum of the allocations in allocs (freed only by dg_destroy)
  double* d_x = nullptr;
  int *d_nbe = nullptr, *d_nbface = nullptr, *d_aln = nullptr, *d_bct = nullptr;
  // shared-face tables of the reduced-precision copies (3D): d_fref5[e][j]
  // addresses slot j of element e in the shared block array (2 * block + 1
  // when read transposed, -1 on the boundary); d_sfsrc[i] = FP64 source
  // block of shared block i; nface_sh = interior faces
  int *d_fref5 = nullptr, *d_sfsrc = nullptr;
  // reference matrices of the affine block build; fast_build: -1 not yet
  // checked, 1 all elements straight-sided, 0 otherwise (quadrature build).
  // general_build (default): every element through the isoparametric
  // Jacobian at each quadrature point, the reference's own formula -- the
  // FP64 solve then stays within 1e-13 of the reference's solution on the
  // pinned cases (the affine build moves the 2D 32x32 case to 1.6e-12);
  // dg_set_build_mode(ctx, 1) selects the affine build (~3.4x faster, equal
  // to rounding) for per-request rebuilds
  double* d_ftab = nullptr;
  int fast_build = -1;
  bool general_build = true;
  // direct Galerkin P1CG operator from the blocks (default; DG_RAP_DIRECT=0
  // restores one FP64 apply per colour of the distance-2 colouring):
  // contribution lists (dg_rap_contributions, packed) and the per-block
  // products.  Equal to the probe operator within 4e-16 relative on the
  // golden cases and c2; operator build at 280k tets 106 -> 82 ms.
  bool rap_direct = true;
  int *d_rap_ptr = nullptr, *d_rap_ent = nullptr;
  double* d_rap_G = nullptr;
  int64_t nface_sh = 0;
  double* d_kappa = nullptr;
  Tables T{};
  double* d_blk = nullptr;
  double* d_W = nullptr;        // (B, N, N) smoother matrices
  double* d_detw = nullptr;
  int* d_err = nullptr;
  // boundary faces for the right-hand side
  int nbf = 0;
  int *d_bf_elem = nullptr, *d_bf_face = nullptr, *d_bf_type = nullptr;
  double *d_bf_sw = nullptr, *d_bf_gn = nullptr, *d_bf_gam = nullptr;
  // P1CG
  std::vector<int64_t> fina, cola, whichc;
  int32_t ncolor = 0;
  std::vector<std::vector<int64_t>> spidx, colidx;
  int *d_p1cg = nullptr, *d_gptr = nullptr, *d_gent = nullptr, *d_pos = nullptr, *d_whichc = nullptr;
  double* d_wdg = nullptr;
  // FP32 copies of wdg and of the P1 -> P3 table for the reduced-precision
  // kernels: an FP64 -> FP32 conversion per use costs FP64-pipe throughput
  float* d_wdg32 = nullptr;
  float* d_P32 = nullptr;
  int *d_spidx = nullptr, *d_colidx = nullptr;
  std::vector<int64_t> sp_off;
  double* d_rar = nullptr;
  std::vector<double> rar_host;
  // SFC levels (device) and the host copy of the hierarchy
  std::vector<DevLevel> lev;
  SfcHierarchy sfc_h;
  // scratch
  double *d_t1 = nullptr, *d_t2 = nullptr, *d_t3 = nullptr, *d_t4 = nullptr, *d_t5 = nullptr;
  double *d_cg1 = nullptr, *d_cg2 = nullptr;
  double* d_r1 = nullptr;   // (nele, ncorner) element P1 restriction scratch
  // Krylov
  double* d_V = nullptr;
  int vcap = 0;
  double *d_part = nullptr, *d_h1 = nullptr, *d_h2 = nullptr, *d_H = nullptr, *d_y = nullptr,
         *d_scal = nullptr;
  int nred = 0;
  bool built = false;
  // SFC V-cycle as one thread-block-cluster kernel (0 = per-level launches)
  int vc_cluster = 0;
  // levels with at most this many rows run in the one-CTA tail kernel
  int tail_max64 = 320, tail_max32 = 800;
  // mixed preconditioner: exact (dense inverse) solve on the first SFC level
  // with at most this many rows (0 = keep the V-cycle to the one-node level)
  int dense_max32 = 2400;
  int dense_n = 0;
  // mixed preconditioner reads BF16 copies of the blocks / smoother matrices
  bool precond_bf16 = true;
  // ... streamed by the persistent bulk-copy (TMA) kernel (3D)
  bool bf16_tma = true;
  // FP32 operator copy (3D) in the chunked layout, read by the bulk-copy kernel
  bool f32_tma = true;
  // bulk-copy block streams read with an L2 evict-first policy
  bool l2_hint = true;
  // store each interior face block once in the reduced-precision copies
  // (c2: DRAM bytes of the BF16 step 238 -> 161 MB and of the FP32 apply
  // 385 -> 235 MB, but 37.5 -> 49 us and 59 -> 70 us: the transposed reads
  // are column reads from shared memory; kept as an option)
  bool shared_faces = false;
  // mixed preconditioner: DG-level smoothing steps before / after the coarse
  // correction and Jacobi sweeps on the SFC levels (-1 = the configured
  // pre_smooth_its, as in the FP64 preconditioner)
  int mixed_sweeps = -1, mixed_lev_sweeps = -1;
  // FP32 SFC V-cycle legs of the mixed preconditioner as thread-block-
  // cluster launches: -1 = the largest cluster (16, else 8) that the device
  // schedules, 0 = the launch chain (default: measured faster at c2),
  // 8 / 16 = that cluster size (dg_set_vcycle_cluster, DG_MIXED_VC_CLUSTER)
  int vc32_cluster = 0;
  // dense coarse inverse of the mixed preconditioner by the one-pivot FP64
  // Gauss-Jordan (DG_DENSE_FP64=1) instead of the blocked FP32 form
  bool dense_fp64 = false;
  // the launch chain of that V-cycle without launches of its own for the
  // transfers between levels (vcycle32_fused; DG_MIXED_VC_FUSED=0: off)
  bool vc32_fused = true;
  // mixed preconditioner with 2 to 4 DG-level smoothing steps: step k damped
  // by mixed_smooth_w * mixed_wscale[k] (pre-smoothing k = 0, 1, ...;
  // post-smoothing in reverse), a Chebyshev polynomial smoother of that
  // degree whose factors are set at each mixed build from an estimate of
  // lambda_max(A_ee^-1 A) (set_smoother_schedule); one step takes the
  // uniform damping w
  float mixed_wscale[kMaxSmoothSteps] = {1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.0f};
  double smoother_lmax = 0.0;
  // beta = margin x the estimated lambda_max (c2: margin 1.05 / 1.1 / 1.2
  // -> 80 / 84 / 88 inner steps; c3: 94 / 94 / 106); a larger margin keeps
  // the polynomial below 1 further past an underestimated lambda_max
  double cheb_margin = 1.05;
  // the Chebyshev interval is [beta / cheb_ratio, beta] (c2 / c3 with 5 steps:
  // ratio 32 / 64 / 128 -> 37 / 34 / 33 and - / 36 / - inner steps; with 2
  // steps the ratio 8 of the first schedule).  With host checks every 3
  // steps, ratio 128 gave c2 12.88 ms (30 steps) and c3 99.3 ms (33) against
  // 13.26 / 104.9 ms, but on a 2D case (64^2 x 2 triangles) the inner steps
  // then moved from 64 to 81 with a rounding-level change of the coarse
  // inverse; 64 keeps them within 2
  double cheb_ratio = 64.0;
  // the batched preconditioner's schedule: steps per leg (-1 = kBatchedChebSteps,
  // or DG_MIXED_SWEEPS when that is set) and Chebyshev interval ratio
  int batched_sweeps = -1;
  double cheb_ratio_b = 128.0;
  bool omegas_set = false;   // DG_MIXED_OMEGAS given: its factors, for any step count
  // mixed inner FGMRES: per-step convergence test on the device, chunk
  // graphs with one conditional node per step (c2: 100 -> 98 inner steps,
  // but 30.5 -> 31.4 ms: the stops land where the chunk checks already did
  // and the per-step nodes cost ~15 us; kept as an option)
  bool cond_graph = false;
  // inner Arnoldi steps per captured graph; the host checks the
  // least-squares residual after each, so a refinement step runs at most
  // chunk - 1 steps past its target (c2 with the Chebyshev smoothing:
  // chunk 10 / 5 / 4 / 3 -> 90 / 85 / 80 / 81 steps, 27.4 / 25.9 / 24.6 /
  // 25.0 ms; c3: chunk 10 / 5 -> 212 / 202 ms)
  // (with the adaptive cut below, c2: chunk 4 / 5 / 6 / 8 -> 24.73 / 24.61 /
  // 24.51 / 24.78 ms at 80 / 80 / 80 / 81 steps; with the 5-step Chebyshev
  // smoothing, ~8 inner steps per refinement step: chunk 2 / 3 / 4 / 6 / 8
  // -> 13.18 / 13.10 / 13.46 / 14.25 / 14.94 ms, c3: chunk 3 / 6 -> 103.9 /
  // 106.6 ms)
  int mixed_chunk = 3;
  // cut a chunk that would run past the inner target to the step count the
  // observed convergence rate predicts (its remaining steps run as direct
  // launches); DG_ADAPTIVE_CHUNK=0 keeps whole chunks.  c2: 84 -> 80 steps
  // (25.86 -> 24.73 ms) with the quadrature build, c3: 94 -> 90 (201 ->
  // 192 ms); whole chunks stop up to chunk - 1 steps past the target, so
  // the step count jumped with rounding-level changes of the operator
  bool adaptive_chunk = true;
  // link the kernels of an inner Arnoldi step by programmatic dependent launch
  bool use_pdl = true;
  // batched solve: BF16 preconditioner steps on the tensor cores (mma.sync)
  bool batched_mma = true;
  // ... through the persistent bulk-copy form (c2, 64 RHS: 0.63 s per 64
  // solves vs 0.57 s for one CTA per element, whose 5 CTAs per SM hide more
  // of the per-element latency; kept as a tuning option)
  bool batched_tma = false;
  int batched_warps = 4;   // warps per CTA of the per-element batched smoothing kernel (4 or 8)
  // batched BF16 smoothing kernel variant (bsmooth): 0 CUDA cores, 1 / 2
  // mma.sync per element (4 / 8 warps), 3 mma.sync persistent bulk-copy, 4
  // tcgen05 persistent bulk-copy, 5 tcgen05 on split x, 6 the same
  // warp-specialized; chosen by timing at the first batched
  // solve of each mixed build unless pinned (DG_BATCHED_KERNEL or the older
  // DG_BATCHED_MMA / _TMA / _WARPS switches)
  int batched_kernel = 1;
  // batched Gram-Schmidt with one thread per (row lane, RHS) (bmdot2 /
  // baxpy2); DG_BATCHED_GS2=0 keeps the float4 forms
  bool batched_gs2 = true;
  bool batched_pinned = false;
  int tma_variant = 0;   // elements per group / stages / CTAs per SM of that kernel
  bool autotune = true;  // pick tma_variant by timing at the first mixed solve after a build
  // mixed preconditioner (3D, BF16 bulk-copy path): smoothing steps after
  // the zero-start one read the face blocks scaled by the smoother,
  // S_ef = W_e A_ef, and c = W b (no self block, no smoother matrix)
  bool scaled_faces = true;
  int sc_variant = 0;    // launch shape of that kernel (autotuned with tma_variant)
  bool sc_pinned = false;   // sc_variant set by DG_SCALED_VARIANT: not autotuned
  bool verbose = false;
  // mixed preconditioner smoother: 0 = the reference's three point-Jacobi
  // sweeps, 1 = damped exact block inverse w_b * A_ee^{-1}
  int mixed_smoother = 1;
  double mixed_smooth_w = 0.8;
  // Gram-Schmidt passes of the FP32 inner Arnoldi (1 = classical GS with
  // FP64 partial sums; 2 = CGS2).  One pass: the FP64 refinement bounds the
  // result, and c2 / c3 need the same inner iterations either way.
  int mixed_cgs_passes = 1;
  // Gram-Schmidt of the inner Arnoldi with the reductions fused into the
  // last CTA of the dot and update kernels (3 launches per step instead of
  // 5); measured slower on c2 (25.9 -> 26.9 ms per solve: the last CTA's
  // reduction of ~940 partials is a serial tail), so off by default
  bool gs_fused = false;
  // orthogonalisation of the FP64 GMRES Arnoldi step: 0 = CGS2 (two classical
  // passes, 2 reductions per step), 1 = modified Gram-Schmidt in the
  // reference's order (z06/volume_mf_diff.py:1814-1819; j + 1 dependent
  // dot / update pairs per step)
  int gmres_ortho = 0;
  // captured Arnoldi cycle (GMRES(m) inner loop) replayed as one CUDA graph
  bool use_graph = true;
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t arnoldi_exec = nullptr;
  int arnoldi_m = 0;
  int arnoldi_ortho = 0;
  const double* arnoldi_vptr = nullptr;
  // mixed-precision state (dg_mixed.cuh) and operator versions
  void* mixed_state = nullptr;
  int build_version = 0;
  // operator build whose FP64 smoother matrices d_W are current (built on
  // first use: only the FP64 smoothing reads them)
  int w_version = -1;
  // the SFC level structure and summation lists are on the device: later
  // builds form the level values there (no RAR download, host sums, upload)
  bool lev_maps_ready = false;
  double* rar_pinned = nullptr;   // pinned host copy of the Galerkin values (host-summed levels)
  // geometry record of the affine build (GeomRec), formed once per context;
  // geom_ok once a build that formed it passed the Jacobian check
  double* d_geom = nullptr;
  bool geom_ok = false;
  int mixed_version = -1;
  long long arnoldi_kernels = 0;   // kernels in the captured Arnoldi cycle graph
};

namespace {

int fail(dg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  set_thread_error(code, msg);
  return code;
}

#define CK(ctx, call)                                                                    \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess)                                                               \
      return fail((ctx), DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define CKL(ctx) CK(ctx, cudaGetLastError())

template <typename T>
int dalloc(dg_ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return fail(c, DG_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back((void*)*p);
  c->dev_bytes += (int64_t)(count * sizeof(T));
  return DG_OK;
}

template <typename T>
int upload(dg_ctx* c, T** p, const T* src, size_t count) {
  int rc = dalloc(c, p, count);
  if (rc) return rc;
  if (count) CK(c, cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return DG_OK;
}

template <typename T>
int upload_vec(dg_ctx* c, T** p, const std::vector<T>& v) {
  return upload(c, p, v.data(), v.size());
}

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline unsigned nblk(int64_t n, int tb) { return (unsigned)((n + tb - 1) / tb); }

// ---------------------------------------------------------------------------
// template dispatch on the element type
template <int D>
struct Elem;
template <>
struct Elem<3> {
  static constexpr int N = 20, F = 4, VG = 24, SG = 12, NC = 4, EPB = 8;
};
template <>
struct Elem<2> {
  static constexpr int N = 10, F = 3, VG = 12, SG = 4, NC = 3, EPB = 16;
};

// SFC level values from the Galerkin values: entry d is the sum of
// rar[vk[j]] for j in [vptr[d], vptr[d+1]), left to right (the host
// builder's order); diag[i] = the value of row i's diagonal entry (0 if none)
__global__ void sfc_level_values_kernel(const double* __restrict__ rar, const int* __restrict__ vptr,
                                        const int* __restrict__ vk, int nnz, double* __restrict__ val) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nnz) return;
  const int j0 = vptr[d], j1 = vptr[d + 1];
  double s = rar[vk[j0]];
  for (int j = j0 + 1; j < j1; ++j) s += rar[vk[j]];
  val[d] = s;
}

__global__ void sfc_level_diag_kernel(const double* __restrict__ val, const int* __restrict__ didx, int n,
                                      double* __restrict__ diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diag[i] = didx[i] >= 0 ? val[didx[i]] : 0.0;
}

template <int D>
int launch_build(dg_ctx* c, cudaStream_t st) {
  using E = Elem<D>;
  using Sm = BuildSmem<D, E::N, E::F, E::VG, E::SG>;
  BuildParams p;
  p.T = c->T;
  p.x = c->d_x;
  p.nbe = c->d_nbe;
  p.nbface = c->d_nbface;
  p.aln = c->d_aln;
  p.bct = c->d_bct;
  p.kappa = c->d_kappa;
  p.blk = c->d_blk;
  p.detw = c->d_detw;
  p.eta = c->cfg.eta_e;
  p.mu = c->cfg.mu_f;
  p.B = c->B;
  p.err = c->d_err;
  p.face_kappa = c->face_kappa;
  if (c->fast_build < 0 && c->B > 0) {
    // straight-sided elements (constant Jacobian) take the table build;
    // decided once, the coordinates are fixed for the context
    unsigned long long* dv = nullptr;
    int rc;
    if ((rc = dalloc(c, &dv, 1))) return rc;
    CK(c, cudaMemsetAsync(dv, 0, sizeof(unsigned long long), st));
    affine_check_kernel<D, E::N, E::VG><<<nblk(c->B, 128), 128, 0, st>>>(c->d_x, c->T.nlx, c->B, dv);
    bump();
    unsigned long long hv = 0;
    CK(c, cudaMemcpyAsync(&hv, dv, sizeof(hv), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    double rel;
    std::memcpy(&rel, &hv, sizeof(rel));
    c->fast_build = rel < 1e-10 ? 1 : 0;
    if (c->verbose) std::fprintf(stderr, "[dg_build_operator] Jacobian variation %.3e: %s build\n", rel,
                                 c->fast_build ? "affine" : "quadrature");
  }
  if (c->fast_build == 1 && !c->general_build && c->d_ftab) {
    using GR = GeomRec<D, E::F>;
    if (!c->geom_ok) {   // kappa-free geometry, once per context (again after a failed build)
      int rc;
      if (!c->d_geom && (rc = dalloc(c, &c->d_geom, (size_t)std::max<int64_t>(c->B, 1) * GR::Size))) return rc;
      if (c->B > 0) geom_affine_kernel<D, E::N, E::F, E::VG, E::SG><<<nblk(c->B, 128), 128, 0, st>>>(p, c->d_geom);
      bump();
      CKL(c);
    }
    if (c->B > 0)
      build_blocks_affine_kernel<D, E::N, E::F, E::VG, E::SG><<<(unsigned)c->B, E::N * E::N, 0, st>>>(p, c->d_ftab,
                                                                                                   c->d_geom);
  } else {
    auto k = build_blocks_kernel<D, E::N, E::F, E::VG, E::SG>;
    CK(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm)));
    if (c->B > 0) k<<<(unsigned)c->B, E::N * E::N, sizeof(Sm), st>>>(p);
  }
  bump();
  CKL(c);
  if (c->nbf > 0) {
    BFaceParams q;
    q.T = c->T;
    q.x = c->d_x;
    q.elem = c->d_bf_elem;
    q.face = c->d_bf_face;
    q.sw = c->d_bf_sw;
    q.gn = c->d_bf_gn;
    q.gam = c->d_bf_gam;
    q.eta = c->cfg.eta_e;
    q.nbf = c->nbf;
    bface_geom_kernel<D, E::N, E::F, E::SG><<<c->nbf, 64, 0, st>>>(q);
    bump();
    CKL(c);
  }
  return DG_OK;
}

// The reference's three-sweep Jacobi smoother matrices W_e of the current
// operator build (FP64): formed on first use, since only the FP64 smoothing
// reads them (the mixed preconditioner's default smoother is its own block
// inverse).
template <int D>
int ensure_w64_t(dg_ctx* c, cudaStream_t st) {
  using E = Elem<D>;
  if (c->w_version == c->build_version) return DG_OK;
  if (c->B > 0)
    smoother_matrix_kernel<E::N, E::F><<<(unsigned)c->B, E::N * E::N, 0, st>>>(c->d_blk, c->d_W, c->B,
                                                                             c->cfg.jac_wei);
  bump();
  CKL(c);
  c->w_version = c->build_version;
  return DG_OK;
}

int ensure_w64(dg_ctx* c, cudaStream_t st) { return c->D == 3 ? ensure_w64_t<3>(c, st) : ensure_w64_t<2>(c, st); }

template <int D>
int launch_residual(dg_ctx* c, const double* x, const double* b, double* r, double* x_out, int flags,
                    cudaStream_t st, double* r1) {
  using E = Elem<D>;
  if (flags & RF_SMOOTH) {
    int rc;
    if ((rc = ensure_w64_t<D>(c, st))) return rc;
  }
  unsigned g = nblk(c->B, E::EPB);
  if (g) residual_kernel<E::N, E::F, E::EPB><<<g, E::EPB * E::N, 0, st>>>(
      c->d_blk, c->d_W, c->d_nbe, x, b, r, x_out, c->B, flags, c->T.P, r1);
  bump();
  CKL(c);
  return DG_OK;
}

// flags RF_*; with RF_RESTRICT, r1 (nele, ncorner) receives the P3->P1
// element restriction of the residual (not combined with RF_SMOOTH)
int residual(dg_ctx* c, const double* x, const double* b, double* r, double* x_out, int flags,
             cudaStream_t st, double* r1 = nullptr) {
  return c->D == 3 ? launch_residual<3>(c, x, b, r, x_out, flags, st, r1)
                   : launch_residual<2>(c, x, b, r, x_out, flags, st, r1);
}

// vertex gather of the element restrictions r1 (curve order when sfc_order)
template <typename T>
int gather_cg(dg_ctx* c, const T* r1, T* out, bool sfc_order, cudaStream_t st) {
  gather_cg_kernel<T><<<nblk(c->ncg, 128), 128, 0, st>>>(r1, c->d_gptr, c->d_gent, c->d_wdg,
                                                         sfc_order ? c->d_pos : nullptr, out, (int)c->ncg);
  bump();
  CKL(c);
  return DG_OK;
}

template <int D>
int launch_restrict(dg_ctx* c, const double* r, double* out, bool sfc_order, cudaStream_t st) {
  using E = Elem<D>;
  restrict_cg_kernel<E::N, E::NC><<<nblk(c->ncg, 128), 128, 0, st>>>(
      r, c->T.P, c->d_gptr, c->d_gent, c->d_wdg, sfc_order ? c->d_pos : nullptr, out, (int)c->ncg);
  bump();
  CKL(c);
  return DG_OK;
}

int restrict_cg(dg_ctx* c, const double* r, double* out, bool sfc_order, cudaStream_t st) {
  return c->D == 3 ? launch_restrict<3>(c, r, out, sfc_order, st) : launch_restrict<2>(c, r, out, sfc_order, st);
}

template <int D>
int launch_prolong(dg_ctx* c, double* x, const double* ecg, bool sfc_order, int color, bool add,
                   cudaStream_t st) {
  using E = Elem<D>;
  prolong_cg_kernel<E::N, E::NC><<<nblk(c->B * E::N, 256), 256, 0, st>>>(
      x, ecg, sfc_order ? c->d_pos : nullptr, c->d_p1cg, c->d_wdg, c->T.P,
      color > 0 ? c->d_whichc : nullptr, color, c->B, add ? 1 : 0);
  bump();
  CKL(c);
  return DG_OK;
}

int prolong_cg(dg_ctx* c, double* x, const double* ecg, bool sfc_order, int color, bool add, cudaStream_t st) {
  return c->D == 3 ? launch_prolong<3>(c, x, ecg, sfc_order, color, add, st)
                   : launch_prolong<2>(c, x, ecg, sfc_order, color, add, st);
}

// First SFC level handled by the one-CTA tail kernel (<= top; == top means
// only the one-node solve).  Levels above it use per-level launches.
int tail_start(const dg_ctx* c, int tail_max) {
  const int nl = (int)c->lev.size();
  if (nl > VMAXLEV) return nl - 1;
  for (int l = 0; l < nl; ++l)
    if (c->lev[l].n <= tail_max) return std::max(l, 0);
  return nl - 1;
}

// Pick the cluster size for the one-launch V-cycle (16 if the device can
// co-schedule it, else 8, else 0 = fall back to per-level launches).
void choose_vcycle_cluster(dg_ctx* c) {
  c->vc_cluster = 0;
  if ((int)c->lev.size() > VMAXLEV) return;
  // Default off: inside the captured GMRES cycle the per-level launches
  // (~0.9 us apart) beat the one-launch cluster V-cycle, whose row sweeps on
  // 16 SMs are latency-bound.  DG_VCYCLE_CLUSTER=16|8 selects it.
  const char* env = std::getenv("DG_VCYCLE_CLUSTER");
  int want[2] = {0, 0};
  if (env && env[0]) want[0] = std::atoi(env);
  cudaFuncSetAttribute(vcycle_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  for (int cs : want) {
    if (cs <= 0) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs, 1, 1);
    cfg.blockDim = dim3(1024, 1, 1);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, vcycle_cluster_kernel, &cfg) == cudaSuccess && nclusters > 0) {
      c->vc_cluster = cs;
      break;
    }
    cudaGetLastError();
  }
}

int vcycle_cluster(dg_ctx* c, const double* r_sfc, cudaStream_t st) {
  VCycleParams p;
  p.nlevel = (int)c->lev.size();
  for (int l = 0; l < p.nlevel; ++l) {
    const DevLevel& L = c->lev[l];
    p.lev[l] = VLevel{L.rowptr, L.col, L.val, L.diag, L.up, L.e, L.e2, L.r, L.rr, L.n};
  }
  p.pre = c->cfg.pre_smooth_its;
  p.post = c->cfg.post_smooth_its;
  p.w = c->cfg.jac_wei;
  p.r_in = r_sfc;
  p.e_out = nullptr;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c->vc_cluster, 1, 1);
  cfg.blockDim = dim3(1024, 1, 1);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = c->vc_cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(c, cudaLaunchKernelEx(&cfg, vcycle_cluster_kernel, p));
  bump();
  return DG_OK;
}

// One SFC V-cycle; r_sfc is level-0 input, result left in lev[0].e
int vcycle(dg_ctx* c, const double* r_sfc, cudaStream_t st) {
  if (c->vc_cluster > 0) {
    if (c->lev.back().n != 1) return fail(c, DG_ERR_STATE, "coarsest SFC level must hold one node");
    return vcycle_cluster(c, r_sfc, st);
  }
  const int nl = (int)c->lev.size();
  const int top = nl - 1;
  const double w = c->cfg.jac_wei;
  const int TB = 128;
  const int l0 = tail_start(c, c->tail_max64);
  CK(c, cudaMemcpyAsync(c->lev[0].r, r_sfc, sizeof(double) * c->lev[0].n, cudaMemcpyDeviceToDevice, st));
  CK(c, cudaMemsetAsync(c->lev[0].e, 0, sizeof(double) * c->lev[0].n, st));
  for (int l = 0; l < std::min(l0, top); ++l) {
    DevLevel& L = c->lev[l];
    for (int it = 0; it < c->cfg.pre_smooth_its; ++it) {
      lev_jacobi_kernel<double><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e, L.r,
                                                                      L.e2, nullptr, L.n, w); bump();
      std::swap(L.e, L.e2);
    }
    // the residual-forming call also updates e in place (reference quirk)
    lev_jacobi_kernel<double><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e, L.r,
                                                                    L.e2, L.rr, L.n, w); bump();
    std::swap(L.e, L.e2);
    DevLevel& Nx = c->lev[l + 1];
    lev_restrict_kernel<double><<<nblk(Nx.n, TB), TB, 0, st>>>(L.rr, L.e, Nx.r, Nx.e, L.n, Nx.n); bump();
  }
  if (c->lev[top].n != 1) return fail(c, DG_ERR_STATE, "coarsest SFC level must hold one node");
  if (l0 < top) {
    TailParams<double> tp;
    tp.l0 = l0;
    tp.top = top;
    tp.pre = c->cfg.pre_smooth_its;
    tp.post = c->cfg.post_smooth_its;
    tp.w = w;
    for (int l = 0; l < nl; ++l) {
      const DevLevel& L = c->lev[l];
      tp.lev[l] = TLevel<double>{L.rowptr, L.col, L.val, L.diag, L.up, L.e, L.e2, L.r, L.rr, L.n};
    }
    vcycle_tail_kernel<double><<<1, 1024, 0, st>>>(tp);
    bump();
  } else {
    DevLevel& L = c->lev[top];
    lev_coarse_kernel<double><<<1, 32, 0, st>>>(L.val, L.r, L.e); bump();
  }
  for (int l = std::min(l0, top) - 1; l >= 0; --l) {
    DevLevel& L = c->lev[l];
    lev_prolong_kernel<double><<<nblk(L.n, TB), TB, 0, st>>>(L.e, c->lev[l + 1].e, L.up, L.n); bump();
    for (int it = 0; it < c->cfg.post_smooth_its; ++it) {
      lev_jacobi_kernel<double><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag, L.e, L.r,
                                                                      L.e2, nullptr, L.n, w); bump();
      std::swap(L.e, L.e2);
    }
  }
  CKL(c);
  return DG_OK;
}

// z = M^{-1} r.  Scratch: t3, t4 (smoother iterates), t5 (residual); z and r
// must be distinct and not among those.
int precond(dg_ctx* c, const double* r, double* z, cudaStream_t st) {
  int rc;
  const int nsm = c->cfg.pre_smooth_its;
  double* cur = c->d_t3;
  double* other = c->d_t4;
  // pre-smoothing from x = 0: the first sweep needs no operator apply
  if (nsm > 0) {
    if ((rc = residual(c, nullptr, r, nullptr, cur, RF_ZEROX | RF_SMOOTH, st))) return rc;
    for (int it = 1; it < nsm; ++it) {
      if ((rc = residual(c, cur, r, nullptr, other, RF_SMOOTH, st))) return rc;
      std::swap(cur, other);
    }
  } else {
    CK(c, cudaMemsetAsync(cur, 0, sizeof(double) * c->nonods, st));
  }
  // residual restricted to P1 per element, gathered to P1CG in curve order,
  // V-cycle, prolongation
  if ((rc = residual(c, cur, r, nullptr, nullptr, RF_RESTRICT, st, c->d_r1))) return rc;
  if ((rc = gather_cg<double>(c, c->d_r1, c->d_cg1, true, st))) return rc;
  if ((rc = vcycle(c, c->d_cg1, st))) return rc;
  if ((rc = prolong_cg(c, cur, c->lev[0].e, true, 0, true, st))) return rc;
  // post-smoothing (the reference repeats pre_smooth_its times, :2021)
  for (int it = 0; it < nsm; ++it) {
    double* out = (it == nsm - 1) ? z : other;
    if ((rc = residual(c, cur, r, nullptr, out, RF_SMOOTH, st))) return rc;
    other = cur;
    cur = out;
  }
  if (nsm == 0) CK(c, cudaMemcpyAsync(z, cur, sizeof(double) * c->nonods, cudaMemcpyDeviceToDevice, st));
  return DG_OK;
}

int ensure_krylov(dg_ctx* c, int m) {
  if (c->vcap >= m + 1) return DG_OK;
  int rc;
  if ((rc = dalloc(c, &c->d_V, (size_t)(m + 1) * c->nonods))) return rc;
  if ((rc = dalloc(c, &c->d_H, (size_t)(m + 1) * m))) return rc;
  c->vcap = m + 1;
  return DG_OK;
}

// h[0..nv) = V[0..nv)^T z (FP64 accumulation; chunks of KMAXV vectors)
template <typename VT>
int mdot_t(dg_ctx* c, const VT* V, int nv, const VT* z, double* h, cudaStream_t st) {
  for (int off = 0; off < nv; off += KMAXV) {
    int cnt = std::min(KMAXV, nv - off);
    dim3 grid(c->nred, cnt);
    mdot2d_kernel<RED_TB, VT><<<grid, RED_TB, 0, st>>>(V + (size_t)off * c->nonods, c->nonods, z, c->nonods,
                                                       c->d_part);
    bump();
    reduce_partial_kernel<<<cnt, 128, 0, st>>>(c->d_part, c->nred, cnt, h + off, 0, 0);
    bump();
  }
  CKL(c);
  return DG_OK;
}

int mdot(dg_ctx* c, const double* V, int nv, const double* z, double* h, int accumulate, cudaStream_t st) {
  (void)accumulate;
  return mdot_t<double>(c, V, nv, z, h, st);
}

// Norm of z into *out (device)
template <typename VT>
int norm_t(dg_ctx* c, const VT* z, double* out, cudaStream_t st) {
  dim3 grid(c->nred, 1);
  mdot2d_kernel<RED_TB, VT><<<grid, RED_TB, 0, st>>>(z, c->nonods, z, c->nonods, c->d_part);
  bump();
  reduce_partial_kernel<<<1, 128, 0, st>>>(c->d_part, c->nred, 1, out, 0, 1);
  bump();
  CKL(c);
  return DG_OK;
}

int norm2(dg_ctx* c, const double* z, double* out, cudaStream_t st) { return norm_t<double>(c, z, out, st); }

// CGS2 step: h1 = V^T z, z -= V h1, h2 = V^T z, z -= V h2 (with |z|^2);
// H column j = h1 + h2, H[j+1][j] = |z|, V[j+1] = z / |z|.
template <typename VT>
int cgs2_t(dg_ctx* c, VT* Vbase, double* Hbase, int j, VT* z, int m, cudaStream_t st) {
  const int nv = j + 1;
  double* Hc = Hbase + (size_t)j * (m + 1);     // column-major (m+1) x m
  int rc;
  if ((rc = mdot_t<VT>(c, Vbase, nv, z, c->d_h1, st))) return rc;
  axpy_multi_kernel<RED_TB, VT><<<c->nred, RED_TB, 0, st>>>(Vbase, c->nonods, nv, c->d_h1, z, c->nonods, c->d_part, 0);
  bump();
  if ((rc = mdot_t<VT>(c, Vbase, nv, z, c->d_h2, st))) return rc;
  axpy_multi_kernel<RED_TB, VT><<<c->nred, RED_TB, 0, st>>>(Vbase, c->nonods, nv, c->d_h2, z, c->nonods, c->d_part, 1);
  bump();
  reduce_partial_kernel<<<1, 128, 0, st>>>(c->d_part, c->nred, 1, Hc + nv, 0, 1);
  bump();
  CK(c, cudaMemcpyAsync(Hc, c->d_h1, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
  for (int off = 0; off < nv; off += KMAXV) {
    int cnt = std::min(KMAXV, nv - off);
    reduce_partial_kernel<<<cnt, 32, 0, st>>>(c->d_h2 + off, 1, cnt, Hc + off, 1, 0);
    bump();
  }
  scale_kernel<VT><<<nblk(c->nonods, 256), 256, 0, st>>>(z, Hc + nv, Vbase + (size_t)nv * c->nonods, c->nonods);
  bump();
  CKL(c);
  return DG_OK;
}

int cgs2(dg_ctx* c, int j, double* z, int m, cudaStream_t st) { return cgs2_t<double>(c, c->d_V, c->d_H, j, z, m, st); }

// Modified Gram-Schmidt step in the reference's order
// (z06/volume_mf_diff.py:1814-1819): for i = 0..j, H[i][j] = z . V[i] then
// z -= H[i][j] V[i]; H[j+1][j] = |z|, V[j+1] = z / |z|.
int mgs(dg_ctx* c, int j, double* z, int m, cudaStream_t st) {
  const int nv = j + 1;
  double* Hc = c->d_H + (size_t)j * (m + 1);
  for (int i = 0; i < nv; ++i) {
    const double* Vi = c->d_V + (size_t)i * c->nonods;
    mdot2d_kernel<RED_TB, double><<<dim3(c->nred, 1), RED_TB, 0, st>>>(Vi, c->nonods, z, c->nonods, c->d_part);
    bump();
    reduce_partial_kernel<<<1, 128, 0, st>>>(c->d_part, c->nred, 1, Hc + i, 0, 0);
    bump();
    axpy_multi_kernel<RED_TB, double><<<c->nred, RED_TB, 0, st>>>(Vi, c->nonods, 1, Hc + i, z, c->nonods,
                                                                   c->d_part, i == j ? 1 : 0);
    bump();
  }
  reduce_partial_kernel<<<1, 128, 0, st>>>(c->d_part, c->nred, 1, Hc + nv, 0, 1);
  bump();
  scale_kernel<double><<<nblk(c->nonods, 256), 256, 0, st>>>(z, Hc + nv, c->d_V + (size_t)nv * c->nonods, c->nonods);
  bump();
  CKL(c);
  return DG_OK;
}

// The m Arnoldi steps of one GMRES cycle (V[0] already set): w = A v_j,
// r = M^-1 w, CGS2 against V[0..j], V[j+1] = r / ||r||.
int arnoldi_steps(dg_ctx* c, int m, cudaStream_t st) {
  int rc;
  double* r = c->d_t1;
  double* w = c->d_t2;
  for (int j = 0; j < m; ++j) {
    if ((rc = residual(c, c->d_V + (size_t)j * c->nonods, nullptr, w, nullptr, RF_NEG, st))) return rc;
    if ((rc = precond(c, w, r, st))) return rc;
    if ((rc = c->gmres_ortho == 1 ? mgs(c, j, r, m, st) : cgs2(c, j, r, m, st))) return rc;
  }
  return DG_OK;
}

int run_arnoldi(dg_ctx* c, int m, cudaStream_t st) {
  if (!c->use_graph) return arnoldi_steps(c, m, st);
  if (!c->arnoldi_exec || c->arnoldi_m != m || c->arnoldi_vptr != c->d_V || c->arnoldi_ortho != c->gmres_ortho) {
    if (c->arnoldi_exec) {
      cudaGraphExecDestroy(c->arnoldi_exec);
      c->arnoldi_exec = nullptr;
    }
    if (!c->cap_stream) CK(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    CK(c, cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    const long long k0 = g_launches.load();
    int rc = arnoldi_steps(c, m, c->cap_stream);
    c->arnoldi_kernels = g_launches.load() - k0;
    g_launches.fetch_sub(c->arnoldi_kernels);   // captured, counted per replay below
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(c->cap_stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ee != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
    cudaError_t ie = cudaGraphInstantiate(&c->arnoldi_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    c->arnoldi_m = m;
    c->arnoldi_vptr = c->d_V;
    c->arnoldi_ortho = c->gmres_ortho;
  }
  CK(c, cudaGraphLaunch(c->arnoldi_exec, st));
  bump(c->arnoldi_kernels);
  return DG_OK;
}

// least squares min || beta e1 - H y || by Givens rotations (host, FP64)
bool solve_hessenberg(const std::vector<double>& Hcm, int m, double beta, std::vector<double>& y) {
  // Hcm column-major (m+1) x m
  std::vector<double> R((size_t)(m + 1) * m);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i <= m; ++i) R[(size_t)i * m + j] = Hcm[(size_t)j * (m + 1) + i];
  std::vector<double> g(m + 1, 0.0);
  g[0] = beta;
  for (int j = 0; j < m; ++j) {
    double a = R[(size_t)j * m + j], b = R[(size_t)(j + 1) * m + j];
    double r = std::hypot(a, b);
    if (r == 0.0) return false;
    double cs = a / r, sn = b / r;
    for (int k = j; k < m; ++k) {
      double t1 = R[(size_t)j * m + k], t2 = R[(size_t)(j + 1) * m + k];
      R[(size_t)j * m + k] = cs * t1 + sn * t2;
      R[(size_t)(j + 1) * m + k] = -sn * t1 + cs * t2;
    }
    double g1 = g[j], g2 = g[j + 1];
    g[j] = cs * g1 + sn * g2;
    g[j + 1] = -sn * g1 + cs * g2;
  }
  y.assign(m, 0.0);
  for (int i = m - 1; i >= 0; --i) {
    double s = g[i];
    for (int k = i + 1; k < m; ++k) s -= R[(size_t)i * m + k] * y[k];
    if (R[(size_t)i * m + i] == 0.0) return false;
    y[i] = s / R[(size_t)i * m + i];
  }
  return true;
}

int read_scalar(dg_ctx* c, const double* d, double* h, cudaStream_t st) {
  CK(c, cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  return DG_OK;
}

}  // namespace

#include "dg_mixed.cuh"
#include "dg_batched.cuh"

// ===========================================================================
extern "C" {

long long dg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char* dg_last_error(const dg_ctx* ctx) {
  if (ctx) return ctx->err.c_str();
  return g_thread_error.c_str();
}

void dg_destroy(dg_ctx* ctx) {
  if (!ctx) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(ctx->dev);
  if (ctx->arnoldi_exec) cudaGraphExecDestroy(ctx->arnoldi_exec);
  destroy_mixed(ctx);
  if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
  if (ctx->rar_pinned) cudaFreeHost(ctx->rar_pinned);
  for (void* p : ctx->allocs) cudaFree(p);
  cudaSetDevice(cur);
  delete ctx;
}

int dg_info(const dg_ctx* ctx, int64_t* out, int32_t nout) {
  if (!ctx || !out) return set_thread_error(DG_ERR_ARG, "dg_info: null argument");
  const bool sf = ctx->D == 3 && ctx->shared_faces && ctx->d_fref5 && ctx->f32_tma && ctx->bf16_tma &&
                  ctx->precond_bf16;
  const bool sc = ctx->scaled_faces && ctx->D == 3 && ctx->precond_bf16 && ctx->bf16_tma && !sf &&
                  ctx->mixed_smoother == 1;
  int64_t v[19] = {ctx->D, ctx->N, ctx->B, ctx->nonods, ctx->ncg, (int64_t)ctx->cola.size(), ctx->ncolor,
                   (int64_t)ctx->lev.size(), ctx->nbf, ctx->built ? 1 : 0, ctx->VG, ctx->SG, ctx->tma_variant,
                   ctx->batched_kernel == 3 ? 1 : 0, sf ? ctx->nface_sh : 0, ctx->batched_kernel, sc ? 1 : 0,
                   ctx->sc_variant, ctx->dev_bytes};
  for (int i = 0; i < nout && i < 19; ++i) out[i] = v[i];
  return DG_OK;
}

int dg_create(const dg_mesh_desc* m, const dg_config* cfg, dg_ctx** out) {
  if (!m || !cfg || !out) return set_thread_error(DG_ERR_ARG, "dg_create: null argument");
  *out = nullptr;
  const int D = m->ndim;
  if (D != 2 && D != 3) return set_thread_error(DG_ERR_ARG, "dg_create: ndim must be 2 or 3");
  const int N = D == 3 ? 20 : 10, F = D + 1, VG = D == 3 ? 24 : 12, SG = D == 3 ? 12 : 4;
  if (m->nloc != N || m->ngi != VG || m->sngi != SG)
    return set_thread_error(DG_ERR_ARG, "dg_create: only P3 elements with degree-6 quadrature are supported");
  if (m->nele <= 0 || m->cg_nonods <= 0 || !m->x_ref_in || !m->nbf || !m->alnmt || !m->glb_bcface_type ||
      !m->p1cg || !m->sfc_order || !m->n || !m->nlx || !m->weight || !m->sn || !m->snlx || !m->sweight ||
      !m->gi_align || !m->drst_duv || !m->p1_to_p3)
    return set_thread_error(DG_ERR_ARG, "dg_create: missing mesh array");
  if (m->nele * (int64_t)N > (int64_t)INT32_MAX / 2)
    return set_thread_error(DG_ERR_ARG, "dg_create: mesh too large for 32-bit element indexing");
  std::unique_ptr<dg_ctx> c(new dg_ctx());
  c->dev = cfg->device;
  c->cfg = *cfg;
  c->D = D; c->N = N; c->F = F; c->NC = D + 1; c->VG = VG; c->SG = SG;
  c->B = m->nele;
  c->nonods = c->B * N;
  c->ncg = m->cg_nonods;
  CK(c.get(), cudaSetDevice(c->dev));
  cudaDeviceProp prop;
  CK(c.get(), cudaGetDeviceProperties(&prop, c->dev));
  c->nsm = prop.multiProcessorCount;
  {
    const char* t64 = std::getenv("DG_TAIL_MAX64");
    const char* t32 = std::getenv("DG_TAIL_MAX32");
    if (t64 && t64[0]) c->tail_max64 = std::atoi(t64);
    if (t32 && t32[0]) c->tail_max32 = std::atoi(t32);
    const char* dm = std::getenv("DG_DENSE_MAX32");
    if (dm && dm[0]) c->dense_max32 = std::atoi(dm);
    const char* vb = std::getenv("DG_VERBOSE");
    c->verbose = vb && vb[0] && vb[0] != '0';
    const char* ms = std::getenv("DG_MIXED_SMOOTHER");
    if (ms && ms[0]) c->mixed_smoother = std::atoi(ms);
    const char* mw = std::getenv("DG_MIXED_SMOOTH_W");
    if (mw && mw[0]) c->mixed_smooth_w = std::atof(mw);
    const char* pb = std::getenv("DG_PRECOND_BF16");
    if (pb && pb[0]) c->precond_bf16 = pb[0] != '0';
    const char* bt = std::getenv("DG_BF16_TMA");
    if (bt && bt[0]) c->bf16_tma = bt[0] != '0';
    const char* ft = std::getenv("DG_F32_TMA");
    if (ft && ft[0]) c->f32_tma = ft[0] != '0';
    const char* bt2 = std::getenv("DG_BATCHED_TMA");
    if (bt2 && bt2[0]) c->batched_tma = bt2[0] != '0';
    const char* bw = std::getenv("DG_BATCHED_WARPS");
    if (bw && bw[0]) c->batched_warps = std::atoi(bw) == 8 ? 8 : 4;
    const char* bm = std::getenv("DG_BATCHED_MMA");
    if (bm && bm[0]) c->batched_mma = bm[0] != '0';
    if (bt2 || bw || bm) {
      if ((bt2 && bt2[0]) || (bw && bw[0]) || (bm && bm[0])) {
        c->batched_kernel = !c->batched_mma ? 0 : (c->batched_tma ? 3 : (c->batched_warps == 8 ? 2 : 1));
        c->batched_pinned = true;
      }
    }
    const char* bk = std::getenv("DG_BATCHED_KERNEL");
    if (bk && bk[0]) {
      c->batched_kernel = std::min(std::max(std::atoi(bk), 0), kBatchedVariants - 1);
      c->batched_pinned = true;
    }
    const char* pd = std::getenv("DG_PDL");
    if (pd && pd[0]) c->use_pdl = pd[0] != '0';
    const char* lh = std::getenv("DG_L2_HINT");
    if (lh && lh[0]) c->l2_hint = lh[0] != '0';
    const char* sf = std::getenv("DG_SHARED_FACES");
    if (sf && sf[0]) c->shared_faces = sf[0] != '0';
    const char* rd = std::getenv("DG_RAP_DIRECT");
    if (rd && rd[0]) c->rap_direct = rd[0] != '0';
    const char* gb = std::getenv("DG_BUILD_GENERAL");
    if (gb && gb[0]) c->general_build = gb[0] != '0';
    const char* cmg = std::getenv("DG_CHEB_MARGIN");
    if (cmg && cmg[0]) c->cheb_margin = std::max(1.0, std::atof(cmg));
    const char* bsw = std::getenv("DG_BATCHED_SWEEPS");
    if (bsw && bsw[0]) c->batched_sweeps = std::atoi(bsw);
    const char* bcr = std::getenv("DG_BATCHED_CHEB_RATIO");
    if (bcr && bcr[0]) c->cheb_ratio_b = std::max(1.5, std::atof(bcr));
    const char* crt = std::getenv("DG_CHEB_RATIO");
    if (crt && crt[0]) c->cheb_ratio = std::max(1.5, std::atof(crt));
    const char* mch = std::getenv("DG_MIXED_CHUNK");
    if (mch && mch[0]) c->mixed_chunk = std::max(1, std::atoi(mch));
    const char* cg = std::getenv("DG_COND_GRAPH");
    if (cg && cg[0]) c->cond_graph = cg[0] != '0';
    const char* om = std::getenv("DG_MIXED_OMEGAS");   // absolute damping per step, "w0,w1,..."
    if (om && om[0]) {
      c->omegas_set = true;
      for (float& v : c->mixed_wscale) v = 1.0f;
      const char* q = om;
      for (int k = 0; k < kMaxSmoothSteps && *q; ++k) {
        char* end = nullptr;
        const double v = std::strtod(q, &end);
        if (end == q) break;
        c->mixed_wscale[k] = (float)(v / c->mixed_smooth_w);
        q = (*end == ',') ? end + 1 : end;
      }
    }
    const char* msw = std::getenv("DG_MIXED_SWEEPS");
    if (msw && msw[0]) c->mixed_sweeps = std::atoi(msw);
    const char* mlw = std::getenv("DG_MIXED_LEV_SWEEPS");
    if (mlw && mlw[0]) c->mixed_lev_sweeps = std::atoi(mlw);
    const char* dfp = std::getenv("DG_DENSE_FP64");
    if (dfp && dfp[0]) c->dense_fp64 = dfp[0] != '0';
    const char* vcc = std::getenv("DG_MIXED_VC_CLUSTER");
    if (vcc && vcc[0]) c->vc32_cluster = std::atoi(vcc);
    const char* vcf = std::getenv("DG_MIXED_VC_FUSED");
    if (vcf && vcf[0]) c->vc32_fused = vcf[0] != '0';
    const char* tv = std::getenv("DG_TMA_VARIANT");
    if (tv && tv[0]) {
      c->tma_variant = std::atoi(tv);
      c->autotune = false;
    }
    const char* scf = std::getenv("DG_SCALED_FACES");
    if (scf && scf[0]) c->scaled_faces = scf[0] != '0';
    const char* scv = std::getenv("DG_SCALED_VARIANT");
    if (scv && scv[0]) {
      c->sc_variant = std::atoi(scv);
      c->sc_pinned = true;
    }
    const char* at = std::getenv("DG_AUTOTUNE");
    if (at && at[0]) c->autotune = at[0] != '0';
    const char* bg = std::getenv("DG_BATCHED_GS2");
    if (bg && bg[0]) c->batched_gs2 = bg[0] != '0';
    const char* ac = std::getenv("DG_ADAPTIVE_CHUNK");
    if (ac && ac[0]) c->adaptive_chunk = ac[0] != '0';
    const char* gf = std::getenv("DG_GS_FUSED");
    if (gf && gf[0]) c->gs_fused = gf[0] != '0';
    const char* mc = std::getenv("DG_MIXED_CGS");
    if (mc && mc[0]) c->mixed_cgs_passes = std::atoi(mc) == 1 ? 1 : 2;
  }
  {
    const char* ng = std::getenv("DG_NO_GRAPH");
    c->use_graph = !(ng && ng[0] && ng[0] != '0');
  }
  c->nred = 2 * c->nsm;
  const int64_t nf = c->B * F;
  // face arrays
  std::vector<int> nbe(nf), nbface(nf), aln(nf), bct(nf);
  for (int64_t k = 0; k < nf; ++k) {
    int64_t t = m->glb_bcface_type[k];
    int64_t nb = m->nbf[k];
    bct[k] = (int)t;
    aln[k] = (int)std::max<int64_t>(m->alnmt[k], 0);
    if (t < 0) {
      if (nb < 0 || nb >= nf)
        return fail(c.get(), DG_ERR_MESH, "interior face without a neighbour (untagged boundary face)");
      if (m->alnmt[k] < 0 || m->alnmt[k] >= D)
        return fail(c.get(), DG_ERR_MESH, "interior face with an invalid alignment code");
      nbe[k] = (int)(nb / F);
      nbface[k] = (int)(nb % F);
    } else {
      nbe[k] = -1;
      nbface[k] = 0;
      if (t == 0 || t == 1) {
        c->bf_elem.push_back((int)(k / F));
        c->bf_face.push_back((int)(k % F));
        c->bf_type.push_back((int)t);
      }
    }
  }
  c->nbf = (int)c->bf_elem.size();
  c->p1cg.assign(m->p1cg, m->p1cg + c->B * c->NC);
  c->sfc.assign(m->sfc_order, m->sfc_order + c->ncg);
  for (int64_t v : c->p1cg)
    if (v < 0 || v >= c->ncg) return fail(c.get(), DG_ERR_MESH, "p1cg vertex out of range");
  int rc;
  if ((rc = upload(c.get(), &c->d_x, m->x_ref_in, (size_t)c->B * D * N))) return rc;
  if ((rc = upload_vec(c.get(), &c->d_nbe, nbe))) return rc;
  if ((rc = upload_vec(c.get(), &c->d_nbface, nbface))) return rc;
  if (D == 3) {
    // shared-face tables: an interior face belongs to its lower-numbered
    // element; the tables are left out (five-block copies only) unless every
    // face pair is reciprocal
    std::vector<int> fref5((size_t)c->B * (F + 1), -1), sfsrc((size_t)c->B), fid(nf, -1);
    bool ok = (int64_t)c->B * (F + 1) * 4 < (int64_t)INT32_MAX;
    for (int64_t e = 0; e < c->B; ++e) {
      sfsrc[e] = (int)(e * (F + 1));
      fref5[e * (F + 1)] = (int)(2 * e);
    }
    for (int64_t k = 0; ok && k < nf; ++k) {
      const int64_t e = k / F, nb = nbe[k];
      if (nb < 0) continue;
      const int64_t kb = nb * F + nbface[k];
      if (nb == e || nbe[kb] != e || nbface[kb] != (int)(k % F)) ok = false;
      else if (e < nb) {
        fid[k] = (int)(sfsrc.size() - c->B);
        sfsrc.push_back((int)(e * (F + 1) + 1 + k % F));
      }
    }
    for (int64_t k = 0; ok && k < nf; ++k) {
      const int64_t e = k / F, nb = nbe[k];
      if (nb < 0) continue;
      const int64_t own = e < nb ? k : nb * F + nbface[k];
      fref5[e * (F + 1) + 1 + k % F] = (int)(2 * (c->B + fid[own]) + (e < nb ? 0 : 1));
    }
    if (ok) {
      c->nface_sh = (int64_t)sfsrc.size() - c->B;
      if ((rc = upload_vec(c.get(), &c->d_fref5, fref5))) return rc;
      if ((rc = upload_vec(c.get(), &c->d_sfsrc, sfsrc))) return rc;
    }
  }
  if ((rc = upload_vec(c.get(), &c->d_aln, aln))) return rc;
  if ((rc = upload_vec(c.get(), &c->d_bct, bct))) return rc;
  c->kappa.assign(c->B, 1.0);
  if ((rc = upload_vec(c.get(), &c->d_kappa, c->kappa))) return rc;
  // element tables
  {
    double* p;
    if ((rc = upload(c.get(), &p, m->n, (size_t)N * VG))) return rc;
    c->T.n = p;
    if ((rc = upload(c.get(), &p, m->nlx, (size_t)D * N * VG))) return rc;
    c->T.nlx = p;
    if ((rc = upload(c.get(), &p, m->weight, (size_t)VG))) return rc;
    c->T.weight = p;
    if ((rc = upload(c.get(), &p, m->sn, (size_t)F * N * SG))) return rc;
    c->T.sn = p;
    if ((rc = upload(c.get(), &p, m->snlx, (size_t)F * D * N * SG))) return rc;
    c->T.snlx = p;
    if ((rc = upload(c.get(), &p, m->sweight, (size_t)SG))) return rc;
    c->T.sweight = p;
    if ((rc = upload(c.get(), &p, m->drst_duv, (size_t)F * D * (D - 1)))) return rc;
    c->T.drst = p;
    if ((rc = upload(c.get(), &p, m->p1_to_p3, (size_t)N * (D + 1)))) return rc;
    c->T.P = p;
    std::vector<float> p32(m->p1_to_p3, m->p1_to_p3 + (size_t)N * (D + 1));
    if ((rc = upload_vec(c.get(), &c->d_P32, p32))) return rc;
    std::vector<int> al(D * SG);
    for (int k = 0; k < D * SG; ++k) {
      if (m->gi_align[k] < 0 || m->gi_align[k] >= SG) return fail(c.get(), DG_ERR_ARG, "gi_align out of range");
      al[k] = (int)m->gi_align[k];
    }
    int* q;
    if ((rc = upload_vec(c.get(), &q, al))) return rc;
    c->T.align = q;
    // reference matrices of the straight-sided (affine) block build, entry
    // (m, n) of each N x N matrix at [m * N + n]: K[jj][kk], R[f][jj], Mf[f],
    // Q[f][fn][al][jj], P[f][fn][al][jj], S[f][fn][al] (see
    // build_blocks_affine_kernel)
    const int NN = N * N;
    const int nK = D * D, nR = F * D, nM = F, nQ = F * F * D * D, nS = F * F * D;
    std::vector<double> ft((size_t)(nK + nR + nM + 2 * nQ + nS) * NN, 0.0);
    double* tK = ft.data();
    double* tR = tK + (size_t)nK * NN;
    double* tM = tR + (size_t)nR * NN;
    double* tQ = tM + (size_t)nM * NN;
    double* tP = tQ + (size_t)nQ * NN;
    double* tS = tP + (size_t)nQ * NN;
    auto nlx = [&](int jj, int n, int g) { return m->nlx[(jj * N + n) * VG + g]; };
    auto sn = [&](int f, int n, int g) { return m->sn[(f * N + n) * SG + g]; };
    auto snlx = [&](int f, int jj, int n, int g) { return m->snlx[(size_t)f * D * N * SG + (jj * N + n) * SG + g]; };
    for (int jj = 0; jj < D; ++jj)
      for (int kk = 0; kk < D; ++kk)
        for (int a = 0; a < N; ++a)
          for (int b = 0; b < N; ++b) {
            double t = 0.0;
            for (int g = 0; g < VG; ++g) t += m->weight[g] * nlx(jj, a, g) * nlx(kk, b, g);
            tK[(size_t)(jj * D + kk) * NN + a * N + b] = t;
          }
    for (int f = 0; f < F; ++f)
      for (int a = 0; a < N; ++a)
        for (int b = 0; b < N; ++b) {
          double t = 0.0;
          for (int g = 0; g < SG; ++g) t += m->sweight[g] * sn(f, a, g) * sn(f, b, g);
          tM[(size_t)f * NN + a * N + b] = t;
          for (int jj = 0; jj < D; ++jj) {
            double r = 0.0;
            for (int g = 0; g < SG; ++g) r += m->sweight[g] * sn(f, a, g) * snlx(f, jj, b, g);
            tR[(size_t)(f * D + jj) * NN + a * N + b] = r;
          }
        }
    for (int f = 0; f < F; ++f)
      for (int fn = 0; fn < F; ++fn)
        for (int lg = 0; lg < D; ++lg) {
          const int cmb = (f * F + fn) * D + lg;
          for (int a = 0; a < N; ++a)
            for (int b = 0; b < N; ++b) {
              double ts = 0.0;
              for (int g = 0; g < SG; ++g) ts += m->sweight[g] * sn(f, a, g) * sn(fn, b, al[lg * SG + g]);
              tS[(size_t)cmb * NN + a * N + b] = ts;
              for (int jj = 0; jj < D; ++jj) {
                double tq = 0.0, tp = 0.0;
                for (int g = 0; g < SG; ++g) {
                  const int ag = al[lg * SG + g];
                  tq += m->sweight[g] * sn(f, a, g) * snlx(fn, jj, b, ag);
                  tp += m->sweight[g] * snlx(f, jj, a, g) * sn(fn, b, ag);
                }
                tQ[(size_t)(cmb * D + jj) * NN + a * N + b] = tq;
                tP[(size_t)(cmb * D + jj) * NN + a * N + b] = tp;
              }
            }
        }
    double* dft;
    if ((rc = upload_vec(c.get(), &dft, ft))) return rc;
    c->d_ftab = dft;
  }
  if ((rc = dalloc(c.get(), &c->d_blk, (size_t)c->B * (F + 1) * N * N))) return rc;
  if ((rc = dalloc(c.get(), &c->d_W, (size_t)c->B * N * N))) return rc;
  if ((rc = dalloc(c.get(), &c->d_detw, (size_t)c->B * VG))) return rc;
  if ((rc = dalloc(c.get(), &c->d_err, 1))) return rc;
  CK(c.get(), cudaMemset(c->d_err, 0, sizeof(int)));
  if (c->nbf) {
    if ((rc = upload_vec(c.get(), &c->d_bf_elem, c->bf_elem))) return rc;
    if ((rc = upload_vec(c.get(), &c->d_bf_face, c->bf_face))) return rc;
    if ((rc = upload_vec(c.get(), &c->d_bf_type, c->bf_type))) return rc;
    if ((rc = dalloc(c.get(), &c->d_bf_sw, (size_t)c->nbf * SG))) return rc;
    if ((rc = dalloc(c.get(), &c->d_bf_gn, (size_t)c->nbf * N * SG))) return rc;
    if ((rc = dalloc(c.get(), &c->d_bf_gam, (size_t)c->nbf))) return rc;
  }
  // P1CG sparsity, colours, probe indices, transfer lists
  if ((rc = p1cg_sparsity(c->B, c->NC, c->p1cg.data(), c->ncg, c->fina, c->cola)))
    return fail(c.get(), rc, g_thread_error);
  if ((rc = color2(c->ncg, c->fina.data(), c->cola.data(), c->whichc, c->ncolor)))
    return fail(c.get(), rc, g_thread_error);
  sparse_idx_for_color(c->ncg, c->fina.data(), c->cola.data(), c->whichc, c->ncolor, c->spidx, c->colidx);
  {
    std::vector<int> sp, ci;
    c->sp_off.assign(1, 0);
    for (int k = 0; k < c->ncolor; ++k) {
      for (int64_t v : c->spidx[k]) sp.push_back((int)v);
      for (int64_t v : c->colidx[k]) ci.push_back((int)v);
      c->sp_off.push_back((int64_t)sp.size());
    }
    if ((rc = upload_vec(c.get(), &c->d_spidx, sp))) return rc;
    if ((rc = upload_vec(c.get(), &c->d_colidx, ci))) return rc;
    std::vector<int> wc(c->whichc.begin(), c->whichc.end());
    if ((rc = upload_vec(c.get(), &c->d_whichc, wc))) return rc;
    std::vector<int> p1(c->p1cg.begin(), c->p1cg.end());
    if ((rc = upload_vec(c.get(), &c->d_p1cg, p1))) return rc;
    std::vector<double> cnt(c->ncg, 0.0), wdg(c->B * c->NC);
    for (int64_t v : c->p1cg) cnt[v] += 1.0;
    for (size_t k = 0; k < c->p1cg.size(); ++k) wdg[k] = 1.0 / cnt[c->p1cg[k]];
    if ((rc = upload_vec(c.get(), &c->d_wdg, wdg))) return rc;
    std::vector<float> wdg32(wdg.begin(), wdg.end());
    if ((rc = upload_vec(c.get(), &c->d_wdg32, wdg32))) return rc;
    std::vector<int> gptr(c->ncg + 1, 0), gent(c->p1cg.size());
    for (int64_t v : c->p1cg) gptr[v + 1]++;
    for (int64_t i = 0; i < c->ncg; ++i) gptr[i + 1] += gptr[i];
    std::vector<int> fill(gptr.begin(), gptr.end() - 1);
    for (size_t k = 0; k < c->p1cg.size(); ++k) gent[fill[c->p1cg[k]]++] = (int)k;   // ascending DG index
    if ((rc = upload_vec(c.get(), &c->d_gptr, gptr))) return rc;
    if ((rc = upload_vec(c.get(), &c->d_gent, gent))) return rc;
    std::vector<int> pos(c->ncg);
    std::vector<char> seen(c->ncg, 0);
    for (int64_t i = 0; i < c->ncg; ++i) {
      int64_t p = c->sfc[i] - 1;
      if (p < 0 || p >= c->ncg || seen[p]) return fail(c.get(), DG_ERR_ARG, "sfc_order is not a permutation of 1..cg_nonods");
      seen[p] = 1;
      pos[i] = (int)p;
    }
    if ((rc = upload_vec(c.get(), &c->d_pos, pos))) return rc;
  }
  if (c->rap_direct) {
    std::vector<int64_t> nbe64(nbe.begin(), nbe.end()), rptr;
    std::vector<std::array<int64_t, 3>> rent;
    if ((rc = rap_contributions(c->B, D, c->p1cg.data(), nbe64.data(), c->fina.data(), c->cola.data(), c->ncg, rptr,
                                rent)))
      return fail(c.get(), rc, g_thread_error);
    if ((int64_t)c->B * (F + 1) * 16 >= (int64_t)INT32_MAX || (int64_t)rent.size() >= (int64_t)INT32_MAX)
      return fail(c.get(), DG_ERR_ARG, "mesh too large for the direct P1CG assembly");
    std::vector<int> rp(rptr.begin(), rptr.end()), re(rent.size());
    for (size_t t = 0; t < rent.size(); ++t) re[t] = (int)(rent[t][0] * 16 + rent[t][1] * 4 + rent[t][2]);
    if ((rc = upload_vec(c.get(), &c->d_rap_ptr, rp))) return rc;
    if ((rc = upload_vec(c.get(), &c->d_rap_ent, re))) return rc;
    if ((rc = dalloc(c.get(), &c->d_rap_G, (size_t)c->B * (F + 1) * c->NC * c->NC))) return rc;
  }
  if ((rc = dalloc(c.get(), &c->d_rar, c->cola.size()))) return rc;
  for (double** t : {&c->d_t1, &c->d_t2, &c->d_t3, &c->d_t4, &c->d_t5})
    if ((rc = dalloc(c.get(), t, (size_t)c->nonods))) return rc;
  for (double** t : {&c->d_cg1, &c->d_cg2})
    if ((rc = dalloc(c.get(), t, (size_t)c->ncg))) return rc;
  if ((rc = dalloc(c.get(), &c->d_r1, (size_t)c->B * c->NC))) return rc;
  if ((rc = dalloc(c.get(), &c->d_part, (size_t)c->nred * KMAXV))) return rc;
  for (double** t : {&c->d_h1, &c->d_h2, &c->d_y, &c->d_scal})
    if ((rc = dalloc(c.get(), t, 256))) return rc;
  *out = c.release();
  return DG_OK;
}

int dg_set_kappa(dg_ctx* c, const double* kappa) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_kappa: null context");
  if (kappa) {
    for (int64_t e = 0; e < c->B; ++e)
      if (!(kappa[e] > 0.0) || !std::isfinite(kappa[e])) return fail(c, DG_ERR_ARG, "kappa must be positive and finite");
    c->kappa.assign(kappa, kappa + c->B);
  } else {
    c->kappa.assign(c->B, 1.0);
  }
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaMemcpy(c->d_kappa, c->kappa.data(), sizeof(double) * c->B, cudaMemcpyHostToDevice));
  c->built = false;
  return DG_OK;
}

int dg_set_face_kappa(dg_ctx* c, int32_t mode) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_face_kappa: null context");
  if (mode != 0 && mode != 1) return fail(c, DG_ERR_ARG, "dg_set_face_kappa: mode 0 (mean) or 1 (harmonic)");
  if (c->face_kappa != mode) c->built = false;
  c->face_kappa = mode;
  return DG_OK;
}

int dg_build_operator(dg_ctx* c, void* stream) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_build_operator: null context");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  int rc;
  const auto t0 = std::chrono::steady_clock::now();
  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
  if ((rc = (c->D == 3 ? launch_build<3>(c, st) : launch_build<2>(c, st)))) return rc;
  int herr = 0;
  CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  const double t_blocks = ms_since(t0);
  if (herr) return fail(c, DG_ERR_MESH, "non-positive element Jacobian (element not positively oriented)");
  if (c->d_geom) c->geom_ok = true;
  c->built = true;   // blocks are usable from here on (the probes below apply them)
  ++c->build_version;
  // colour-probe Galerkin operator on P1CG (volume_mf_diff.py:1696-1754), or
  // the same product formed directly from the blocks
  CK(c, cudaMemsetAsync(c->d_rar, 0, sizeof(double) * c->cola.size(), st));
  if (c->rap_direct && c->d_rap_ptr) {
    const int64_t nb = c->B * (c->F + 1);
    if (c->D == 3)
      block_galerkin_kernel<20, 4><<<nblk(nb, 4), 128, 0, st>>>(c->d_blk, c->T.P, c->d_rap_G, nb);
    else
      block_galerkin_kernel<10, 3><<<nblk(nb, 4), 128, 0, st>>>(c->d_blk, c->T.P, c->d_rap_G, nb);
    bump();
    rap_gather_kernel<<<nblk((int64_t)c->cola.size(), 128), 128, 0, st>>>(
        c->d_rap_G, c->d_rap_ptr, c->d_rap_ent, c->d_wdg, c->d_nbe, c->F, c->NC, c->d_rar,
        (int64_t)c->cola.size());
    bump();
    CKL(c);
  }
  for (int col = 1; col <= ((c->rap_direct && c->d_rap_ptr) ? 0 : c->ncolor); ++col) {
    if ((rc = prolong_cg(c, c->d_t1, nullptr, false, col, false, st))) return rc;
    if ((rc = residual(c, c->d_t1, nullptr, c->d_t2, nullptr, RF_NEG, st))) return rc;   // t2 = A t1
    if ((rc = restrict_cg(c, c->d_t2, c->d_cg1, false, st))) return rc;
    int64_t a = c->sp_off[col - 1], b = c->sp_off[col];
    if (b > a)
      rar_scatter_kernel<<<nblk(b - a, 128), 128, 0, st>>>(c->d_rar, c->d_cg1, c->d_spidx + a, c->d_colidx + a,
                                                            (int)(b - a)); bump();
    CKL(c);
  }
  SfcHierarchy& h = c->sfc_h;
  if (c->lev_maps_ready) {
    // SFC level values and diagonals from the Galerkin values, on the device,
    // in the host builder's summation order (same bits)
    const double t_probes = ms_since(t0);
    bool any_host = false;
    for (int l = 0; l < h.nlevel; ++l) {
      DevLevel& L = c->lev[l];
      if (L.host_sum) {
        any_host = true;
        continue;
      }
      if (L.nnz > 0)
        sfc_level_values_kernel<<<nblk(L.nnz, 256), 256, 0, st>>>(c->d_rar, L.vptr, L.vk, L.nnz, L.val);
      sfc_level_diag_kernel<<<nblk(L.n, 256), 256, 0, st>>>(L.val, L.didx, L.n, L.diag);
      bump(2);
    }
    CKL(c);
    if (any_host) {
      if (!c->rar_pinned) CK(c, cudaMallocHost((void**)&c->rar_pinned, sizeof(double) * c->cola.size()));
      CK(c, cudaMemcpyAsync(c->rar_pinned, c->d_rar, sizeof(double) * c->cola.size(), cudaMemcpyDeviceToHost, st));
      CK(c, cudaStreamSynchronize(st));
      struct HV {
        std::vector<double> val, diag;
      };
      std::vector<HV> hv(h.nlevel);
      parallel_for(h.nlevel, [&](int l) {
        const DevLevel& L = c->lev[l];
        if (!L.host_sum) return;
        HV& o = hv[l];
        o.val.resize(L.nnz);
        for (int d = 0; d < L.nnz; ++d) {
          int j = L.h_vptr[d];
          double sum = c->rar_pinned[L.h_vk[j]];
          for (++j; j < L.h_vptr[d + 1]; ++j) sum += c->rar_pinned[L.h_vk[j]];
          o.val[d] = sum;
        }
        o.diag.resize(L.n);
        for (int i = 0; i < L.n; ++i) o.diag[i] = L.h_didx[i] >= 0 ? o.val[L.h_didx[i]] : 0.0;
      });
      for (int l = 0; l < h.nlevel; ++l) {
        const DevLevel& L = c->lev[l];
        if (!L.host_sum) continue;
        CK(c, cudaMemcpyAsync(L.val, hv[l].val.data(), sizeof(double) * L.nnz, cudaMemcpyHostToDevice, st));
        CK(c, cudaMemcpyAsync(L.diag, hv[l].diag.data(), sizeof(double) * L.n, cudaMemcpyHostToDevice, st));
      }
    }
    CK(c, cudaStreamSynchronize(st));
    if (c->verbose)
      std::fprintf(stderr, "[dg_build_operator] ms: blocks %.2f, colour probes %.2f, SFC level values (device) %.2f\n",
                   t_blocks, t_probes - t_blocks, ms_since(t0) - t_probes);
    return DG_OK;
  }
  c->rar_host.assign(c->cola.size(), 0.0);
  CK(c, cudaMemcpyAsync(c->rar_host.data(), c->d_rar, sizeof(double) * c->cola.size(), cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  const double t_probes = ms_since(t0);
  // SFC levels (compact_fcode.f90 + get_a_diaga)
  h = SfcHierarchy();
  std::vector<std::vector<int64_t>> visit_tgt;
  if ((rc = sfc_levels(c->ncg, c->fina.data(), c->cola.data(), c->rar_host.data(), c->sfc.data(), h, &visit_tgt)))
    return fail(c, rc, g_thread_error);
  const double t_sfc = ms_since(t0);
  // (re)allocate the device levels
  if (c->lev.size() != (size_t)h.nlevel) {
    c->lev.assign(h.nlevel, DevLevel());
    for (int l = 0; l < h.nlevel; ++l) {
      DevLevel& L = c->lev[l];
      L.n = (int)h.sizes[l];
      int64_t nnz = h.row_ptr[h.start[l + 1]] - h.row_ptr[h.start[l]];
      if ((rc = dalloc(c, &L.rowptr, L.n + 1))) return rc;
      if ((rc = dalloc(c, &L.col, nnz))) return rc;
      if ((rc = dalloc(c, &L.val, nnz))) return rc;
      if ((rc = dalloc(c, &L.diag, L.n))) return rc;
      if ((rc = dalloc(c, &L.e, L.n))) return rc;
      if ((rc = dalloc(c, &L.e2, L.n))) return rc;
      if ((rc = dalloc(c, &L.r, L.n))) return rc;
      if ((rc = dalloc(c, &L.rr, L.n))) return rc;
      if (l + 1 < h.nlevel) {
        // nn.Upsample(scale_factor = n_l / n_{l+1}, nearest) source index:
        // floor(float32(dst * (1 / s))) with the product in double
        int nc = (int)h.sizes[l + 1];
        double s = (double)L.n / (double)nc;
        int out = (int)std::floor((double)nc * s);
        if (out != L.n) return fail(c, DG_ERR_STATE, "upsampled level size differs from the fine level");
        std::vector<int> up(L.n);
        for (int i = 0; i < L.n; ++i) {
          int src;
          if (L.n == nc) src = i;
          else if (L.n == 2 * nc) src = i >> 1;
          else src = (int)std::floor((float)((double)i * (1.0 / s)));
          up[i] = std::min(src, nc - 1);
        }
        if ((rc = upload_vec(c, &L.up, up))) return rc;
      }
    }
  }
  choose_vcycle_cluster(c);
  // rows sorted by column (torch CSR from COO) and the diagonal taken, level
  // by level on parallel host threads; then the uploads in level order
  // the fine entries in the order the level sums visit them
  std::vector<int> vk;
  {
    std::vector<int64_t> inv(c->ncg);
    for (int64_t i = 0; i < c->ncg; ++i) inv[c->sfc[i] - 1] = i;
    vk.reserve(c->cola.size());
    for (int64_t sidx = 0; sidx < c->ncg; ++sidx) {
      const int64_t node = inv[sidx];
      for (int64_t k = c->fina[node]; k < c->fina[node + 1]; ++k) vk.push_back((int)k);
    }
  }
  struct Up {
    std::vector<int> rp, cl;
    std::vector<double> vl, dg;
    std::vector<int> vptr, vkl, didx;   // summation lists in device entry order
  };
  std::vector<Up> ups(h.nlevel);
  parallel_for(h.nlevel, [&](int l) {
    Up& U = ups[l];
    const int n = (int)h.sizes[l];
    const int64_t r0 = h.start[l];
    const int64_t base = h.row_ptr[r0];
    const int64_t nnz = h.row_ptr[h.start[l + 1]] - base;
    U.rp.resize(n + 1);
    U.cl.resize(nnz);
    U.vl.resize(nnz);
    U.dg.assign(n, 0.0);
    U.didx.assign(n, -1);
    std::vector<int64_t> dev_of(nnz);   // host (level-local) entry -> device entry
    std::vector<std::pair<int64_t, int64_t>> row;   // (column, host entry)
    for (int i = 0; i < n; ++i) {
      const int64_t a = h.row_ptr[r0 + i], b = h.row_ptr[r0 + i + 1];
      row.clear();
      for (int64_t k = a; k < b; ++k) row.emplace_back(h.col[k], k - base);
      std::sort(row.begin(), row.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
      U.rp[i] = (int)(a - base);
      for (size_t k = 0; k < row.size(); ++k) {
        const int64_t d = a - base + (int64_t)k;
        U.cl[d] = (int)row[k].first;
        U.vl[d] = h.val[base + row[k].second];
        dev_of[row[k].second] = d;
        if (row[k].first == i) {
          U.dg[i] = U.vl[d];
          U.didx[i] = (int)d;
        }
      }
    }
    U.rp[n] = (int)nnz;
    // counting sort of the visits by device entry, visit order kept
    const std::vector<int64_t>& tg = visit_tgt[l];
    U.vptr.assign(nnz + 1, 0);
    for (int64_t t : tg) U.vptr[dev_of[t] + 1]++;
    for (int64_t d = 0; d < nnz; ++d) U.vptr[d + 1] += U.vptr[d];
    std::vector<int> fill(U.vptr.begin(), U.vptr.end() - 1);
    U.vkl.resize(tg.size());
    for (size_t v = 0; v < tg.size(); ++v) U.vkl[fill[dev_of[tg[v]]]++] = vk[v];
  });
  for (int l = 0; l < h.nlevel; ++l) {
    DevLevel& L = c->lev[l];
    const Up& U = ups[l];
    // on the context's stream: no legacy-stream copy that would wait for
    // other streams (several contexts serve concurrently); copies from
    // pageable memory return once the source has been staged
    CK(c, cudaMemcpyAsync(L.rowptr, U.rp.data(), sizeof(int) * U.rp.size(), cudaMemcpyHostToDevice, st));
    CK(c, cudaMemcpyAsync(L.col, U.cl.data(), sizeof(int) * U.cl.size(), cudaMemcpyHostToDevice, st));
    CK(c, cudaMemcpyAsync(L.val, U.vl.data(), sizeof(double) * U.vl.size(), cudaMemcpyHostToDevice, st));
    CK(c, cudaMemcpyAsync(L.diag, U.dg.data(), sizeof(double) * U.dg.size(), cudaMemcpyHostToDevice, st));
    L.nnz = (int)U.cl.size();
    int maxlen = 0;
    for (int d = 0; d < L.nnz; ++d) maxlen = std::max(maxlen, U.vptr[d + 1] - U.vptr[d]);
    L.host_sum = maxlen > 64;
    if (L.host_sum) {
      L.h_vptr = U.vptr;
      L.h_vk = U.vkl;
      L.h_didx = U.didx;
    } else {
      if (!L.vptr) {
        if ((rc = dalloc(c, &L.vptr, U.vptr.size()))) return rc;
        if ((rc = dalloc(c, &L.vk, std::max<size_t>(U.vkl.size(), 1)))) return rc;
        if ((rc = dalloc(c, &L.didx, std::max<size_t>(U.didx.size(), 1)))) return rc;
      }
      CK(c, cudaMemcpyAsync(L.vptr, U.vptr.data(), sizeof(int) * U.vptr.size(), cudaMemcpyHostToDevice, st));
      CK(c, cudaMemcpyAsync(L.vk, U.vkl.data(), sizeof(int) * U.vkl.size(), cudaMemcpyHostToDevice, st));
      CK(c, cudaMemcpyAsync(L.didx, U.didx.data(), sizeof(int) * U.didx.size(), cudaMemcpyHostToDevice, st));
    }
  }
  CK(c, cudaStreamSynchronize(st));
  c->lev_maps_ready = true;
  if (c->verbose)
    std::fprintf(stderr, "[dg_build_operator] ms: blocks %.2f, colour probes %.2f, SFC levels (host) %.2f, "
                 "level upload %.2f\n", t_blocks, t_probes - t_blocks, t_sfc - t_probes, ms_since(t0) - t_sfc);
  return DG_OK;
}

int dg_get_bdiag(dg_ctx* c, double* bdiag, double* diag, void* stream) {
  if (!c || !bdiag) return set_thread_error(DG_ERR_ARG, "dg_get_bdiag: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_get_bdiag: operator not built");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  const int N = c->N, F = c->F;
  // blocks are stored column-major: transpose block 0 of every element
  CK(c, cudaMemcpy2DAsync(bdiag, sizeof(double) * N * N, c->d_blk, sizeof(double) * N * N * (F + 1),
                          sizeof(double) * N * N, c->B, cudaMemcpyDeviceToDevice, st));
  // in-place transpose on the device copy (row-major output)
  // (A_ee is symmetric up to roundoff; transpose keeps the exact entries)
  std::vector<double> h((size_t)c->B * N * N);
  CK(c, cudaMemcpyAsync(h.data(), bdiag, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  std::vector<double> t(h.size()), dgv((size_t)c->B * N);
  for (int64_t e = 0; e < c->B; ++e)
    for (int m = 0; m < N; ++m) {
      for (int n = 0; n < N; ++n) t[(e * N + m) * N + n] = h[(e * N + n) * N + m];
      dgv[e * N + m] = h[(e * N + m) * N + m];
    }
  CK(c, cudaMemcpyAsync(bdiag, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, st));
  if (diag) CK(c, cudaMemcpyAsync(diag, dgv.data(), sizeof(double) * dgv.size(), cudaMemcpyHostToDevice, st));
  CK(c, cudaStreamSynchronize(st));
  return DG_OK;
}

int dg_get_rar(dg_ctx* c, double* values, void* stream) {
  if (!c || !values) return set_thread_error(DG_ERR_ARG, "dg_get_rar: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_get_rar: operator not built");
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaMemcpyAsync(values, c->d_rar, sizeof(double) * c->cola.size(), cudaMemcpyDeviceToDevice, S(stream)));
  return DG_OK;
}

int dg_residual(dg_ctx* c, const double* x, const double* b, double* r, double* x_out, int32_t do_smooth,
                void* stream) {
  if (!c || !x || !r) return set_thread_error(DG_ERR_ARG, "dg_residual: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_residual: operator not built");
  if (do_smooth && !x_out) return fail(c, DG_ERR_ARG, "dg_residual: x_out required for smoothing");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  if (!do_smooth) return residual(c, x, b, r, nullptr, 0, st);
  double* dst = (x_out == x) ? c->d_t1 : x_out;
  int rc = residual(c, x, b, r, dst, RF_SMOOTH, st);
  if (rc) return rc;
  if (dst != x_out) CK(c, cudaMemcpyAsync(x_out, dst, sizeof(double) * c->nonods, cudaMemcpyDeviceToDevice, st));
  return DG_OK;
}

int dg_apply(dg_ctx* c, const double* x, double* y, void* stream) {
  if (!c || !x || !y) return set_thread_error(DG_ERR_ARG, "dg_apply: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_apply: operator not built");
  CK(c, cudaSetDevice(c->dev));
  return residual(c, x, nullptr, y, nullptr, RF_NEG, S(stream));
}

int dg_rhs(dg_ctx* c, const double* f, const double* g, const double* gn, double* b, void* stream) {
  if (!c || !f || !b) return set_thread_error(DG_ERR_ARG, "dg_rhs: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_rhs: operator not built");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  if (c->D == 3) {
    using E = Elem<3>;
    rhs_mass_kernel<E::N, E::VG, E::EPB><<<nblk(c->B, E::EPB), E::EPB * E::N, 0, st>>>(c->T.n, c->d_detw, f, b, c->B); bump();
  } else {
    using E = Elem<2>;
    rhs_mass_kernel<E::N, E::VG, E::EPB><<<nblk(c->B, E::EPB), E::EPB * E::N, 0, st>>>(c->T.n, c->d_detw, f, b, c->B); bump();
  }
  CKL(c);
  for (int mode = 0; mode < 2; ++mode) {
    const double* src = mode == 0 ? g : gn;
    if (!src || c->nbf == 0) continue;
    for (int fsel = 0; fsel < c->F; ++fsel) {
      if (c->D == 3)
        rhs_bface_kernel<20, 12><<<nblk(c->nbf, 8), 8 * 20, 0, st>>>(
            c->T.sn, c->d_bf_elem, c->d_bf_face, c->d_bf_type, c->d_bf_sw, c->d_bf_gn, c->d_bf_gam, c->d_kappa, src,
            b, c->nbf, fsel, mode, c->cfg.mu_f);
      else
        rhs_bface_kernel<10, 4><<<nblk(c->nbf, 16), 16 * 10, 0, st>>>(
            c->T.sn, c->d_bf_elem, c->d_bf_face, c->d_bf_type, c->d_bf_sw, c->d_bf_gn, c->d_bf_gam, c->d_kappa, src,
            b, c->nbf, fsel, mode, c->cfg.mu_f);
      bump();
      CKL(c);
    }
  }
  return DG_OK;
}

int dg_precond(dg_ctx* c, const double* r, double* z, void* stream) {
  if (!c || !r || !z) return set_thread_error(DG_ERR_ARG, "dg_precond: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_precond: operator not built");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  if (z == r) {
    int rc = precond(c, r, c->d_t1, st);
    if (rc) return rc;
    CK(c, cudaMemcpyAsync(z, c->d_t1, sizeof(double) * c->nonods, cudaMemcpyDeviceToDevice, st));
    return DG_OK;
  }
  return precond(c, r, z, st);
}

int dg_mg_vcycle(dg_ctx* c, const double* r_sfc, double* e_sfc, void* stream) {
  if (!c || !r_sfc || !e_sfc) return set_thread_error(DG_ERR_ARG, "dg_mg_vcycle: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_mg_vcycle: operator not built");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  int rc = vcycle(c, r_sfc, st);
  if (rc) return rc;
  CK(c, cudaMemcpyAsync(e_sfc, c->lev[0].e, sizeof(double) * c->ncg, cudaMemcpyDeviceToDevice, st));
  return DG_OK;
}

int dg_set_build_mode(dg_ctx* c, int32_t mode) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_build_mode: null context");
  if (mode != 0 && mode != 1) return fail(c, DG_ERR_ARG, "dg_set_build_mode: mode must be 0 (quadrature) or 1 (affine)");
  const bool general = mode == 0;
  if (general != c->general_build) c->built = false;
  c->general_build = general;
  return DG_OK;
}

int dg_set_gmres_ortho(dg_ctx* c, int32_t mode) {
  if (!c) return set_thread_error(DG_ERR_ARG, "dg_set_gmres_ortho: null context");
  if (mode != 0 && mode != 1) return fail(c, DG_ERR_ARG, "dg_set_gmres_ortho: mode must be 0 (CGS2) or 1 (MGS)");
  c->gmres_ortho = mode;
  return DG_OK;
}

int dg_gmres(dg_ctx* c, double* x, const double* b, double tol, int32_t m, int32_t max_its, int32_t* its_out,
             double* res_out, void* stream) {
  if (!c || !x || !b) return set_thread_error(DG_ERR_ARG, "dg_gmres: null argument");
  if (!c->built) return fail(c, DG_ERR_STATE, "dg_gmres: operator not built");
  if (m <= 0 || m > 256 || max_its < 0) return fail(c, DG_ERR_ARG, "dg_gmres: 1 <= m <= 256 required");
  cudaStream_t st = S(stream);
  CK(c, cudaSetDevice(c->dev));
  int rc;
  if ((rc = ensure_krylov(c, m))) return rc;
  double* r = c->d_t1;
  double* w = c->d_t2;
  int its = 0;
  double r0l2 = 1.0;   // the reference starts from 1 and tests before each cycle
  std::vector<double> Hh((size_t)(m + 1) * m), y;
  int status = DG_OK;
  while (r0l2 > tol && its < max_its) {
    CK(c, cudaMemsetAsync(c->d_H, 0, sizeof(double) * (m + 1) * m, st));
    if ((rc = residual(c, x, b, w, nullptr, 0, st))) return rc;          // w = b - A x
    if ((rc = precond(c, w, r, st))) return rc;                           // r = M^-1 w
    if ((rc = norm2(c, r, c->d_scal, st))) return rc;
    double beta;
    if ((rc = read_scalar(c, c->d_scal, &beta, st))) return rc;
    if (!(beta > 0.0) || !std::isfinite(beta)) {
      status = beta == 0.0 ? DG_OK : DG_ERR_NUMERIC;
      break;
    }
    scale_kernel<<<nblk(c->nonods, 256), 256, 0, st>>>(r, c->d_scal, c->d_V, c->nonods); bump();
    CKL(c);
    if ((rc = run_arnoldi(c, m, st))) return rc;
    its += m;
    CK(c, cudaMemcpyAsync(Hh.data(), c->d_H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (!solve_hessenberg(Hh, m, beta, y)) {
      status = DG_ERR_NUMERIC;
      c->err = "GMRES breakdown: singular Hessenberg matrix";
      break;
    }
    CK(c, cudaMemcpyAsync(c->d_y, y.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
    combine_kernel<<<nblk(c->nonods, 256), 256, 0, st>>>(c->d_V, c->nonods, m, c->d_y, x, c->nonods); bump();
    CKL(c);
    if ((rc = residual(c, x, b, w, nullptr, 0, st))) return rc;
    if ((rc = norm2(c, w, c->d_scal, st))) return rc;
    if ((rc = read_scalar(c, c->d_scal, &r0l2, st))) return rc;
    if (!std::isfinite(r0l2)) {
      status = DG_ERR_NUMERIC;
      c->err = "GMRES produced a non-finite residual";
      break;
    }
  }
  if (its_out) *its_out = its;
  if (res_out) *res_out = r0l2;
  if (status == DG_OK && r0l2 > tol && its >= max_its) {
    c->err = "GMRES reached the iteration limit";
    return DG_ERR_NOCONV;
  }
  return status;
}

}  // extern "C"

#include "dg_noalloc.cuh"
