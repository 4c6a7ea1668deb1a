/*
 * dgsip.h -- C ABI of the GB300 SIP-DG diffusion solver (libdgsip.so).
 *
 * Symmetric interior-penalty DG for -div(kappa grad u) = f on cubic (P3)
 * triangles (2D, 10 nodes) and tetrahedra (3D, 20 nodes), with the
 * reference's DG->CG P1 + space-filling-curve multigrid preconditioner and
 * restarted GMRES.  Every function returns 0 on success and a positive
 * error code otherwise; dg_last_error() gives the message.  No function
 * calls exit() or traps the device.
 *
 * Memory: arrays marked [host] are read during the call and copied; arrays
 * marked [device] are caller-owned device pointers (e.g. torch CUDA tensor
 * storage), FP64, element-major (nele, nloc).  A context owns every other
 * device buffer.  All device work of a call is enqueued on `stream`
 * (a cudaStream_t passed as void*, NULL = legacy default stream); calls on
 * one context are not thread-safe.
 *
 * Reference: linfeng810/dg_nn_public, directory z02-implicit/z06-DGtoCG
 * (cited below as z06/) and z00-fortran-src.
 */
#ifndef DGSIP_H
#define DGSIP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dg_ctx dg_ctx;

/* Error codes. */
enum {
  DG_OK = 0,
  DG_ERR_ARG = 1,        /* invalid argument / size */
  DG_ERR_CUDA = 2,       /* CUDA runtime error */
  DG_ERR_MESH = 3,       /* inconsistent mesh arrays */
  DG_ERR_STATE = 4,      /* call order (e.g. solve before build_operator) */
  DG_ERR_NUMERIC = 5,    /* breakdown / non-finite values */
  DG_ERR_NOCONV = 6,     /* iteration limit reached before the tolerance */
  DG_ERR_ALLOC = 7       /* device or host allocation failed */
};

/* Storage precision of the stored operator blocks / multigrid. */
enum { DG_F64 = 0, DG_F32 = 1, DG_BF16 = 2 };

/* Mesh + reference element, in the reference's layout.
 * Replaces the implicit inputs the reference reads from its FuncSpace /
 * Element objects and cmmn_data.SfNdNb (z06/function_space.py:83-404,
 * z06/cmmn_data.py:8-138). */
typedef struct dg_mesh_desc {
  int32_t ndim;                 /* 2 or 3 */
  int32_t nloc;                 /* 10 (tri) or 20 (tet) */
  int64_t nele;
  const double*  x_ref_in;      /* [host] (nele, ndim, nloc) node coordinates */
  const int64_t* nbf;           /* [host] (nele*nface) neighbour face, -1 = none */
  const int64_t* alnmt;         /* [host] (nele*nface) quadrature alignment code */
  const int64_t* glb_bcface_type; /* [host] (nele*nface) -1 interior, 0 Dirichlet, 1 Neumann */
  int64_t cg_nonods;            /* number of P1CG vertices */
  const int64_t* p1cg;          /* [host] (nele, ndim+1) P1CG vertex of each corner, 0-based */
  const int64_t* sfc_order;     /* [host] (cg_nonods) 1-based curve position of each vertex */
  /* reference-element tables (z06/shape_function.py:459-1317) */
  int32_t ngi, sngi;
  const double*  n;             /* [host] (nloc, ngi) */
  const double*  nlx;           /* [host] (ndim, nloc, ngi) */
  const double*  weight;        /* [host] (ngi) */
  const double*  sn;            /* [host] (nface, nloc, sngi) */
  const double*  snlx;          /* [host] (nface, ndim, nloc, sngi) */
  const double*  sweight;       /* [host] (sngi) */
  const int64_t* gi_align;      /* [host] (ndim, sngi) */
  const double*  drst_duv;      /* [host] (nface, ndim, ndim-1) face tangents (z06/function_space.py:200-219) */
  const double*  p1_to_p3;      /* [host] (nloc, ndim+1) element prolongator (z06/mesh_init.py:586-607) */
} dg_mesh_desc;

/* Solver knobs; names follow z06/config.py:103-149, 245. */
typedef struct dg_config {
  double  eta_e;                /* penalty coefficient (gamma = eta_e / h) */
  double  mu_f;                 /* diffusion coefficient multiplier */
  double  jac_wei;              /* Jacobi weight (2/3) */
  int32_t pre_smooth_its;       /* smoothing steps before/after the coarse correction */
  int32_t post_smooth_its;      /* SFC-level post smoothing (reference: post_smooth_its) */
  int32_t device;               /* CUDA device ordinal */
} dg_config;

/* ---- context (replaces module state: z06/config.py, z06/cmmn_data.py) ---- */
int  dg_create(const dg_mesh_desc* mesh, const dg_config* cfg, dg_ctx** out);
void dg_destroy(dg_ctx* ctx);
/* Message of the last failed call on ctx; ctx = NULL gives the last failed
 * dg_create / host-only helper on this thread. */
const char* dg_last_error(const dg_ctx* ctx);
/* out[0..18]: ndim, nloc, nele, nonods, cg_nonods, ncola, ncolor, nlevel,
 * nbface, built, ngi, sngi, chosen bulk-copy launch shape, batched
 * bulk-copy form on/off, interior faces stored once in the reduced-precision
 * copies (0 = five blocks per element), batched smoothing kernel variant,
 * preconditioner smoothing on scaled face blocks (see dg_smooth_scaled),
 * launch shape of that kernel, bytes of device memory the context has
 * allocated (held until dg_destroy). */
int  dg_info(const dg_ctx* ctx, int64_t* out, int32_t nout);
/* Number of CUDA kernels this library has launched in this process (all
 * contexts); used to account for device work in benchmarks. */
long long dg_launch_count(void);

/* ---- operator ---- */
/* Per-element diffusivity (z05-ns/volume_mf_um_diff_varprop.py:422-426,
 * 567, 682); NULL restores kappa = 1. */
int dg_set_kappa(dg_ctx* ctx, const double* kappa /* [host] (nele) or NULL */);
/* Interior-face diffusivity of the SIP form: mode 0 = (kappa_e + kappa_nb)/2
 * on all three face terms, the reference's variable-property convention
 * (z05-ns/volume_mf_um_diff_varprop.py:422-426); mode 1 = the harmonic mean
 * 2 kappa_e kappa_nb / (kappa_e + kappa_nb), the weighted-average SIP of Ern,
 * Stephansen and Zunino (IMA J. Numer. Anal. 29, 2009), which stays coercive
 * under large kappa jumps (no counterpart in the reference).  Takes effect
 * at the next dg_build_operator. */
int dg_set_face_kappa(dg_ctx* ctx, int32_t mode);
/* Element-block assembly: mode 0 (default) evaluates every element through
 * the isoparametric Jacobian at each quadrature point, the reference's own
 * formula (z06/volume_mf_diff.py:487-617, 909-1556); mode 1 forms the blocks
 * of straight-sided elements from reference matrices times per-element
 * geometric factors (equal to mode 0 within 1e-13 relative, ~3.4x faster;
 * curved elements still take mode 0).  Takes effect at the next
 * dg_build_operator. */
int dg_set_build_mode(dg_ctx* ctx, int32_t mode);
/* Assemble the stored element blocks, the block diagonal, the Galerkin P1CG
 * operator (per-block products P^T A_b P summed over fixed contribution
 * lists; the environment variable DG_RAP_DIRECT=0 selects the reference's
 * colour-probe form instead, one operator apply per colour of a distance-2
 * colouring, z06/volume_mf_diff.py:1696-1754) and the SFC levels.  Replaces get_bdiag_diag()
 * (z06/get_bdiag_diag.py:30-62) and _get_RAR_and_sfc_data_Um()
 * (z06/volume_mf_diff.py:1642-1693, multigrid_linearelastic.py:175-283). */
int dg_build_operator(dg_ctx* ctx, void* stream);
/* Copy bdiagK (nele, nloc, nloc) and diagK (nele, nloc) out. */
int dg_get_bdiag(dg_ctx* ctx, double* bdiag /* [device] */, double* diag /* [device] or NULL */, void* stream);
/* Copy the P1CG Galerkin values (ncola) into a device buffer. */
int dg_get_rar(dg_ctx* ctx, double* values /* [device] */, void* stream);

/* r = b - A x, and with do_smooth != 0 also x_out = x + w*c where c is three
 * point-Jacobi sweeps on each element block.  b may be NULL (taken as 0).
 * x_out may alias x.  Replaces get_residual_or_smooth
 * (z06/volume_mf_diff.py:403-483) with its _k_res_one_batch (:487-617) and
 * _s_res_one_batch (:1563-1639) callees. */
int dg_residual(dg_ctx* ctx, const double* x, const double* b, double* r, double* x_out,
                int32_t do_smooth, void* stream);
/* y = A x */
int dg_apply(dg_ctx* ctx, const double* x, double* y, void* stream);
/* b = M f + Dirichlet lifting of g + Neumann flux gn (z06/volume_mf_diff.py:153-359).
 * g, gn may be NULL. */
int dg_rhs(dg_ctx* ctx, const double* f, const double* g, const double* gn, double* b, void* stream);

/* ---- preconditioner ---- */
/* z = one DG->CG + SFC multigrid V-cycle applied to r, starting from z = 0
 * (_um_left_precond, z06/volume_mf_diff.py:1934-2029). */
int dg_precond(dg_ctx* ctx, const double* r, double* z, void* stream);
/* e = one SFC V-cycle on the P1CG residual r, both in SFC order
 * (mg_on_P1CG, z06/multigrid_linearelastic.py:112-172). */
int dg_mg_vcycle(dg_ctx* ctx, const double* r_sfc, double* e_sfc, void* stream);

/* ---- Krylov (z06/volume_mf_diff.py:1757-1841) ---- */
/* Left-preconditioned restarted GMRES(m) from the initial guess in x.
 * Stops when ||b - A x|| <= tol (absolute, tested after each restart cycle
 * as the reference does) or after max_its Arnoldi steps (status
 * DG_ERR_NOCONV, x holds the last iterate).  Arnoldi uses classical
 * Gram-Schmidt with one reorthogonalisation (CGS2).  its and res_norm
 * (final ||b - A x||) may be NULL. */
int dg_gmres(dg_ctx* ctx, double* x, const double* b, double tol, int32_t m, int32_t max_its,
             int32_t* its, double* res_norm, void* stream);
/* Orthogonalisation of dg_gmres's Arnoldi step: mode 0 = CGS2 (default; two
 * classical Gram-Schmidt passes, two reductions per step), mode 1 = modified
 * Gram-Schmidt in the reference's order (z06/volume_mf_diff.py:1814-1819:
 * h_ij = w . v_i then w -= h_ij v_i for i = 0..j), j + 1 dependent
 * reductions per step.  Takes effect at the next dg_gmres. */
int dg_set_gmres_ortho(dg_ctx* ctx, int32_t mode);

/* ---- mixed precision (new in this build; no counterpart in the reference) ----
 * FP64 iterative refinement around an FP32 inner solve: r = b - A x in FP64;
 * the correction solves A d = r/||r|| with right-preconditioned flexible
 * GMRES(m) in FP32 (FP32 copies of the operator blocks, smoother matrices
 * and SFC levels, FP64-accumulated CGS2, FP64 Hessenberg least squares),
 * stopping when the inner residual estimate is below inner_rtol; x += ||r|| d
 * in FP64, until ||b - A x|| <= tol (absolute).  its counts inner Arnoldi
 * steps, outer the refinement steps; all three outputs may be NULL. */
int dg_solve_mixed(dg_ctx* ctx, double* x, const double* b, double tol, int32_t m, int32_t max_its,
                   double inner_rtol, int32_t* its, double* res_norm, int32_t* outer, void* stream);
/* y = A x with the FP32 copy of the operator blocks (FP32 vectors). */
int dg_apply_f32(dg_ctx* ctx, const float* x, float* y, void* stream);
/* Batched mixed-precision solve (P3 tetrahedra): nrhs <= 64 systems
 * A x_q = b_q on one operator, x and b (nrhs, nonods) FP64 [device],
 * RHS-major; each stops at ||b_q - A x_q|| <= tol[q] [host] (FP64 true
 * residual).  The inner flexible GMRES(m <= 31) runs all active RHS in
 * lockstep on RHS-interleaved FP32 vectors, so every kernel reads the stored
 * blocks once for all of them.  its / res_norm [host] (nrhs, may be NULL).
 * The batched counterpart of _gmres_mg_solver (z06/volume_mf_diff.py:1757). */
int dg_solve_mixed_batched(dg_ctx* ctx, double* x, const double* b, int32_t nrhs, const double* tol, int32_t m,
                           int32_t max_its, double inner_rtol, int32_t* its, double* res_norm, void* stream);
/* Multi-RHS operator stages on RHS-interleaved FP32 vectors of 64 right-hand
 * sides (x[(e * 20 + n) * 64 + q], P3 tetrahedra; the layout of the batched
 * solve), the batched counterparts of get_residual_or_smooth
 * (z06/volume_mf_diff.py:403-483) with its per-element bmm smoother
 * (:474-480):
 *   dg_apply_batched:     Y = A X with the FP32 operator copy;
 *   dg_smooth_pc_batched: X_out = X + W (B - A X) with the preconditioner's
 *                         BF16 block copies (X NULL = zero guess), through
 *                         the batched smoothing kernel in use.
 * x_out must not alias x. */
int dg_apply_batched(dg_ctx* ctx, const float* x, float* y, void* stream);
int dg_smooth_pc_batched(dg_ctx* ctx, const float* x, const float* b, float* x_out, void* stream);
/* Kernel of the batched BF16 smoothing step (no counterpart in the
 * reference): -1 = chosen by timing every variant at the next batched solve
 * (the default, once per operator build), 0 = CUDA cores, 1 / 2 = mma.sync
 * tensor-core tiles, one element per CTA (4 / 8 warps), 3 = mma.sync in a
 * persistent bulk-copy pipeline, 4 = tcgen05.mma with tensor-memory
 * accumulators in a persistent bulk-copy pipeline, 5 = the same on an
 * iterate kept in the tensor-core operand layout (BF16 high + low parts,
 * bulk-copied straight into the MMA operand; the batched preconditioner
 * keeps its iterates in that layout and writes its output in FP32), 6 = the
 * same in one warp-specialized CTA per SM (a copy warp, an MMA-issuing
 * thread and eight epilogue warps on double-buffered accumulators).
 * dg_batched_tuning
 * reports the last timing per variant (microseconds per launch, -1 = not
 * timed; tune_us may be NULL) and the variant in use. */
int dg_set_batched_kernel(dg_ctx* ctx, int32_t variant);
int dg_batched_tuning(const dg_ctx* ctx, float* tune_us, int32_t n, int32_t* chosen);
/* z = the mixed-precision preconditioner applied once to r (FP32 vectors):
 * the DG->CG SFC V-cycle of dg_precond with the FP32/BF16 block copies and
 * the options of dg_set_mixed_options -- the reduced-precision counterpart
 * of _um_left_precond (z06/volume_mf_diff.py:1934-2029).  z must not alias r. */
int dg_precond_f32(dg_ctx* ctx, const float* r, float* z, void* stream);
/* One smoothing step of the mixed preconditioner on FP32 vectors,
 * x_out = x + W (b - A x) with the preconditioner's block copies (BF16 when
 * precond_bf16) -- the reduced-precision counterpart of
 * get_residual_or_smooth(do_smooth=True), z06/volume_mf_diff.py:403.
 * x_out must not alias x. */
int dg_smooth_pc(dg_ctx* ctx, const float* x, const float* b, float* x_out, void* stream);
/* The same step as the mixed preconditioner runs it after its zero-start
 * step, on the scaled face blocks S_ef = W_e A_ef (BF16; W_e = smooth_w *
 * A_ee^{-1}): x_out = x + (cv - smooth_w x - sum_f S_ef x_nb(f)), where cv =
 * W b.  Available when the scaled form is in use (3D, BF16 bulk-copy
 * preconditioner, damped block-inverse smoother; dg_info out[16]); otherwise
 * DG_ERR_STATE.  dg_smooth_pc runs the zero-start step for cv and then this
 * one.  x_out must not alias x. */
int dg_smooth_scaled(dg_ctx* ctx, const float* x, const float* cv, float* x_out, void* stream);
/* dg_smooth_scaled for 64 right-hand sides on RHS-interleaved vectors (the
 * layout of dg_apply_batched): the batched preconditioner's steps after its
 * zero-start one (tensor cores, x split into BF16 hi + lo).  The batched
 * preconditioner uses them with the mma.sync / tcgen05 gathered-x kernel
 * variants 1-4. */
int dg_smooth_scaled_batched(dg_ctx* ctx, const float* x, const float* cv, float* x_out, void* stream);
/* Options of the mixed preconditioner, applied at the next mixed solve:
 * smoother 0 = three point-Jacobi sweeps per element block (as the
 * reference), 1 = damped exact block inverse smooth_w * A_ee^{-1};
 * precond_bf16 != 0 keeps the preconditioner's blocks in BF16; dense_max =
 * size limit of the first SFC level solved exactly with a dense inverse
 * (0 = run the V-cycle down to the one-node level). */
int dg_set_mixed_options(dg_ctx* ctx, int32_t smoother, double smooth_w, int32_t precond_bf16,
                         int32_t dense_max);

/* Launch options (no counterpart in the reference): use_graph != 0 replays
 * GMRES Arnoldi cycles and mixed inner chunks as CUDA graphs (default on);
 * use_pdl != 0 links the kernels of a mixed inner Arnoldi step by
 * programmatic dependent launch (default on).  Cached graphs are captured
 * again at the next solve. */
int dg_set_launch_options(dg_ctx* ctx, int32_t use_graph, int32_t use_pdl);

/* SFC V-cycle of the mixed preconditioner (no counterpart in the reference):
 * cluster = -1 runs its down and up legs each as one thread-block-cluster
 * launch of 16 CTAs (8 where 16 is not schedulable), 0 as the chain of
 * per-sweep launches (default: faster at c2), 8 / 16 with that cluster size.
 * Both give the same bits.  *chosen (may be NULL) receives the size in use,
 * 0 for the chain (also when a CTA's share of the levels does not fit its
 * shared memory), -1 before the first mixed build.  Cached graphs are
 * captured again at the next solve. */
int dg_set_vcycle_cluster(dg_ctx* ctx, int32_t cluster, int32_t* chosen);

/* Allocation-free residual norm (no counterpart in the reference):
 * r = b - A x and *norm_out = ||r||_2, both written on the device (r may be
 * NULL for the norm alone; b NULL means b = 0).  It allocates nothing: its
 * scratch is a static device array of 65536 FP64 partial sums (512 KiB), one
 * per CTA of the residual launch, so meshes above 524288 tetrahedra or
 * 1048576 triangles are rejected with DG_ERR_ARG.  The first call for a
 * device looks up that array's address (cudaGetSymbolAddress, device
 * current) and caches it; make that first call before any stream capture.
 * The cached address assumes the device's primary context lives for the
 * whole process: do not call this after cudaDeviceReset.  Like every entry
 * point here, the call leaves the thread's current device set to the
 * context's device.  Nothing has to start at zero.  Calls whose kernels
 * overlap in time on one device (other streams or other contexts) share the
 * scratch and race. */
int dg_residual_norm_noalloc(dg_ctx* ctx, const double* x, const double* b, double* r, double* norm_out,
                             void* stream);

/* ---- host-only integer layer (no GPU needed) ---- */
/* P1CG sparsity from the element corners: all vertex pairs sharing an
 * element, rows sorted (z06/sparsity.py:102-122 with
 * z00-fortran-src/get_neighbouring.f90:133-157).  fina has cg_nonods+1
 * entries; cola capacity cap; *ncola gets the count. */
int dg_p1cg_sparsity(int64_t nele, int32_t ncorner, const int64_t* p1cg, int64_t cg_nonods,
                     int64_t* fina, int64_t* cola, int64_t cap, int64_t* ncola);
/* Greedy distance-2 colouring in vertex order (z06/sparsity.py:235-269);
 * colours are 1-based. */
int dg_color2(int64_t n, const int64_t* fina, const int64_t* cola, int64_t* whichc, int32_t* ncolor);
/* Space-filling-curve numbering of the P1CG vertices, in the format of the
 * reference's cache file <mesh>fluid_sfc.npy (z06/multigrid_linearelastic.py:
 * 221-229): order[i] = 1-based position of vertex i along the curve.
 * Ordering out (coords != NULL, (n, ndim) row-major): the vertices sorted by
 * the Hilbert index of their coordinates on a 2^bits grid (bits <= 0: 20 in
 * 2D, 16 in 3D), ties by vertex index -- a geometric curve in place of the
 * reference's Fortran graph-bisection curve
 * (z00-fortran-src/combined_fortran_source.f90:10575-10875), which needs a
 * Fortran compiler.  Ordering in (coords == NULL): order holds a curve read
 * from the reference's cache and is checked to be a permutation of 1..n;
 * dg_create accepts it unchanged. */
int dg_sfc_order(int32_t ndim, int64_t n, const double* coords, int32_t bits, int64_t* order);
/* Number of SFC grid levels (z00-fortran-src/compact_fcode.f90:229-250). */
int32_t dg_nlevel_sfc(int64_t nonods);
/* All SFC grid levels of a CSR matrix (compact_fcode.f90:7-225):
 * level_start (nlevel+1) gives each level's first row in the stacked
 * numbering; row_ptr (total+1) indexes col (cap) and val (cap), which hold
 * the stacked level matrices with 0-based level-local column indices in the
 * Fortran first-appearance order and values summed in the Fortran traversal
 * order.  The matrix rows and sfc_order use the caller's vertex numbering;
 * the levels are in curve order. */
int dg_sfc_levels(int64_t n, const int64_t* fina, const int64_t* cola, const double* a,
                  const int64_t* sfc_order, int32_t* nlevel, int64_t* level_start,
                  int64_t* row_ptr, int64_t* col, double* val, int64_t cap, int64_t* nnz);
/* Contribution lists of the Galerkin P1CG operator I_cf A I_fc from the
 * stored blocks, the direct form of the colour-probe assembly of
 * z06/volume_mf_diff.py:1696-1754: for every P1CG nonzero k (fina / cola),
 * entries[ptr[k] .. ptr[k+1]) are (block, a, c) triples with block =
 * e * (nface + 1) + slot (slot 0 = own block, 1 + f = neighbour across face
 * f, nbe (nele, nface) = neighbour element or -1), so that
 * RAP[k] = sum w(e, a) w(nb, c) (P^T A_block P)[a][c] with w = 1/#copies
 * (vertex pairs outside the P1CG sparsity are left out: their face-block
 * contributions cancel).  ptr has nnz+1 entries; entries capacity cap
 * triples; *count gets the number of triples. */
int dg_rap_contributions(int32_t ndim, int64_t nele, const int64_t* p1cg, const int64_t* nbe,
                         const int64_t* fina, const int64_t* cola, int64_t cg_nonods, int64_t* ptr,
                         int64_t* entries, int64_t cap, int64_t* count);
/* Face connectivity of cells in the reference's internal corner order
 * (z06/mesh_init.py:298-401): nbf and alnmt for all nele*nface faces. */
int dg_face_connectivity(int32_t ndim, int64_t nele, const int64_t* corners /* (nele, ndim+1) */,
                         int64_t* nbf, int64_t* alnmt);

/* ---- serving: native request queue (dg_enqueue / dg_poll) ----
 * The reference serves one solve at a time from one Python thread on the
 * default stream (z06/main.py:205-206 -> solve_for_diff); here nworkers host
 * threads, each with its own non-blocking CUDA stream on `device`, take the
 * queued requests in arrival order.  A request runs, on its context, the
 * optional operator rebuild for new diffusivities (dg_set_kappa with a copy
 * of kappa taken at enqueue time, then dg_build_operator) and the solve:
 * mode 0 dg_solve_mixed(tol, m, max_its, inner_rtol), mode 1 dg_gmres(tol,
 * m, max_its).  A context serves one request at a time; requests on one
 * context run in their order, requests on other contexts may pass a request
 * that waits for its context.  x and b are device pointers of the context's
 * size that must stay valid, and the context must not be used by the caller,
 * until the request is reported done; the workers' streams do not wait for
 * the caller's streams, so x and b must be ready when dg_enqueue is called.
 * Results are those of the same calls made directly. */
typedef struct dg_server dg_server;
enum { DG_REQ_QUEUED = 0, DG_REQ_RUNNING = 1, DG_REQ_DONE = 2 };
/* 1 <= nworkers <= 64; DG_ERR_CUDA without such a device. */
int dg_server_create(int32_t device, int32_t nworkers, dg_server** out);
/* Runs the queued requests to the end, then stops the workers. */
int dg_server_destroy(dg_server* srv);
/* *id receives the request's id (> 0). kappa [host] (nele) or NULL = keep
 * the context's operator. */
int dg_enqueue(dg_server* srv, dg_ctx* ctx, double* x, const double* b, double tol, int32_t mode, int32_t m,
               int32_t max_its, double inner_rtol, const double* kappa, int64_t* id);
/* *state = DG_REQ_QUEUED / RUNNING / DONE (may be NULL).  Once DONE:
 * status = the solve's return code (DG_OK, DG_ERR_NOCONV, ...; the message
 * is dg_last_error(ctx)), its, res_norm and seconds[2] = {queued, running}
 * (each may be NULL), and the request is forgotten: a later poll of its id
 * returns DG_ERR_ARG. */
int dg_poll(dg_server* srv, int64_t id, int32_t* state, int32_t* status, int32_t* its, double* res_norm,
            double* seconds);
/* dg_poll after waiting until the request is done or timeout_s has passed
 * (timeout_s < 0: no limit). */
int dg_wait(dg_server* srv, int64_t id, double timeout_s, int32_t* state, int32_t* status, int32_t* its,
            double* res_norm, double* seconds);

#ifdef __cplusplus
}
#endif
#endif /* DGSIP_H */
