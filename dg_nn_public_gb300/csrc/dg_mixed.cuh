// Mixed-precision solve: FP64 iterative refinement around an FP32 inner
// solver.  Included into dg_solver.cu (same translation unit: it uses the
// context and the launch helpers defined there).
//
//   outer (FP64):  r = b - A x;  stop when ||r|| <= tol
//   inner (FP32):  solve A d = r / ||r|| with right-preconditioned flexible
//                  GMRES(m): z_j = M v_j, w = A z_j, CGS2 (FP64 accumulated
//                  dot products), Hessenberg least squares in FP64 on the
//                  host; stops when the Hessenberg residual estimate falls
//                  below inner_rtol (checked every `chunk` steps)
//   x += ||r|| * d  (FP64)
//
// The FP32 operator, smoother matrices and SFC level values are copies of
// the FP64 ones (the smoother is the same three-sweep block-Jacobi map), so
// the inner solve runs the reference's preconditioner in single precision.

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
};

__global__ void f64_to_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n, double scale) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)(a[k] * scale);
}

// e = Ainv r for a small dense level matrix: one warp per row
__global__ void dense_matvec_kernel(const float* __restrict__ Ainv, const float* __restrict__ r,
                                    float* __restrict__ e, int n) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* a = Ainv + (size_t)row * n;
  float s = 0.0f;
  for (int k = lane; k < n; k += 32) s += a[k] * r[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) e[row] = s;
}

// Gauss-Jordan inverse with partial pivoting (host, FP64); false if singular
bool invert_dense(std::vector<double>& A, int n, std::vector<double>& inv) {
  inv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    double best = std::fabs(A[(size_t)col * n + col]);
    for (int r = col + 1; r < n; ++r) {
      double v = std::fabs(A[(size_t)r * n + col]);
      if (v > best) { best = v; piv = r; }
    }
    if (!(best > 0.0)) return false;
    if (piv != col)
      for (int k = 0; k < n; ++k) {
        std::swap(A[(size_t)piv * n + k], A[(size_t)col * n + k]);
        std::swap(inv[(size_t)piv * n + k], inv[(size_t)col * n + k]);
      }
    const double d = 1.0 / A[(size_t)col * n + col];
    for (int k = 0; k < n; ++k) {
      A[(size_t)col * n + k] *= d;
      inv[(size_t)col * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = A[(size_t)r * n + col];
      if (f == 0.0) continue;
      double* ar = &A[(size_t)r * n];
      double* ir = &inv[(size_t)r * n];
      const double* ac = &A[(size_t)col * n];
      const double* ic = &inv[(size_t)col * n];
      for (int k = 0; k < n; ++k) {
        ar[k] -= f * ac[k];
        ir[k] -= f * ic[k];
      }
    }
  }
  return true;
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
  delete M;
  c->mixed_state = nullptr;
}

template <int D>
int launch_residual32(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags,
                      cudaStream_t st) {
  using E = Elem<D>;
  Mixed& M = mixed_of(c);
  unsigned g = nblk(c->B, E::EPB);
  if (g)
    residual_kernel<E::N, E::F, E::EPB, float, float, float><<<g, E::EPB * E::N, 0, st>>>(
        M.blk, M.W, c->d_nbe, x, b, r, x_out, c->B, flags, c->T.P, M.r1);
  bump();
  CKL(c);
  return DG_OK;
}

int residual32(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags, cudaStream_t st) {
  return c->D == 3 ? launch_residual32<3>(c, x, b, r, x_out, flags, st)
                   : launch_residual32<2>(c, x, b, r, x_out, flags, st);
}

// residual / smoothing with the BF16 block copies (FP32 vectors and sums)
template <int D>
int launch_residual16(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags,
                      cudaStream_t st) {
  using E = Elem<D>;
  Mixed& M = mixed_of(c);
  unsigned g = nblk(c->B, E::EPB);
  if (g)
    residual_kernel<E::N, E::F, E::EPB, __nv_bfloat16, float, float><<<g, E::EPB * E::N, 0, st>>>(
        M.blk16, M.W16, c->d_nbe, x, b, r, x_out, c->B, flags, c->T.P, M.r1);
  bump();
  CKL(c);
  return DG_OK;
}

// residual in the preconditioner: BF16 blocks when enabled, FP32 otherwise
int residual_pc(dg_ctx* c, const float* x, const float* b, float* r, float* x_out, int flags, cudaStream_t st) {
  if (c->precond_bf16)
    return c->D == 3 ? launch_residual16<3>(c, x, b, r, x_out, flags, st)
                     : launch_residual16<2>(c, x, b, r, x_out, flags, st);
  return residual32(c, x, b, r, x_out, flags, st);
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
    prolong_cg_kernel<E::N, E::NC, float><<<nblk(c->B * E::N, 256), 256, 0, st>>>(
        x_add, e_sfc, c->d_pos, c->d_p1cg, c->d_wdg, c->T.P, nullptr, 0, c->B, 1);
    bump();
  }
  CKL(c);
  return DG_OK;
}

int transfer32(dg_ctx* c, const float* r, float* cg_out, float* x_add, const float* e_sfc, cudaStream_t st) {
  return c->D == 3 ? launch_transfer32<3>(c, r, cg_out, x_add, e_sfc, st)
                   : launch_transfer32<2>(c, r, cg_out, x_add, e_sfc, st);
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
    const int lc = M.dense_l;
    if (lc == 0) {
      CK(c, cudaMemcpyAsync(M.lev[0].r, r_sfc, sizeof(float) * M.lev[0].n, cudaMemcpyDeviceToDevice, st));
    } else {
      CK(c, cudaMemcpyAsync(M.lev[0].r, r_sfc, sizeof(float) * M.lev[0].n, cudaMemcpyDeviceToDevice, st));
      CK(c, cudaMemsetAsync(M.lev[0].e, 0, sizeof(float) * M.lev[0].n, st));
    }
    for (int l = 0; l < lc; ++l) {
      Lev32& L = M.lev[l];
      for (int it = 0; it < c->cfg.pre_smooth_its; ++it) {
        lev_jacobi_kernel<float><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag,
                                                                             L.e, L.r, L.e2, nullptr, L.n, w);
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
    {
      Lev32& L = M.lev[lc];
      dense_matvec_kernel<<<nblk(L.n, 8), 256, 0, st>>>(M.dense_inv, L.r, L.e, L.n);
      bump();
    }
    for (int l = lc - 1; l >= 0; --l) {
      Lev32& L = M.lev[l];
      lev_prolong_kernel<float><<<nblk(L.n, TB), TB, 0, st>>>(L.e, M.lev[l + 1].e, L.up, L.n);
      bump();
      for (int it = 0; it < c->cfg.post_smooth_its; ++it) {
        lev_jacobi_kernel<float><<<nblk((int64_t)L.n * LPR, TB), TB, 0, st>>>(L.rowptr, L.col, L.val, L.diag,
                                                                             L.e, L.r, L.e2, nullptr, L.n, w);
        bump();
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

// z = M32^{-1} r (FP32, same schedule as precond()); scratch t3, t4, t5
int precond32(dg_ctx* c, const float* r, float* z, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  const int nsm = c->cfg.pre_smooth_its;
  float* cur = M.t3;
  float* other = M.t4;
  if (nsm > 0) {
    if ((rc = residual_pc(c, nullptr, r, nullptr, cur, RF_ZEROX | RF_SMOOTH, st))) return rc;
    for (int it = 1; it < nsm; ++it) {
      if ((rc = residual_pc(c, cur, r, nullptr, other, RF_SMOOTH, st))) return rc;
      std::swap(cur, other);
    }
  } else {
    CK(c, cudaMemsetAsync(cur, 0, sizeof(float) * c->nonods, st));
  }
  if ((rc = residual_pc(c, cur, r, nullptr, nullptr, RF_RESTRICT, st))) return rc;   // -> M.r1
  if ((rc = gather_cg<float>(c, M.r1, M.cg1, true, st))) return rc;
  if ((rc = vcycle32(c, M.cg1, st))) return rc;
  if ((rc = transfer32(c, nullptr, nullptr, cur, M.lev[0].e, st))) return rc;
  for (int it = 0; it < nsm; ++it) {
    float* out = (it == nsm - 1) ? z : other;
    if ((rc = residual_pc(c, cur, r, nullptr, out, RF_SMOOTH, st))) return rc;
    other = cur;
    cur = out;
  }
  if (nsm == 0) CK(c, cudaMemcpyAsync(z, cur, sizeof(float) * c->nonods, cudaMemcpyDeviceToDevice, st));
  return DG_OK;
}

__global__ void convert_f64_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)a[k];
}

__global__ void convert_f64_bf16_kernel(const double* __restrict__ a, __nv_bfloat16* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = __float2bfloat16_rn((float)a[k]);
}

int build_mixed(dg_ctx* c, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  const size_t nb = (size_t)c->B * (c->F + 1) * c->N * c->N;
  const size_t nw = (size_t)c->B * c->N * c->N;
  if (!M.blk) {
    if ((rc = dalloc(c, &M.blk, nb))) return rc;
    if ((rc = dalloc(c, &M.W, nw))) return rc;
    for (float** t : {&M.t1, &M.t2, &M.t3, &M.t4, &M.t5, &M.t6})
      if ((rc = dalloc(c, t, (size_t)c->nonods))) return rc;
    if ((rc = dalloc(c, &M.cg1, (size_t)c->ncg))) return rc;
    if ((rc = dalloc(c, &M.r1, (size_t)c->B * c->NC))) return rc;
  }
  convert_f64_f32_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk, (int64_t)nb);
  bump();
  // smoother matrices of the mixed preconditioner
  const double* Wsrc = c->d_W;
  double* Winv = nullptr;
  if (c->mixed_smoother == 1) {
    CK(c, cudaMalloc((void**)&Winv, sizeof(double) * nw));
    CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
    if (c->D == 3)
      block_inverse_kernel<20, 4><<<(unsigned)c->B, 400, 0, st>>>(c->d_blk, Winv, c->B, c->mixed_smooth_w, c->d_err);
    else
      block_inverse_kernel<10, 3><<<(unsigned)c->B, 100, 0, st>>>(c->d_blk, Winv, c->B, c->mixed_smooth_w, c->d_err);
    bump();
    Wsrc = Winv;
  }
  convert_f64_f32_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(Wsrc, M.W, (int64_t)nw);
  bump();
  if (c->precond_bf16) {
    if (!M.blk16) {
      if ((rc = dalloc(c, &M.blk16, nb))) return rc;
      if ((rc = dalloc(c, &M.W16, nw))) return rc;
    }
    convert_f64_bf16_kernel<<<nblk((int64_t)nb, 256), 256, 0, st>>>(c->d_blk, M.blk16, (int64_t)nb);
    bump();
    convert_f64_bf16_kernel<<<nblk((int64_t)nw, 256), 256, 0, st>>>(Wsrc, M.W16, (int64_t)nw);
    bump();
  }
  if (Winv) {
    int herr = 0;
    CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    cudaFree(Winv);
    if (herr) return fail(c, DG_ERR_NUMERIC, "element block with a non-positive pivot (not positive definite)");
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
      CK(c, cudaMemcpy(&nnz, D.rowptr + D.n, sizeof(int), cudaMemcpyDeviceToHost));
      if ((rc = dalloc(c, &L.val, (size_t)nnz))) return rc;
      for (float** t : {&L.diag, &L.e, &L.e2, &L.r, &L.rr})
        if ((rc = dalloc(c, t, (size_t)L.n))) return rc;
    }
  }
  for (size_t l = 0; l < c->lev.size(); ++l) {
    Lev32& L = M.lev[l];
    const DevLevel& D = c->lev[l];
    int nnz = 0;
    CK(c, cudaMemcpy(&nnz, D.rowptr + D.n, sizeof(int), cudaMemcpyDeviceToHost));
    convert_f64_f32_kernel<<<nblk(nnz, 256), 256, 0, st>>>(D.val, L.val, nnz);
    bump();
    convert_f64_f32_kernel<<<nblk(D.n, 256), 256, 0, st>>>(D.diag, L.diag, D.n);
    bump();
  }
  // exact coarse solve on the first level with at most dense_max rows
  M.dense_l = -1;
  if (c->dense_max32 > 0) {
    const SfcHierarchy& h = c->sfc_h;
    int lc = -1;
    for (int l = 0; l < h.nlevel; ++l)
      if (h.sizes[l] <= c->dense_max32) { lc = l; break; }
    if (lc >= 0) {
      const int n = (int)h.sizes[lc];
      std::vector<double> A((size_t)n * n, 0.0), inv;
      const int64_t r0 = h.start[lc];
      for (int i = 0; i < n; ++i)
        for (int64_t k = h.row_ptr[r0 + i]; k < h.row_ptr[r0 + i + 1]; ++k) A[(size_t)i * n + h.col[k]] += h.val[k];
      if (invert_dense(A, n, inv)) {
        std::vector<float> invf(inv.begin(), inv.end());
        if (!M.dense_inv || c->dense_n != n) {
          if ((rc = dalloc(c, &M.dense_inv, (size_t)n * n))) return rc;
          c->dense_n = n;
        }
        CK(c, cudaMemcpy(M.dense_inv, invf.data(), sizeof(float) * invf.size(), cudaMemcpyHostToDevice));
        M.dense_l = lc;
      }
    }
  }
  CKL(c);
  M.built = true;
  return DG_OK;
}

int ensure_krylov32(dg_ctx* c, int m) {
  Mixed& M = mixed_of(c);
  if (M.vcap >= m + 1) return DG_OK;
  int rc;
  if ((rc = dalloc(c, &M.V, (size_t)(m + 1) * c->nonods))) return rc;
  if ((rc = dalloc(c, &M.Z, (size_t)m * c->nonods))) return rc;
  if ((rc = dalloc(c, &M.H, (size_t)(m + 1) * m))) return rc;
  M.vcap = m + 1;
  return DG_OK;
}

int norm32(dg_ctx* c, const float* z, double* out, cudaStream_t st) { return norm_t<float>(c, z, out, st); }

// CGS2 of w against V[0..j] (FP32 vectors, FP64 accumulation); writes the
// FP64 Hessenberg column j and V[j+1].
int cgs2_32(dg_ctx* c, int j, float* w, int m, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  return cgs2_t<float>(c, M.V, M.H, j, w, m, st);
}

// inner Arnoldi steps j0 .. j0+cnt-1: z_j = M v_j (kept), w = A z_j, CGS2
int arnoldi32_steps(dg_ctx* c, int j0, int cnt, int m, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  int rc;
  for (int j = j0; j < j0 + cnt; ++j) {
    float* zj = M.Z + (size_t)j * c->nonods;
    if ((rc = precond32(c, M.V + (size_t)j * c->nonods, zj, st))) return rc;
    if ((rc = residual32(c, zj, nullptr, M.t1, nullptr, RF_NEG, st))) return rc;   // t1 = A z_j
    if ((rc = cgs2_32(c, j, M.t1, m, st))) return rc;
  }
  return DG_OK;
}

int run_arnoldi32(dg_ctx* c, int j0, int cnt, int m, int chunk, cudaStream_t st) {
  Mixed& M = mixed_of(c);
  if (!c->use_graph) return arnoldi32_steps(c, j0, cnt, m, st);
  if (M.g_m != m || M.g_chunk != chunk || M.g_vptr != M.V) {
    for (auto& g : M.graphs)
      if (g) cudaGraphExecDestroy(g);
    M.graphs.assign((m + chunk - 1) / chunk, nullptr);
    M.g_m = m;
    M.g_chunk = chunk;
    M.g_vptr = M.V;
  }
  const int gi = j0 / chunk;
  if (cnt != std::min(chunk, m - j0) || j0 % chunk) return arnoldi32_steps(c, j0, cnt, m, st);
  if (!M.graphs[gi]) {
    if (!c->cap_stream) CK(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    CK(c, cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    int rc = arnoldi32_steps(c, j0, cnt, m, c->cap_stream);
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
  CK(c, cudaGraphLaunch(M.graphs[gi], st));
  return DG_OK;
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
  }
  if ((rc = ensure_krylov32(c, m))) return rc;
  const int chunk = std::min(10, m);
  const int64_t n = c->nonods;
  double* r64 = c->d_t2;
  float* rhs32 = M.t2;
  float* d32 = M.t6;
  float* V0 = M.V;
  if ((rc = residual(c, x, b, r64, nullptr, 0, st))) return rc;
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
      int k = 0;
      bool conv = false, ok = true;
      for (int j0 = 0; j0 < m; j0 += chunk) {
        const int cnt = std::min(chunk, m - j0);
        if ((rc = run_arnoldi32(c, j0, cnt, m, chunk, st))) return rc;
        its += cnt;
        k = j0 + cnt;
        CK(c, cudaMemcpyAsync(Hh.data(), M.H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
        CK(c, cudaStreamSynchronize(st));
        double est = hessenberg_ls(Hh, m, k, beta, y, ok);
        if (!ok) break;
        if (est <= target * beta0) {
          conv = true;
          break;
        }
        if (its >= max_its) break;
      }
      if (!ok) {
        status = DG_ERR_NUMERIC;
        c->err = "mixed solve: singular Hessenberg matrix";
        break;
      }
      CK(c, cudaMemcpyAsync(c->d_y, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
      combine_kernel<float, float><<<nblk(n, 256), 256, 0, st>>>(M.Z, n, k, c->d_y, d32, n, 1.0);
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
  return residual_pc(c, x, b, nullptr, x_out, RF_SMOOTH, st);
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
