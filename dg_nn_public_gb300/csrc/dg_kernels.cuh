// Device kernels of libdgsip (FP64 path).
//
// Operator storage.  The SIP-DG operator is kept as dense element blocks:
// for element e, block 0 is the element's own block A_ee (volume term plus
// the own-side terms of its interior and Dirichlet faces -- exactly the
// reference's bdiagK) and block 1+f is the coupling A_{e,nb(e,f)} to the
// face-f neighbour (zero for boundary faces).  Blocks are stored
// column-major, blk[((e*(F+1)+b)*N + n)*N + m] = A_b(m, n), so that the
// threads of an element (one per row m) read a column with one coalesced
// 8*N-byte access.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace dg {

struct Tables {
  const double* n;        // (N, VG)
  const double* nlx;      // (D, N, VG)
  const double* weight;   // (VG)
  const double* sn;       // (F, N, SG)
  const double* snlx;     // (F, D, N, SG)
  const double* sweight;  // (SG)
  const double* drst;     // (F, D, D-1)
  const double* P;        // (N, D+1) P1 -> P3 element prolongator
  const int* align;       // (D, SG)
};

struct BuildParams {
  Tables T;
  const double* x;        // (B, D, N)
  const int* nbe;         // (B*F) neighbour element (interior faces) or -1
  const int* nbface;      // (B*F) neighbour local face
  const int* aln;         // (B*F)
  const int* bct;         // (B*F)
  const double* kappa;    // (B)
  double* blk;            // (B, F+1, N, N)
  double* detw;           // (B, VG) signed det * weight
  double eta, mu;
  int64_t B;
  int* err;               // error word: 1 = non-positive Jacobian
  int face_kappa;         // interior-face kappa: 0 = (ke + kn) / 2, 1 = 2 ke kn / (ke + kn)
};

// ---------------------------------------------------------------------------
// small dense helpers
template <int D>
__device__ __forceinline__ double inv_det(const double* j, double* inv) {
  // j[i*D+k] = d x_k / d l_i; inverse by cofactors like the reference
  if constexpr (D == 3) {
    double det = j[0] * (j[4] * j[8] - j[5] * j[7]) - j[1] * (j[3] * j[8] - j[5] * j[6]) +
                 j[2] * (j[3] * j[7] - j[4] * j[6]);
    inv[0] = (j[4] * j[8] - j[5] * j[7]) / det;
    inv[1] = (j[2] * j[7] - j[1] * j[8]) / det;
    inv[2] = (j[1] * j[5] - j[2] * j[4]) / det;
    inv[3] = (j[5] * j[6] - j[3] * j[8]) / det;
    inv[4] = (j[0] * j[8] - j[2] * j[6]) / det;
    inv[5] = (j[2] * j[3] - j[0] * j[5]) / det;
    inv[6] = (j[3] * j[7] - j[4] * j[6]) / det;
    inv[7] = (j[1] * j[6] - j[0] * j[7]) / det;
    inv[8] = (j[0] * j[4] - j[1] * j[3]) / det;
    return det;
  } else {
    double det = j[0] * j[3] - j[1] * j[2];
    inv[0] = j[3] / det;
    inv[1] = -j[1] / det;
    inv[2] = -j[2] / det;
    inv[3] = j[0] / det;
    return det;
  }
}

// Jacobian at one point from derivative table d (D, N, npts) at column g.
template <int D, int N>
__device__ __forceinline__ void jacobian(const double* __restrict__ d, int npts, int g,
                                         const double* xe, double* j) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int k = 0; k < D; ++k) {
      double s = 0.0;
#pragma unroll 4
      for (int n = 0; n < N; ++n) s += __ldg(d + (i * N + n) * npts + g) * xe[k * N + n];
      j[i * D + k] = s;
    }
}

// Face tangents, unit outward normal and area element at a face point.
template <int D>
__device__ __forceinline__ double face_normal(const double* j, const double* drst_f, double* nrm) {
  if constexpr (D == 3) {
    double t[2][3];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) s += j[i * 3 + c] * drst_f[i * 2 + k];
        t[k][c] = s;
      }
    double cx = t[0][1] * t[1][2] - t[0][2] * t[1][1];
    double cy = t[0][2] * t[1][0] - t[0][0] * t[1][2];
    double cz = t[0][0] * t[1][1] - t[0][1] * t[1][0];
    double sdet = sqrt(cx * cx + cy * cy + cz * cz);
    nrm[0] = cx / sdet;
    nrm[1] = cy / sdet;
    nrm[2] = cz / sdet;
    return sdet;
  } else {
    double t0 = j[0] * drst_f[0] + j[2] * drst_f[1];
    double t1 = j[1] * drst_f[0] + j[3] * drst_f[1];
    double sdet = sqrt(t0 * t0 + t1 * t1);
    nrm[0] = t1 / sdet;
    nrm[1] = -t0 / sdet;
    return sdet;
  }
}

// ---------------------------------------------------------------------------
// Stored-block assembly: one CTA per element, N*N threads.
template <int D, int N, int F, int VG, int SG>
struct BuildSmem {
  double xe[D * N];
  double xnb[F][D * N];
  double ivj[VG][D * D];
  double dtw[VG];
  double nx[D][N][VG];
  double nrm[F][SG][D];
  double sw[F][SG];
  double ivs[F][SG][D * D];
  double ivsn[F][SG][D * D];
  double gn[F][N][SG];
  double gnb[F][N][SG];
  double snb[F][N][SG];
  double gam[F];
  double kf[F];
  int nbi[F], nbfc[F], aln[F], bct[F];
};

template <int D, int N, int F, int VG, int SG>
__global__ void __launch_bounds__(N* N) build_blocks_kernel(BuildParams p) {
  using S = BuildSmem<D, N, F, VG, SG>;
  extern __shared__ double smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  const int NT = N * N;
  const Tables& T = p.T;
  for (int k = tid; k < D * N; k += NT) s.xe[k] = p.x[e * D * N + k];
  if (tid < F) {
    int64_t fi = e * F + tid;
    s.nbi[tid] = p.nbe[fi];
    s.nbfc[tid] = p.nbface[fi];
    s.aln[tid] = p.aln[fi];
    s.bct[tid] = p.bct[fi];
  }
  __syncthreads();
  for (int k = tid; k < F * D * N; k += NT) {
    int f = k / (D * N), r = k % (D * N);
    int nb = s.nbi[f];
    s.xnb[f][r] = nb >= 0 ? p.x[(int64_t)nb * D * N + r] : 0.0;
  }
  __syncthreads();
  // volume Jacobians
  for (int g = tid; g < VG; g += NT) {
    double j[D * D];
    jacobian<D, N>(T.nlx, VG, g, s.xe, j);
    double det = inv_det<D>(j, s.ivj[g]);
    s.dtw[g] = det * T.weight[g];
    if (!(det > 0.0)) atomicExch(p.err, 1);
    p.detw[e * VG + g] = det * T.weight[g];
  }
  // face Jacobians: own side and (interior faces) neighbour side
  for (int k = tid; k < F * SG; k += NT) {
    int f = k / SG, g = k % SG;
    double j[D * D];
    jacobian<D, N>(T.snlx + (size_t)f * D * N * SG, SG, g, s.xe, j);
    inv_det<D>(j, s.ivs[f][g]);
    double sdet = face_normal<D>(j, T.drst + f * D * (D - 1), s.nrm[f][g]);
    s.sw[f][g] = sdet * T.sweight[g];
    if (s.nbi[f] >= 0) {
      int fn = s.nbfc[f];
      jacobian<D, N>(T.snlx + (size_t)fn * D * N * SG, SG, g, s.xnb[f], j);
      inv_det<D>(j, s.ivsn[f][g]);
    }
  }
  __syncthreads();
  // physical gradients at volume points
  for (int k = tid; k < D * N * VG; k += NT) {
    int i = k / (N * VG), r = k % (N * VG), n = r / VG, g = r % VG;
    double v = 0.0;
#pragma unroll
    for (int jj = 0; jj < D; ++jj) v += s.ivj[g][i * D + jj] * __ldg(T.nlx + (jj * N + n) * VG + g);
    s.nx[i][n][g] = v;
  }
  // grad(phi).n on the faces, own side and neighbour side at aligned points
  for (int k = tid; k < F * N * SG; k += NT) {
    int f = k / (N * SG), r = k % (N * SG), n = r / SG, g = r % SG;
    const double* snlx_f = T.snlx + (size_t)f * D * N * SG;
    double v = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double gi = 0.0;
#pragma unroll
      for (int jj = 0; jj < D; ++jj) gi += s.ivs[f][g][i * D + jj] * __ldg(snlx_f + (jj * N + n) * SG + g);
      v += gi * s.nrm[f][g][i];
    }
    s.gn[f][n][g] = v;
    double vb = 0.0, sb = 0.0;
    if (s.nbi[f] >= 0) {
      int fn = s.nbfc[f];
      int a = T.align[s.aln[f] * SG + g];
      const double* snlx_n = T.snlx + (size_t)fn * D * N * SG;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        double gi = 0.0;
#pragma unroll
        for (int jj = 0; jj < D; ++jj) gi += s.ivsn[f][a][i * D + jj] * __ldg(snlx_n + (jj * N + n) * SG + a);
        vb += gi * s.nrm[f][g][i];
      }
      sb = __ldg(T.sn + ((size_t)fn * N + n) * SG + a);
    }
    s.gnb[f][n][g] = vb;
    s.snb[f][n][g] = sb;
  }
  if (tid < F) {
    int f = tid;
    double h = 0.0;
    for (int g = 0; g < SG; ++g) h += s.sw[f][g];
    if (D == 3) h = sqrt(h);
    s.gam[f] = p.eta / h;
    double ke = p.kappa[e];
    if (s.bct[f] < 0) {
      int nb = s.nbi[f];
      const double kn = nb >= 0 ? p.kappa[nb] : ke;
      s.kf[f] = p.mu * (p.face_kappa ? 2.0 * ke * kn / (ke + kn) : 0.5 * (ke + kn));
    } else if (s.bct[f] == 0) {
      s.kf[f] = p.mu * ke;
    } else {
      s.kf[f] = 0.0;
    }
  }
  __syncthreads();
  // entries: thread -> (m, n), m fastest
  const int m = tid % N, n = tid / N;
  double vol = 0.0;
#pragma unroll 4
  for (int g = 0; g < VG; ++g) {
    double dd = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) dd += s.nx[i][m][g] * s.nx[i][n][g];
    vol += s.dtw[g] * dd;
  }
  double diag = p.mu * p.kappa[e] * vol;
  double* out = p.blk + (size_t)e * (F + 1) * N * N;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const double* snf = T.sn + (size_t)f * N * SG;
    double off = 0.0;
    if (s.kf[f] != 0.0) {
      const bool interior = s.bct[f] < 0;
      const double a = interior ? 0.5 : 1.0;
      double cs = 0.0, sc = 0.0, ss = 0.0, cnb = 0.0, snbv = 0.0, ssnb = 0.0;
      for (int g = 0; g < SG; ++g) {
        double w = s.sw[f][g];
        double snm = __ldg(snf + m * SG + g), snn = __ldg(snf + n * SG + g);
        cs += snm * s.gn[f][n][g] * w;
        sc += s.gn[f][m][g] * snn * w;
        ss += snm * snn * w;
        if (interior) {
          cnb += snm * s.gnb[f][n][g] * w;
          snbv += s.gn[f][m][g] * s.snb[f][n][g] * w;
          ssnb += snm * s.snb[f][n][g] * w;
        }
      }
      diag += s.kf[f] * (-a * cs - a * sc + s.gam[f] * ss);
      if (interior) off = s.kf[f] * (-0.5 * cnb + 0.5 * snbv - s.gam[f] * ssnb);
    }
    out[(size_t)(1 + f) * N * N + n * N + m] = off;
  }
  out[n * N + m] = diag;
}

// ---------------------------------------------------------------------------
// Stored-block assembly for straight-sided (affine) elements.  With a
// constant Jacobian J (inverse M, determinant det), a constant unit normal
// n_f and area element sdet_f per face, every quadrature sum of the general
// kernel factors into a geometric coefficient times a reference matrix that
// is the same for all elements (ftab, formed once per context on the host):
//   volume   det * sum_{jj,kk} (M^T M)[jj][kk] K[jj][kk]
//   cs, sc   sdet_f * sum_jj c_f[jj] R[f][jj] (and its transpose),
//            c_f = M^T n_f
//   ss       sdet_f * Mf[f]
//   cnb      sdet_f * sum_jj cn_f[jj] Q[f][fn][al][jj], cn_f = M_nb^T n_f
//   snbv     sdet_f * sum_jj c_f[jj] P[f][fn][al][jj]
//   ssnb     sdet_f * S[f][fn][al]
// with al the face's alignment code and fn the neighbour's local face, so the
// blocks equal the general kernel's to rounding (tested).  Table layout:
// K (D*D), R (F*D), Mf (F), Q (F*F*D*D), P (F*F*D*D), S (F*F*D) matrices of
// N*N doubles, entry (m, n) at [m * N + n].
template <int D, int N, int F>
struct FastTab {
  static constexpr int NN = N * N;
  static constexpr int K = 0;
  static constexpr int R = K + D * D * NN;
  static constexpr int Mf = R + F * D * NN;
  static constexpr int Q = Mf + F * NN;
  static constexpr int P = Q + F * F * D * D * NN;
  static constexpr int S = P + F * F * D * D * NN;
  static constexpr int Size = S + F * F * D * NN;
};

// Per-element geometry of the affine build, kappa-free and fixed for a
// context (the coordinates do not change): det, C = Mi^T Mi, and per face
// the area element sdet, the penalty gam = eta / h, cf = Mi^T n and the
// neighbour's cn = Mn^T n.  One thread per element, so the FP64 work of the
// Jacobians and inverses runs in full warps (on the GB300 a warp's FP64
// instruction occupies its SM partition's FP64 pipe for the whole warp
// whether one lane is active or 32); the record is GeomRec<D, F>::Size
// doubles, and detw is written here too.
template <int D, int F>
struct GeomRec {
  static constexpr int Det = 0, C = 1, Face = 1 + D * D, PerFace = 2 + 2 * D;
  static constexpr int Size = Face + F * PerFace;
};

template <int D, int N, int F, int VG, int SG>
__global__ void __launch_bounds__(128) geom_affine_kernel(BuildParams p, double* __restrict__ geom) {
  using G = GeomRec<D, F>;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.B) return;
  const Tables& T = p.T;
  double* rec = geom + e * G::Size;
  double j[D * D], Mi[D * D];
  jacobian<D, N>(T.nlx, VG, 0, p.x + e * D * N, j);
  const double det = inv_det<D>(j, Mi);
  if (!(det > 0.0)) atomicExch(p.err, 1);
  rec[G::Det] = det;
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) {
      double t = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) t += Mi[i * D + a] * Mi[i * D + b];
      rec[G::C + a * D + b] = t;
    }
  for (int g = 0; g < VG; ++g) p.detw[e * VG + g] = det * T.weight[g];
  for (int f = 0; f < F; ++f) {
    double* fr = rec + G::Face + f * G::PerFace;
    double nrm[D];
    const double sd = face_normal<D>(j, T.drst + f * D * (D - 1), nrm);
    fr[0] = sd;
    double h = 0.0;
    for (int g = 0; g < SG; ++g) h += sd * T.sweight[g];
    if (D == 3) h = sqrt(h);
    fr[1] = p.eta / h;
#pragma unroll
    for (int jj = 0; jj < D; ++jj) {
      double t = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) t += Mi[i * D + jj] * nrm[i];
      fr[2 + jj] = t;
    }
    const int nb = p.nbe[e * F + f];
    if (nb >= 0) {
      double jn[D * D], mn[D * D];
      jacobian<D, N>(T.nlx, VG, 0, p.x + (int64_t)nb * D * N, jn);
      inv_det<D>(jn, mn);
#pragma unroll
      for (int jj = 0; jj < D; ++jj) {
        double t = 0.0;
#pragma unroll
        for (int i = 0; i < D; ++i) t += mn[i * D + jj] * nrm[i];
        fr[2 + D + jj] = t;
      }
    } else {
#pragma unroll
      for (int jj = 0; jj < D; ++jj) fr[2 + D + jj] = 0.0;
    }
  }
}

// Blocks of straight-sided elements from the geometry record and the
// kappa-dependent face coefficients: one CTA per element, one thread per
// block entry, no serial phase (the record is read into shared memory).
template <int D, int N, int F, int VG, int SG>
__global__ void __launch_bounds__(N* N) build_blocks_affine_kernel(BuildParams p, const double* __restrict__ ftab,
                                                                   const double* __restrict__ geom) {
  using TB = FastTab<D, N, F>;
  using G = GeomRec<D, F>;
  constexpr int NN = N * N;
  __shared__ double rec[G::Size];
  __shared__ double kf[F];
  __shared__ int nbi[F], nbfc[F], aln[F], bct[F];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  for (int k = tid; k < G::Size; k += NN) rec[k] = geom[e * G::Size + k];
  if (tid < F) {
    const int64_t fi = e * F + tid;
    const int f = tid;
    nbi[f] = p.nbe[fi];
    nbfc[f] = p.nbface[fi];
    aln[f] = p.aln[fi];
    bct[f] = p.bct[fi];
    const double ke = p.kappa[e];
    if (bct[f] < 0) {
      const int nb = nbi[f];
      const double kn = nb >= 0 ? p.kappa[nb] : ke;
      kf[f] = p.mu * (p.face_kappa ? 2.0 * ke * kn / (ke + kn) : 0.5 * (ke + kn));
    } else if (bct[f] == 0) {
      kf[f] = p.mu * ke;
    } else {
      kf[f] = 0.0;
    }
  }
  __syncthreads();
  const double* C = rec + G::C;
  const double det_s = rec[G::Det];
  const int m = tid % N, n = tid / N;
  const int mn_ = m * N + n, nm_ = n * N + m;
  double vol = 0.0;
#pragma unroll
  for (int a = 0; a < D * D; ++a) vol += C[a] * __ldg(ftab + TB::K + a * NN + mn_);
  double diag = p.mu * p.kappa[e] * det_s * vol;
  double* out = p.blk + (size_t)e * (F + 1) * N * N;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const double* fr = rec + G::Face + f * G::PerFace;
    const double sdet = fr[0], gam = fr[1];
    const double* cf = fr + 2;
    const double* cn = fr + 2 + D;
    double off = 0.0;
    if (kf[f] != 0.0) {
      const bool interior = bct[f] < 0;
      const double a = interior ? 0.5 : 1.0;
      double cs = 0.0, sc = 0.0;
#pragma unroll
      for (int jj = 0; jj < D; ++jj) {
        const double* R = ftab + TB::R + (f * D + jj) * NN;
        cs += cf[jj] * __ldg(R + mn_);
        sc += cf[jj] * __ldg(R + nm_);
      }
      const double ss = __ldg(ftab + TB::Mf + f * NN + mn_);
      diag += kf[f] * sdet * (-a * cs - a * sc + gam * ss);
      if (interior) {
        const int cmb = (f * F + nbfc[f]) * D + aln[f];
        double cnb = 0.0, snbv = 0.0;
#pragma unroll
        for (int jj = 0; jj < D; ++jj) {
          cnb += cn[jj] * __ldg(ftab + TB::Q + (cmb * D + jj) * NN + mn_);
          snbv += cf[jj] * __ldg(ftab + TB::P + (cmb * D + jj) * NN + mn_);
        }
        const double ssnb = __ldg(ftab + TB::S + cmb * NN + mn_);
        off = kf[f] * sdet * (-0.5 * cnb + 0.5 * snbv - gam * ssnb);
      }
    }
    out[(size_t)(1 + f) * N * N + n * N + m] = off;
  }
  out[n * N + m] = diag;
}

// Largest deviation of the volume-point Jacobians of an element from its
// first one, relative to the largest entry (0 for straight-sided elements);
// the maximum over elements goes to *dev (bit pattern of a non-negative
// double, so an integer maximum orders it).
template <int D, int N, int VG>
__global__ void affine_check_kernel(const double* __restrict__ x, const double* __restrict__ nlx, int64_t B,
                                    unsigned long long* dev) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= B) return;
  double xe[D * N];
#pragma unroll
  for (int k = 0; k < D * N; ++k) xe[k] = x[e * D * N + k];
  double j0[D * D], j[D * D];
  jacobian<D, N>(nlx, VG, 0, xe, j0);
  double big = 0.0, d = 0.0;
#pragma unroll
  for (int k = 0; k < D * D; ++k) big = fmax(big, fabs(j0[k]));
  for (int g = 1; g < VG; ++g) {
    jacobian<D, N>(nlx, VG, g, xe, j);
#pragma unroll
    for (int k = 0; k < D * D; ++k) d = fmax(d, fabs(j[k] - j0[k]));
  }
  const double rel = big > 0.0 ? d / big : 1.0;
  atomicMax(dev, (unsigned long long)__double_as_longlong(rel));
}

// ---------------------------------------------------------------------------
// Smoother matrix.  The reference smooths with three point-Jacobi sweeps on
// each element block, c <- c + w D^-1 (r - A_ee c) from c = 0, then
// x += w c (z06/volume_mf_diff.py:474-480).  That is the fixed linear map
// x += W_e r with W_e = w^2 (I + G + G^2) D^-1, G = I - w D^-1 A_ee, which is
// formed once per operator here (one CTA per element, N*N threads) and
// stored column-major like the blocks.
template <int N, int F>
__global__ void __launch_bounds__(N* N) smoother_matrix_kernel(const double* __restrict__ blk,
                                                               double* __restrict__ W, int64_t B,
                                                               double w) {
  __shared__ double G[N][N];
  __shared__ double G2[N][N];
  __shared__ double dinv[N];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  const int m = tid % N, n = tid / N;                 // entry (m, n)
  const double* A = blk + (size_t)e * (F + 1) * N * N; // A(m, n) at [n*N + m]
  if (tid < N) dinv[tid] = 1.0 / A[tid * N + tid];
  __syncthreads();
  G[m][n] = (m == n ? 1.0 : 0.0) - w * dinv[m] * A[n * N + m];
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < N; ++k) s += G[m][k] * G[k][n];
  G2[m][n] = s;
  __syncthreads();
  const double poly = (m == n ? 1.0 : 0.0) + G[m][n] + G2[m][n];
  W[(size_t)e * N * N + n * N + m] = w * w * poly * dinv[n];
}

// Damped block inverse W_e = w A_ee^{-1} (the mixed preconditioner's
// smoother option), stored column-major like the blocks.  Gauss-Jordan in
// FP64 without pivoting: A_ee is symmetric positive definite for a
// sufficient penalty, so every pivot is positive (a non-positive pivot sets
// the error word and leaves W_e as the Jacobi inverse of the diagonal).
// One warp per element, lane m holding row m of [A_ee | I] in registers: per
// pivot one reciprocal, the pivot row broadcast by shuffles, and the row
// update in FP64 FMAs (FP64 throughput is what bounds this kernel, so the
// division is taken once per row and pivot, not per entry).
template <int N, int F>
__global__ void __launch_bounds__(256) block_inverse_kernel(const double* __restrict__ blk, double* __restrict__ W,
                                                            int64_t B, double w, int* err) {
  static_assert(N <= 32, "one lane per row");
  constexpr int WPB = 8;
  const int lane = threadIdx.x & 31;
  const int64_t e = (int64_t)blockIdx.x * WPB + (threadIdx.x >> 5);
  if (e >= B) return;   // whole warp
  const int m = lane < N ? lane : N - 1;   // lanes >= N repeat the last row, write nothing
  const double* A = blk + (size_t)e * (F + 1) * N * N;   // A(m, n) at [n * N + m]
  double a[N], inv[N];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    a[n] = A[n * N + m];
    inv[n] = (n == m) ? 1.0 : 0.0;
  }
  bool bad = false;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const double piv = __shfl_sync(0xffffffffu, a[k], k);
    if (!(piv > 0.0)) {   // uniform: every lane holds the same pivot
      bad = true;
      break;
    }
    const double rp = 1.0 / piv;
    const double fm = a[k];   // this row's entry in the pivot column
#pragma unroll
    for (int n = 0; n < N; ++n) {
      const double pa = __shfl_sync(0xffffffffu, a[n], k) * rp;
      const double pi = __shfl_sync(0xffffffffu, inv[n], k) * rp;
      if (m == k) {
        a[n] = pa;
        inv[n] = pi;
      } else {
        a[n] = fma(-fm, pa, a[n]);
        inv[n] = fma(-fm, pi, inv[n]);
      }
    }
  }
  if (lane >= N) return;
  double* Wo = W + (size_t)e * N * N;
  if (bad) {
    if (lane == 0) atomicExch(err, 2);
#pragma unroll
    for (int n = 0; n < N; ++n) Wo[n * N + m] = (m == n) ? w / A[m * N + m] : 0.0;
    return;
  }
#pragma unroll
  for (int n = 0; n < N; ++n) Wo[n * N + m] = w * inv[n];
}

// The same damped block inverse in FP32 (the mixed preconditioner stores
// its smoother matrices in FP32 / BF16): the FP64 block is read and rounded
// once, the elimination runs in FP32 FMAs.  W (FP32) in the same layout.
template <int N, int F>
__global__ void __launch_bounds__(256) block_inverse32_kernel(const double* __restrict__ blk, float* __restrict__ W,
                                                              int64_t B, float w, int* err) {
  static_assert(N <= 32, "one lane per row");
  constexpr int WPB = 8;
  const int lane = threadIdx.x & 31;
  const int64_t e = (int64_t)blockIdx.x * WPB + (threadIdx.x >> 5);
  if (e >= B) return;   // whole warp
  const int m = lane < N ? lane : N - 1;   // lanes >= N repeat the last row, write nothing
  const double* A = blk + (size_t)e * (F + 1) * N * N;   // A(m, n) at [n * N + m]
  float a[N], inv[N];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    a[n] = (float)A[n * N + m];
    inv[n] = (n == m) ? 1.0f : 0.0f;
  }
  bool bad = false;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const float piv = __shfl_sync(0xffffffffu, a[k], k);
    if (!(piv > 0.0f)) {   // uniform: every lane holds the same pivot
      bad = true;
      break;
    }
    const float rp = 1.0f / piv;
    const float fm = a[k];   // this row's entry in the pivot column
#pragma unroll
    for (int n = 0; n < N; ++n) {
      const float pa = __shfl_sync(0xffffffffu, a[n], k) * rp;
      const float pi = __shfl_sync(0xffffffffu, inv[n], k) * rp;
      if (m == k) {
        a[n] = pa;
        inv[n] = pi;
      } else {
        a[n] = fmaf(-fm, pa, a[n]);
        inv[n] = fmaf(-fm, pi, inv[n]);
      }
    }
  }
  if (lane >= N) return;
  float* Wo = W + (size_t)e * N * N;
  if (bad) {
    if (lane == 0) atomicExch(err, 2);
#pragma unroll
    for (int n = 0; n < N; ++n) Wo[n * N + m] = (m == n) ? w / (float)A[m * N + m] : 0.0f;
    return;
  }
#pragma unroll
  for (int n = 0; n < N; ++n) Wo[n * N + m] = w * inv[n];
}

// ---------------------------------------------------------------------------
// Residual / smoother: EPB elements per CTA, one thread per (element, row).
//   res = b - A x            (b = 0 when null; x = 0 when ZEROX)
//   r  <- sgn * res          (when r != null)
//   SMOOTH: x_out = x + W_e res  (the three-sweep block-Jacobi step)
enum { RF_ZEROX = 1, RF_SMOOTH = 2, RF_NEG = 4, RF_RESTRICT = 8, RF_STREAM_HINT = 16 };

// Programmatic dependent launch: wait until the preceding kernel of the
// stream has completed (its writes visible), then let the next kernel start
// its launch.  Triggering only after the wait means a kernel's pre-wait
// part can read anything produced two or more kernels back.  Both are
// no-ops for a kernel launched without the programmatic attribute.
__device__ __forceinline__ void pdl_wait_then_trigger() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// MT: stored matrix type; VT: vector type; AT: accumulation type.
template <int N, int F, int EPB, typename MT = double, typename VT = double, typename AT = double>
__global__ void __launch_bounds__(EPB* N) residual_kernel(const MT* __restrict__ blk,
                                                          const MT* __restrict__ W,
                                                          const int* __restrict__ nbe,
                                                          const VT* __restrict__ x,
                                                          const VT* __restrict__ b,
                                                          VT* __restrict__ r,
                                                          VT* __restrict__ x_out, int64_t B,
                                                          int flags, const double* __restrict__ P = nullptr,
                                                          VT* __restrict__ r1 = nullptr,
                                                          const float* __restrict__ wsp = nullptr) {
  const AT wscale = wsp ? (AT)*wsp : (AT)1;
  __shared__ AT xs[EPB][F + 1][N];
  __shared__ AT rs[EPB][N];
  __shared__ int nbs[EPB][F];
  const int le = threadIdx.x / N, m = threadIdx.x % N;
  const int64_t e = (int64_t)blockIdx.x * EPB + le;
  const bool valid = e < B;
  const bool zerox = flags & RF_ZEROX;
  if (valid && m < F) nbs[le][m] = nbe[e * F + m];
  __syncthreads();
  if (valid && !zerox) {
    xs[le][0][m] = (AT)x[e * N + m];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      int nb = nbs[le][f];
      xs[le][1 + f][m] = nb >= 0 ? (AT)x[(int64_t)nb * N + m] : (AT)0;
    }
  }
  __syncthreads();
  AT acc = 0;
  const MT* A = blk + (size_t)e * (F + 1) * N * N;
  if (valid && !zerox) {
#pragma unroll
    for (int n = 0; n < N; ++n) acc += (AT)A[n * N + m] * xs[le][0][n];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (nbs[le][f] >= 0) {
        const MT* Af = A + (size_t)(1 + f) * N * N;
#pragma unroll
        for (int n = 0; n < N; ++n) acc += (AT)Af[n * N + m] * xs[le][1 + f][n];
      }
    }
  }
  AT res = 0;
  if (valid) {
    res = (b ? (AT)b[e * N + m] : (AT)0) - acc;
    if (r) r[e * N + m] = (VT)((flags & RF_NEG) ? -res : res);
  }
  if (flags & RF_RESTRICT) {
    // P3 -> P1 element restriction of the residual (the DG->CG transfer
    // needs only these ncorner values per element)
    rs[le][m] = res;
    __syncthreads();
    constexpr int NC = F;   // corners = faces for simplices
    if (valid && m < NC) {
      AT s = 0;
#pragma unroll
      for (int n = 0; n < N; ++n) s += (AT)P[n * NC + m] * rs[le][n];
      r1[e * NC + m] = (VT)s;
    }
  }
  if (flags & RF_SMOOTH) {
    rs[le][m] = res;
    __syncthreads();
    if (valid) {
      const MT* We = W + (size_t)e * N * N;
      AT c = 0;
#pragma unroll
      for (int n = 0; n < N; ++n) c += (AT)We[n * N + m] * rs[le][n];
      x_out[e * N + m] = (VT)((zerox ? (AT)0 : xs[le][0][m]) + wscale * c);
    }
  }
}

}  // namespace dg
