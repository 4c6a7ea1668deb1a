// Host-only integer layer of libdgsip: P1CG sparsity, distance-2 colouring,
// SFC level hierarchy and face connectivity.  No CUDA calls: these entry
// points work on machines without a GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "dg_internal.h"

#include <atomic>
#include <thread>

namespace dg {

thread_local std::string g_thread_error;

int set_thread_error(int code, const std::string& msg) {
  g_thread_error = msg;
  return code;
}

// P1CG sparsity: union of all corner pairs of every element, each row sorted
// (sparsity.py:102-122; getfin_p1cg, get_neighbouring.f90:133-157, and the
// scipy COO->CSR conversion that sorts and merges duplicates).
int p1cg_sparsity(int64_t nele, int ncorner, const int64_t* p1cg, int64_t n,
                  std::vector<int64_t>& fina, std::vector<int64_t>& cola) {
  std::vector<std::vector<int64_t>> rows(n);
  for (int64_t e = 0; e < nele; ++e) {
    const int64_t* c = p1cg + e * ncorner;
    for (int a = 0; a < ncorner; ++a) {
      if (c[a] < 0 || c[a] >= n) return set_thread_error(DG_ERR_MESH, "p1cg vertex out of range");
      for (int b = 0; b < ncorner; ++b) rows[c[a]].push_back(c[b]);
    }
  }
  fina.assign(n + 1, 0);
  cola.clear();
  for (int64_t i = 0; i < n; ++i) {
    auto& r = rows[i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    cola.insert(cola.end(), r.begin(), r.end());
    fina[i + 1] = (int64_t)cola.size();
  }
  return DG_OK;
}

// Greedy distance-2 colouring, vertices visited in order, one colour per
// sweep (sparsity.py:235-269).
int color2(int64_t n, const int64_t* fina, const int64_t* cola, std::vector<int64_t>& whichc,
           int32_t& ncolor) {
  whichc.assign(n, 0);
  std::vector<char> need(n, 1);
  ncolor = 0;
  bool undone = n > 0;
  if (n == 0) { ncolor = 1; return DG_OK; }
  while (undone) {
    ++ncolor;
    for (int64_t i = 0; i < n; ++i) {
      if (!need[i]) continue;
      bool found = false;
      for (int64_t k = fina[i]; k < fina[i + 1] && !found; ++k) {
        int64_t j = cola[k];
        if (whichc[j] == ncolor) { found = true; break; }
        for (int64_t k2 = fina[j]; k2 < fina[j + 1]; ++k2)
          if (whichc[cola[k2]] == ncolor) { found = true; break; }
      }
      if (!found) whichc[i] = ncolor;
    }
    undone = false;
    for (int64_t i = 0; i < n; ++i) {
      need[i] = whichc[i] == 0;
      if (need[i]) undone = true;
    }
    if (ncolor > 100000) return set_thread_error(DG_ERR_STATE, "colouring did not terminate");
  }
  return DG_OK;
}

// For each colour: the first CSR entry of each row whose column has that
// colour (sparsity.py:272-306).
void sparse_idx_for_color(int64_t n, const int64_t* fina, const int64_t* cola,
                          const std::vector<int64_t>& whichc, int32_t ncolor,
                          std::vector<std::vector<int64_t>>& spidx,
                          std::vector<std::vector<int64_t>>& colidx) {
  spidx.assign(ncolor, {});
  colidx.assign(ncolor, {});
  for (int32_t c = 1; c <= ncolor; ++c) {
    for (int64_t i = 0; i < n; ++i) {
      for (int64_t k = fina[i]; k < fina[i + 1]; ++k) {
        if (whichc[cola[k]] == c) {
          colidx[c - 1].push_back(i);
          spidx[c - 1].push_back(k);
          break;
        }
      }
    }
  }
}

int32_t nlevel_sfc(int64_t nonods) {
  if (nonods <= 1) return 1;
  int64_t course = nonods;
  int32_t nlevel = 1;
  for (int il = 2; il <= 200; ++il) {
    int64_t fine = course;
    course = (fine - 1) / 2 + 1;
    nlevel = il;
    if (course == 1) break;
  }
  return nlevel;
}

// SFC level hierarchy (compact_fcode.f90:7-225).  Level l maps curve
// position s to coarse node s >> l; a coarse row lists its columns in the
// order they first appear while the fine rows are visited in curve order
// (each in CSR order), and its values are accumulated in that same order.
int sfc_levels(int64_t n, const int64_t* fina, const int64_t* cola, const double* a,
               const int64_t* sfc_order, SfcHierarchy& h, std::vector<std::vector<int64_t>>* visit_tgt) {
  h.nlevel = nlevel_sfc(n);
  std::vector<int64_t> pos(n), inv(n, -1);
  for (int64_t i = 0; i < n; ++i) {
    int64_t p = sfc_order[i] - 1;
    if (p < 0 || p >= n || inv[p] >= 0) return set_thread_error(DG_ERR_ARG, "sfc_order is not a permutation of 1..n");
    pos[i] = p;
    inv[p] = i;
  }
  h.sizes.clear();
  h.start.assign(1, 0);
  int64_t sz = n;
  for (int l = 0; l < h.nlevel; ++l) {
    h.sizes.push_back(sz);
    h.start.push_back(h.start.back() + sz);
    sz = (sz - 1) / 2 + 1;
  }
  int64_t total = h.start.back();
  // the levels are independent (each is summed from the fine matrix in curve
  // order), so they are formed on parallel host threads
  struct Lv {
    std::vector<int64_t> rp, col;
    std::vector<double> val;
  };
  std::vector<Lv> lv(h.nlevel);
  if (visit_tgt) visit_tgt->assign(h.nlevel, std::vector<int64_t>());
  auto build_level = [&](int l) {
    Lv& L = lv[l];
    std::vector<int64_t>* tg = visit_tgt ? &(*visit_tgt)[l] : nullptr;
    if (tg) tg->reserve((size_t)fina[n]);
    const int64_t nc = h.sizes[l];
    L.rp.assign(nc + 1, 0);
    std::vector<int64_t> slot(nc, -1);   // coarse column -> entry of the current row
    std::vector<int64_t> touched;
    int64_t cur_row = -1;
    for (int64_t s = 0; s < n; ++s) {
      const int64_t ic = s >> l;
      if (ic != cur_row) {
        for (int64_t t : touched) slot[t] = -1;
        touched.clear();
        if (cur_row >= 0) L.rp[cur_row + 1] = (int64_t)L.col.size();
        for (int64_t r = cur_row + 1; r < ic; ++r) L.rp[r + 1] = (int64_t)L.col.size();
        cur_row = ic;
        L.rp[ic] = (int64_t)L.col.size();
      }
      const int64_t node = inv[s];
      for (int64_t k = fina[node]; k < fina[node + 1]; ++k) {
        const int64_t jc = pos[cola[k]] >> l;
        int64_t& sl = slot[jc];
        if (sl >= 0) {
          L.val[sl] += a[k];
        } else {
          sl = (int64_t)L.col.size();
          touched.push_back(jc);
          L.col.push_back(jc);
          L.val.push_back(a[k]);
        }
        if (tg) tg->push_back(sl);
      }
    }
    if (cur_row >= 0) L.rp[cur_row + 1] = (int64_t)L.col.size();
  };
  parallel_for(h.nlevel, build_level);
  h.row_ptr.assign(total + 1, 0);
  h.col.clear();
  h.val.clear();
  for (int l = 0; l < h.nlevel; ++l) {
    const int64_t off = (int64_t)h.col.size();
    for (int64_t i = 0; i <= h.sizes[l]; ++i) h.row_ptr[h.start[l] + i] = off + lv[l].rp[i];
    h.col.insert(h.col.end(), lv[l].col.begin(), lv[l].col.end());
    h.val.insert(h.val.end(), lv[l].val.begin(), lv[l].val.end());
  }
  return DG_OK;
}

// Contribution lists of the Galerkin P1CG operator R A P from the stored
// blocks (R = I_cf, P = I_fc, both weighted 1/#copies as in
// volume_mf_diff.py:1961-1966, 2010-2013):
//   RAP[k] = sum over list k of w(e, a) w(nb, c) (P3^T A_{e,nb} P3)[a][c]
// for the CSR nonzero k = (I, J) of fina / cola, where block (e, slot) couples
// element e's rows to element nb's columns (slot 0: nb = e; slot 1 + f: the
// neighbour across face f), I = p1cg[e][a] and J = p1cg[nb][c].  Entries are
// (block = e * (nface + 1) + slot, a, c), in block order and then (a, c), so a
// fixed-order sum over a list is deterministic.  The colour-probe operator
// equals this product (tested on the CPU restatement).
int rap_contributions(int64_t nele, int ndim, const int64_t* p1cg, const int64_t* nbe, const int64_t* fina,
                      const int64_t* cola, int64_t n, std::vector<int64_t>& ptr,
                      std::vector<std::array<int64_t, 3>>& ent) {
  const int nc = ndim + 1, nf = ndim + 1, ns = nf + 1;
  const int64_t nnz = fina[n];
  auto find = [&](int64_t i, int64_t j) -> int64_t {
    const int64_t* b = cola + fina[i];
    const int64_t* e = cola + fina[i + 1];
    const int64_t* q = std::lower_bound(b, e, j);
    return (q != e && *q == j) ? (int64_t)(q - cola) : -1;
  };
  ptr.assign(nnz + 1, 0);
  // pass 1 counts, pass 2 fills (block order within each list)
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int64_t> fill;
    if (pass == 1) {
      for (int64_t k = 0; k < nnz; ++k) ptr[k + 1] += ptr[k];
      ent.assign(ptr[nnz], {0, 0, 0});
      fill.assign(ptr.begin(), ptr.end() - 1);
    }
    for (int64_t e = 0; e < nele; ++e)
      for (int sl = 0; sl < ns; ++sl) {
        const int64_t nb = sl == 0 ? e : nbe[e * nf + sl - 1];
        if (nb < 0) continue;
        if (nb >= nele) return set_thread_error(DG_ERR_MESH, "rap_contributions: neighbour out of range");
        for (int a = 0; a < nc; ++a)
          for (int c = 0; c < nc; ++c) {
            const int64_t i = p1cg[e * nc + a], j = p1cg[nb * nc + c];
            if (i < 0 || i >= n || j < 0 || j >= n)
              return set_thread_error(DG_ERR_MESH, "rap_contributions: p1cg vertex out of range");
            // a face block also couples vertex pairs that share no element;
            // their contributions cancel (the P1 functions are continuous, so
            // the face terms vanish in the sum) and the probe assembly does
            // not read them either
            const int64_t k = find(i, j);
            if (k < 0) continue;
            if (pass == 0)
              ++ptr[k + 1];
            else
              ent[fill[k]++] = {e * ns + sl, a, c};
          }
      }
  }
  return DG_OK;
}

// Face connectivity in the reference's internal corner order
// (mesh_init.py:298-320 face corner lists, :358-401 matching and alignment).
int face_connectivity(int ndim, int64_t nele, const int64_t* corners, int64_t* nbf, int64_t* alnmt) {
  static const int tet_faces[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
  static const int tri_faces[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  const int nface = ndim + 1;
  const int nc = ndim + 1;
  const int64_t nf = nele * nface;
  std::vector<std::array<int64_t, 3>> keys(nf);
  std::vector<std::array<int64_t, 3>> fn(nf);
  for (int64_t e = 0; e < nele; ++e) {
    for (int f = 0; f < nface; ++f) {
      std::array<int64_t, 3> v = {0, 0, -1};
      for (int k = 0; k < ndim; ++k)
        v[k] = corners[e * nc + (ndim == 3 ? tet_faces[f][k] : tri_faces[f][k])];
      fn[e * nface + f] = v;
      std::array<int64_t, 3> s = v;
      std::sort(s.begin(), s.begin() + ndim);
      keys[e * nface + f] = s;
    }
  }
  std::vector<int64_t> order(nf);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return keys[a] < keys[b] || (keys[a] == keys[b] && a < b);
  });
  for (int64_t i = 0; i < nf; ++i) { nbf[i] = -1; alnmt[i] = -1; }
  for (int64_t i = 0; i + 1 < nf; ++i) {
    int64_t a = order[i], b = order[i + 1];
    if (keys[a] != keys[b]) continue;
    if (i + 2 < nf && keys[order[i + 2]] == keys[a])
      return set_thread_error(DG_ERR_MESH, "a face is shared by more than two elements");
    int64_t lo = std::min(a, b), hi = std::max(a, b);
    nbf[lo] = hi;
    nbf[hi] = lo;
    int64_t code;
    if (ndim == 3)
      code = fn[lo][0] == fn[hi][0] ? 0 : (fn[lo][1] == fn[hi][0] ? 1 : 2);
    else
      code = fn[lo][0] == fn[hi][0] ? 0 : 1;
    alnmt[lo] = code;
    alnmt[hi] = code;
    ++i;
  }
  return DG_OK;
}

// Hilbert-curve index of integer coordinates q[0..ndim) in [0, 2^bits)
// (Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004:
// axes to transposed form, Gray decoding, then the bits interleaved most
// significant first).
int64_t hilbert_index(const int64_t* q, int ndim, int bits) {
  int64_t x[3] = {0, 0, 0};
  for (int i = 0; i < ndim; ++i) x[i] = q[i];
  const int64_t m = (int64_t)1 << (bits - 1);
  for (int64_t Q = m; Q > 1; Q >>= 1) {
    const int64_t P = Q - 1;
    for (int i = 0; i < ndim; ++i) {
      if (x[i] & Q) {
        x[0] ^= P;
      } else {
        const int64_t t = (x[0] ^ x[i]) & P;
        x[0] ^= t;
        x[i] ^= t;
      }
    }
  }
  for (int i = 1; i < ndim; ++i) x[i] ^= x[i - 1];
  int64_t t = 0;
  for (int64_t Q = m; Q > 1; Q >>= 1)
    if (x[ndim - 1] & Q) t ^= Q - 1;
  for (int i = 0; i < ndim; ++i) x[i] ^= t;
  int64_t h = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < ndim; ++i) h = (h << 1) | ((x[i] >> b) & 1);
  return h;
}

// 1-based curve position of each point: coordinates scaled by the largest
// extent onto a 2^bits grid (floor, clipped), sorted by Hilbert index with
// ties by point index.
int sfc_order_hilbert(int ndim, int64_t n, const double* coords, int bits, int64_t* order) {
  if (n == 0) return DG_OK;
  double lo[3], hi[3];
  for (int d = 0; d < ndim; ++d) {
    lo[d] = hi[d] = coords[d];
    for (int64_t i = 1; i < n; ++i) {
      lo[d] = std::min(lo[d], coords[i * ndim + d]);
      hi[d] = std::max(hi[d], coords[i * ndim + d]);
    }
  }
  double span = 0.0;
  for (int d = 0; d < ndim; ++d) span = std::max(span, std::max(hi[d] - lo[d], 1e-300));
  const double scale = (double)(((int64_t)1 << bits) - 1);
  const int64_t qmax = ((int64_t)1 << bits) - 1;
  std::vector<std::pair<int64_t, int64_t>> key(n);
  for (int64_t i = 0; i < n; ++i) {
    int64_t q[3] = {0, 0, 0};
    for (int d = 0; d < ndim; ++d) {
      const double v = std::floor((coords[i * ndim + d] - lo[d]) / span * scale);
      q[d] = std::min<int64_t>(std::max<int64_t>((int64_t)v, 0), qmax);
    }
    key[i] = {hilbert_index(q, ndim, bits), i};
  }
  std::sort(key.begin(), key.end());
  for (int64_t p = 0; p < n; ++p) order[key[p].second] = p + 1;
  return DG_OK;
}

}  // namespace dg

using namespace dg;

extern "C" {

int dg_sfc_order(int32_t ndim, int64_t n, const double* coords, int32_t bits, int64_t* order) {
  if (n < 0 || !order || (ndim != 2 && ndim != 3))
    return set_thread_error(DG_ERR_ARG, "dg_sfc_order: bad arguments");
  if (!coords) {
    // ordering in: a 1-based permutation, e.g. the reference's cached curve
    std::vector<char> seen(n, 0);
    for (int64_t i = 0; i < n; ++i) {
      const int64_t p = order[i] - 1;
      if (p < 0 || p >= n || seen[p])
        return set_thread_error(DG_ERR_ARG, "dg_sfc_order: entry " + std::to_string(i) +
                                                " is not part of a permutation of 1..n");
      seen[p] = 1;
    }
    return DG_OK;
  }
  if (bits <= 0) bits = ndim == 2 ? 20 : 16;
  if (bits * ndim > 62) return set_thread_error(DG_ERR_ARG, "dg_sfc_order: bits * ndim must be <= 62");
  return sfc_order_hilbert(ndim, n, coords, bits, order);
}

int dg_p1cg_sparsity(int64_t nele, int32_t ncorner, const int64_t* p1cg, int64_t cg_nonods,
                     int64_t* fina, int64_t* cola, int64_t cap, int64_t* ncola) {
  if (nele < 0 || ncorner <= 0 || cg_nonods < 0 || (!p1cg && nele > 0) || !fina || !ncola)
    return set_thread_error(DG_ERR_ARG, "dg_p1cg_sparsity: bad arguments");
  std::vector<int64_t> f, c;
  int rc = p1cg_sparsity(nele, ncorner, p1cg, cg_nonods, f, c);
  if (rc) return rc;
  *ncola = (int64_t)c.size();
  std::memcpy(fina, f.data(), sizeof(int64_t) * f.size());
  if ((int64_t)c.size() > cap || (!cola && !c.empty()))
    return set_thread_error(DG_ERR_ARG, "dg_p1cg_sparsity: cola capacity too small");
  if (!c.empty()) std::memcpy(cola, c.data(), sizeof(int64_t) * c.size());
  return DG_OK;
}

int dg_color2(int64_t n, const int64_t* fina, const int64_t* cola, int64_t* whichc, int32_t* ncolor) {
  if (n < 0 || !fina || !whichc || !ncolor) return set_thread_error(DG_ERR_ARG, "dg_color2: bad arguments");
  std::vector<int64_t> w;
  int rc = color2(n, fina, cola, w, *ncolor);
  if (rc) return rc;
  if (n) std::memcpy(whichc, w.data(), sizeof(int64_t) * n);
  return DG_OK;
}

int32_t dg_nlevel_sfc(int64_t nonods) { return nlevel_sfc(nonods); }

int dg_rap_contributions(int32_t ndim, int64_t nele, const int64_t* p1cg, const int64_t* nbe, const int64_t* fina,
                         const int64_t* cola, int64_t cg_nonods, int64_t* ptr, int64_t* entries, int64_t cap,
                         int64_t* count) {
  if ((ndim != 2 && ndim != 3) || nele < 0 || cg_nonods < 0 || !fina || !ptr || !count ||
      (nele > 0 && (!p1cg || !nbe || !cola)))
    return set_thread_error(DG_ERR_ARG, "dg_rap_contributions: bad arguments");
  std::vector<int64_t> p;
  std::vector<std::array<int64_t, 3>> ent;
  int rc = rap_contributions(nele, ndim, p1cg, nbe, fina, cola, cg_nonods, p, ent);
  if (rc) return rc;
  *count = (int64_t)ent.size();
  std::memcpy(ptr, p.data(), sizeof(int64_t) * p.size());
  if ((int64_t)ent.size() > cap || (!entries && !ent.empty()))
    return set_thread_error(DG_ERR_ARG, "dg_rap_contributions: entries capacity too small");
  if (!ent.empty()) std::memcpy(entries, ent.data(), sizeof(int64_t) * 3 * ent.size());
  return DG_OK;
}

int dg_sfc_levels(int64_t n, const int64_t* fina, const int64_t* cola, const double* a,
                  const int64_t* sfc_order, int32_t* nlevel, int64_t* level_start, int64_t* row_ptr,
                  int64_t* col, double* val, int64_t cap, int64_t* nnz) {
  if (n <= 0 || !fina || !cola || !a || !sfc_order || !nlevel || !level_start || !row_ptr || !nnz)
    return set_thread_error(DG_ERR_ARG, "dg_sfc_levels: bad arguments");
  SfcHierarchy h;
  int rc = sfc_levels(n, fina, cola, a, sfc_order, h);
  if (rc) return rc;
  *nlevel = h.nlevel;
  *nnz = (int64_t)h.col.size();
  std::memcpy(level_start, h.start.data(), sizeof(int64_t) * h.start.size());
  std::memcpy(row_ptr, h.row_ptr.data(), sizeof(int64_t) * h.row_ptr.size());
  if ((int64_t)h.col.size() > cap || !col || !val)
    return set_thread_error(DG_ERR_ARG, "dg_sfc_levels: capacity too small");
  std::memcpy(col, h.col.data(), sizeof(int64_t) * h.col.size());
  std::memcpy(val, h.val.data(), sizeof(double) * h.val.size());
  return DG_OK;
}

int dg_face_connectivity(int32_t ndim, int64_t nele, const int64_t* corners, int64_t* nbf, int64_t* alnmt) {
  if ((ndim != 2 && ndim != 3) || nele < 0 || !corners || !nbf || !alnmt)
    return set_thread_error(DG_ERR_ARG, "dg_face_connectivity: bad arguments");
  return face_connectivity(ndim, nele, corners, nbf, alnmt);
}

}  // extern "C"
