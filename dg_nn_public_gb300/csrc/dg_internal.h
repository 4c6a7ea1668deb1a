// Internal declarations shared by the translation units of libdgsip.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../../include/dgsip.h"

namespace dg {

int set_thread_error(int code, const std::string& msg);
extern thread_local std::string g_thread_error;

struct SfcHierarchy {
  int32_t nlevel = 0;
  std::vector<int64_t> sizes;     // nodes per level
  std::vector<int64_t> start;     // stacked first node of each level (nlevel+1)
  std::vector<int64_t> row_ptr;   // stacked CSR rows (total+1), into col/val
  std::vector<int64_t> col;       // level-local column index
  std::vector<double> val;
};

// Runs fn(0) .. fn(count - 1) on up to hardware_concurrency() host threads
// (independent items, taken in order from a shared counter).
template <typename Fn>
void parallel_for(int count, Fn fn) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<unsigned>(hw, (unsigned)std::max(count, 0));
  if (nt <= 1) {
    for (int i = 0; i < count; ++i) fn(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&] {
      for (int i = next.fetch_add(1); i < count; i = next.fetch_add(1)) fn(i);
    });
  for (auto& x : th) x.join();
}

int rap_contributions(int64_t nele, int ndim, const int64_t* p1cg, const int64_t* nbe, const int64_t* fina,
                      const int64_t* cola, int64_t n, std::vector<int64_t>& ptr,
                      std::vector<std::array<int64_t, 3>>& ent);
int p1cg_sparsity(int64_t nele, int ncorner, const int64_t* p1cg, int64_t n,
                  std::vector<int64_t>& fina, std::vector<int64_t>& cola);
int color2(int64_t n, const int64_t* fina, const int64_t* cola, std::vector<int64_t>& whichc,
           int32_t& ncolor);
void sparse_idx_for_color(int64_t n, const int64_t* fina, const int64_t* cola,
                          const std::vector<int64_t>& whichc, int32_t ncolor,
                          std::vector<std::vector<int64_t>>& spidx,
                          std::vector<std::vector<int64_t>>& colidx);
int32_t nlevel_sfc(int64_t nonods);
// visit_tgt (optional): per level, for each fine entry in the order the
// level sums visit them (rows in curve order, entries in row order), the
// index of the level entry it is added to
int sfc_levels(int64_t n, const int64_t* fina, const int64_t* cola, const double* a,
               const int64_t* sfc_order, SfcHierarchy& h,
               std::vector<std::vector<int64_t>>* visit_tgt = nullptr);
int face_connectivity(int ndim, int64_t nele, const int64_t* corners, int64_t* nbf, int64_t* alnmt);

}  // namespace dg
