// Host-side planning for the Cholesky-direct mode, in which (ia|bc) is never held whole: the
// o v^3 block is formed one occupied index at a time (a slab (ia|bc) for all a, b, c) into a cache
// of C slots, as the triplets need them.
//
// Order: the triplets of a call are visited by blocks of occupied indices of width b = max(1, C/3)
// (sorted by (i / b, j / b, k / b), then by (i, j, k)), so the triplets of one block triple need
// at most 3 b <= C slabs and the slabs of the two lower blocks stay resident while the third block
// advances.  Cache: least recently used slot among those the current batch does not need.
// Pure host code (no CUDA), shared by the library and its CPU tests.
#pragma once

#include <algorithm>
#include <numeric>
#include <tuple>
#include <utility>
#include <vector>

namespace ccsdt {

// Visiting order of n triplets tri[3 t] (i <= j <= k) for a cache of C slabs.
inline std::vector<long> slab_order(const int* tri, long n, int C) {
  const int         b = std::max(1, C / 3);
  std::vector<long> idx(n);
  std::iota(idx.begin(), idx.end(), 0L);
  auto key = [&](long t) {
    const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    return std::make_tuple(i / b, j / b, k / b, i, j, k, t);
  };
  std::sort(idx.begin(), idx.end(), [&](long x, long y) { return key(x) < key(y); });
  return idx;
}

class SlabCache {
 public:
  void reset(int o, int C) {
    slot_.assign(o, -1);
    owner_.assign(C, -1);
    used_.assign(C, 0);
    clock_  = 0;
    builds_ = 0;
  }
  int  capacity() const { return (int) owner_.size(); }
  int  slot(int x) const { return slot_[x]; }
  int  owner(int c) const { return owner_[c]; }
  long builds() const { return builds_; }
  const std::vector<int>& slots() const { return slot_; }
  // Makes the n occupied indices need[] resident.  Appends to `out` the (index, slot) pairs that
  // must be formed, in order; false when the distinct indices exceed the capacity.
  bool require(const int* need, int n, std::vector<std::pair<int, int>>& out) {
    std::vector<int> uniq(need, need + n);
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    if((int) uniq.size() > capacity()) return false;
    ++clock_;
    for(int x: uniq)
      if(slot_[x] >= 0) used_[slot_[x]] = clock_; // resident: keep for this batch
    for(int x: uniq) {
      if(slot_[x] >= 0) continue;
      int victim = -1;
      for(int c = 0; c < capacity(); c++) {
        if(used_[c] == clock_) continue;          // holds an index this batch needs (or just formed)
        if(victim < 0 || used_[c] < used_[victim]) victim = c;
      }
      if(victim < 0) return false;                // cannot happen while uniq fits
      if(owner_[victim] >= 0) slot_[owner_[victim]] = -1;
      owner_[victim] = x;
      slot_[x]       = victim;
      used_[victim]  = clock_;
      builds_++;
      out.emplace_back(x, victim);
    }
    return true;
  }

 private:
  std::vector<int>  slot_, owner_;
  std::vector<long> used_;
  long              clock_ = 0, builds_ = 0;
};

} // namespace ccsdt
