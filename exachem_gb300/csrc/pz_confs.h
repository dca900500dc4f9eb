// Compiled configurations of the persistent split-precision contraction, and their launchers.
//
// A configuration is (S digit planes, NT N-tile columns, ST pipeline stages, KC K chunk).  Every
// configuration computes bit-identical P arrays: the MMA level sums are exact integers whatever
// the tiling, and each element's fold (four terms in a fixed order, Horner over the levels) does
// not depend on the tile.  The autotuner (ccsdt_autotune) may therefore pick any of them.
// Constraints a configuration meets: S NT <= 256 (MMA N), 2 S NT <= 512 (two TMEM level buffers),
// NT a multiple of 16 (epilogue column quarters of a multiple of 4), KC in {64, 32}, ST stages of
// S 128 KC 2 + S NT KC 2 bytes within the 227 KB of shared memory.
#pragma once

#include <cuda_runtime.h>

namespace ccsdt {

struct PzParams;

struct PzConf {
  int S, NT, ST, KC;
};

// Grouped by S; the first configuration of each S is the default (the fastest measured at
// o=60 v=500 on GB300).
constexpr PzConf kPzConfs[] = {
  {1, 64, 4, 64}, {1, 32, 6, 64},                 // 0, 1
  {2, 128, 3, 64}, {2, 96, 4, 64}, {2, 64, 4, 64}, {2, 32, 5, 64}, // 2, 3, 4, 5
  {3, 64, 3, 64}, {3, 32, 3, 64}, {3, 48, 3, 64},                  // 6, 7, 8
  {4, 64, 4, 32}, {4, 32, 5, 32}, {4, 64, 2, 64}, {4, 48, 5, 32},  // 9, 10, 11, 12
  {5, 48, 4, 32}, {5, 32, 4, 32}, {5, 32, 2, 64},                  // 13, 14, 15
  {6, 32, 3, 32}, {7, 32, 3, 32}, {8, 32, 2, 32},                  // 16, 17, 18
};
constexpr int kPzNConfs = sizeof(kPzConfs) / sizeof(kPzConfs[0]);
// configurations [0, kPzSplit) live in pz_launch_a.cu, [kPzSplit, kPzSplit2) in pz_launch_b.cu,
// the rest in pz_launch_c.cu (three translation units that compile in parallel)
constexpr int kPzSplit = 9, kPzSplit2 = 16;

constexpr int pz_default_conf(int S) {
  for(int c = 0; c < kPzNConfs; c++)
    if(kPzConfs[c].S == S) return c;
  return -1;
}
constexpr int pz_smem_bytes(const PzConf& c) {
  return c.ST * (c.S * 128 * c.KC * 2 + c.S * c.NT * c.KC * 2) + 1024 + 512;
}
constexpr bool pz_conf_ok(const PzConf& c) {
  return c.S >= 1 && c.S <= 8 && c.S * c.NT <= 256 && 2 * c.S * c.NT <= 512 && c.NT % 16 == 0 &&
         (c.KC == 64 || c.KC == 32) && c.ST >= 2 && pz_smem_bytes(c) <= 227 * 1024;
}
constexpr bool pz_all_ok() {
  for(int c = 0; c < kPzNConfs; c++)
    if(!pz_conf_ok(kPzConfs[c]) || (c > 0 && kPzConfs[c].S < kPzConfs[c - 1].S)) return false;
  return true;
}
static_assert(pz_all_ok(), "every compiled configuration must fit the kernels' limits, grouped by S");

// Launch configuration `conf` (an index into kPzConfs) of the persistent kernel on `grid` CTAs.
cudaError_t pz_launch_single(int conf, const PzParams& p, int grid, cudaStream_t st);

} // namespace ccsdt
