// Instantiations of the persistent contraction for configurations [kPzSplit, kPzSplit2) of kPzConfs
// (S = 4, 5); pz_launch_a.cu and pz_launch_c.cu hold the others, so the three compile in parallel.
#include "pz_launch.cuh"

namespace ccsdt {

static_assert(kPzSplit2 == 16 && kPzConfs[15].S == 5 && kPzConfs[16].S == 6, "the cases below list [kPzSplit, kPzSplit2)");

#define PZ_CASES(X) X(9) X(10) X(11) X(12) X(13) X(14) X(15)

cudaError_t pz_launch_single_b(int conf, const PzParams& p, int grid, cudaStream_t st) {
#define X(c) \
  case c: return pz_launch_single_t<c>(p, grid, st);
  switch(conf) { PZ_CASES(X) }
#undef X
  return cudaErrorInvalidValue;
}

} // namespace ccsdt
