// Instantiations of the persistent contraction for configurations [0, kPzSplit) of kPzConfs
// (S = 1 to 3); pz_launch_b.cu holds the others, so the two compile in parallel.
#include "pz_launch.cuh"

namespace ccsdt {

static_assert(kPzSplit == 9 && kPzConfs[8].S == 3 && kPzConfs[9].S == 4, "the split of the configurations");

#define PZ_CASES(X) X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8)

cudaError_t pz_launch_single_a(int conf, const PzParams& p, int grid, cudaStream_t st) {
#define X(c) \
  case c: return pz_launch_single_t<c>(p, grid, st);
  switch(conf) { PZ_CASES(X) }
#undef X
  return cudaErrorInvalidValue;
}

} // namespace ccsdt
