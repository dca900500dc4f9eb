// Instantiations of the persistent contraction for configurations [kPzSplit2, kPzNConfs) of kPzConfs
// (S = 6 to 8); pz_launch_a.cu and pz_launch_b.cu hold the others, so the three compile in parallel.
#include "pz_launch.cuh"

namespace ccsdt {

static_assert(kPzNConfs == 19, "the cases below list every configuration from kPzSplit2 on");

#define PZ_CASES(X) X(16) X(17) X(18)

cudaError_t pz_launch_single_c(int conf, const PzParams& p, int grid, cudaStream_t st) {
#define X(c) \
  case c: return pz_launch_single_t<c>(p, grid, st);
  switch(conf) { PZ_CASES(X) }
#undef X
  return cudaErrorInvalidValue;
}

} // namespace ccsdt
