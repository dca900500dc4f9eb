// Instantiations of the persistent contraction for configurations [kPzSplit, kPzNConfs) of kPzConfs
// (S = 4, 5); pz_launch_a.cu holds the others, so the two compile in parallel.
#include "pz_launch.cuh"

namespace ccsdt {

static_assert(kPzNConfs == 15, "the cases below list every configuration from kPzSplit on");

#define PZ_CASES(X) X(8) X(9) X(10) X(11) X(12) X(13) X(14)

cudaError_t pz_launch_single_b(int conf, const PzParams& p, int grid, cudaStream_t st) {
#define X(c) \
  case c: return pz_launch_single_t<c>(p, grid, st);
  switch(conf) { PZ_CASES(X) }
#undef X
  return cudaErrorInvalidValue;
}

} // namespace ccsdt
