// Launchers of one compiled configuration of the persistent contraction (kPzConfs[C]); included
// by the two translation units that instantiate them (pz_launch_a.cu, pz_launch_b.cu).
#pragma once

#include <cuda_runtime.h>

#include "oz_persist.cuh"
#include "pz_confs.h"

namespace ccsdt {

template<int C>
cudaError_t pz_launch_single_t(const PzParams& p, int grid, cudaStream_t st) {
  constexpr PzConf c = kPzConfs[C];
  using Cfg          = PzCfg<c.S, c.NT, c.ST, c.KC>;
  cudaError_t e = cudaFuncSetAttribute(oz_persist_kernel<c.S, c.NT, c.ST, c.KC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  if(e != cudaSuccess) return e;
  oz_persist_kernel<c.S, c.NT, c.ST, c.KC><<<grid, PZ_THREADS, Cfg::SMEM, st>>>(p);
  return cudaGetLastError();
}

} // namespace ccsdt
