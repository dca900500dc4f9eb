// Launchers of one compiled configuration of the persistent contraction (kPzConfs[C]); included
// by the two translation units that instantiate them (pz_launch_a.cu, pz_launch_b.cu).
#pragma once

#include <cuda_runtime.h>

#include "oz_pair.cuh"
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

template<int C>
cudaLaunchConfig_t pz_pair_launch_config(int ncl, cudaLaunchAttribute* attr) {
  constexpr PzConf c = kPzConfs[C];
  using Cfg          = PzCfg<c.S, c.NT, c.ST, c.KC>;
  cudaLaunchConfig_t cfg = {};
  attr[0].id               = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim              = dim3(2 * ncl, 1, 1);
  cfg.blockDim             = dim3(PZ_THREADS, 1, 1);
  cfg.dynamicSmemBytes     = Cfg::SMEM;
  cfg.attrs                = attr;
  cfg.numAttrs             = 1;
  return cfg;
}

template<int C>
cudaError_t pz_launch_pair_t(const PzParams& p, int ncl, cudaStream_t st) {
  constexpr PzConf c = kPzConfs[C];
  using Cfg          = PzCfg<c.S, c.NT, c.ST, c.KC>;
  cudaError_t e = cudaFuncSetAttribute(oz_pair_kernel<c.S, c.NT, c.ST, c.KC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  if(e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t  cfg = pz_pair_launch_config<C>(ncl, attr);
  cfg.stream              = st;
  e = cudaLaunchKernelEx(&cfg, oz_pair_kernel<c.S, c.NT, c.ST, c.KC>, p);
  if(e != cudaSuccess) return e;
  return cudaGetLastError();
}

// co-resident two-CTA clusters of the cluster kernel (0: cannot run)
template<int C>
int pz_pair_clusters_t() {
  constexpr PzConf c = kPzConfs[C];
  using Cfg          = PzCfg<c.S, c.NT, c.ST, c.KC>;
  if(cudaFuncSetAttribute(oz_pair_kernel<c.S, c.NT, c.ST, c.KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          Cfg::SMEM) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int sm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t  cfg = pz_pair_launch_config<C>(sm / 2, attr);
  int                 n   = 0;
  if(cudaOccupancyMaxActiveClusters(&n, oz_pair_kernel<c.S, c.NT, c.ST, c.KC>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

} // namespace ccsdt
