// Batched, persistent split-precision (T): host orchestration.
//
// The non-zero triplets of a call (i < k) go into a device table (i, j, k, output index).  A batch
// of B triplets runs as: l-sum contraction (persistent, work queue), d-sum contraction (persistent),
// tiled energy of the B triplets, per-triplet reduction, advance of the device batch base.  With
// opts->use_graph that sequence is captured once per call into a CUDA graph and replayed for every
// full batch; the remainder batch is launched directly.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ccsdt_internal.cuh"
#include "energy_tiled.cuh"
#include "fp64_kernels.cuh"
#include "oz_pair.cuh"
#include "oz_persist.cuh"

using namespace ccsdt;

namespace {

template<int S>
struct PzPick;
template<>
struct PzPick<1> {
  static constexpr int NT = 64, ST = 4, KC = 64;
};
template<>
struct PzPick<2> {
  static constexpr int NT = 64, ST = 4, KC = 64;
};
template<>
struct PzPick<3> {
  static constexpr int NT = 64, ST = 3, KC = 64; // (NT = 48 with three level buffers measured 1.5x slower)
};
// S = 4, 5: a 64-wide K chunk takes 96 / 100 KB a stage, so only two stages fit and the TMA latency
// shows; 32-wide chunks (64-byte rows, 64-byte swizzle) give four stages in the same space
template<>
struct PzPick<4> {
  static constexpr int NT = 64, ST = 4, KC = 32;
};
template<>
struct PzPick<5> {
  static constexpr int NT = 32, ST = 4, KC = 32;
};

int pz_nt(int S) {
  switch(S) {
    case 1: return PzPick<1>::NT;
    case 2: return PzPick<2>::NT;
    case 3: return PzPick<3>::NT;
    case 4: return PzPick<4>::NT;
    case 5: return PzPick<5>::NT;
  }
  return 0;
}
int pz_kc(int S) {
  switch(S) {
    case 1: return PzPick<1>::KC;
    case 2: return PzPick<2>::KC;
    case 3: return PzPick<3>::KC;
    case 4: return PzPick<4>::KC;
    case 5: return PzPick<5>::KC;
  }
  return 0;
}

template<int S>
cudaError_t launch_pz(const PzParams& p, int grid, cudaStream_t st) {
  constexpr int NT = PzPick<S>::NT, ST = PzPick<S>::ST, KC = PzPick<S>::KC;
  using Cfg        = PzCfg<S, NT, ST, KC>;
  cudaError_t e = cudaFuncSetAttribute(oz_persist_kernel<S, NT, ST, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  if(e != cudaSuccess) return e;
  oz_persist_kernel<S, NT, ST, KC><<<grid, PZ_THREADS, Cfg::SMEM, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_pz_any(int S, const PzParams& p, int grid, cudaStream_t st) {
  switch(S) {
    case 1: return launch_pz<1>(p, grid, st);
    case 2: return launch_pz<2>(p, grid, st);
    case 3: return launch_pz<3>(p, grid, st);
    case 4: return launch_pz<4>(p, grid, st);
    case 5: return launch_pz<5>(p, grid, st);
  }
  return cudaErrorInvalidValue;
}

// Item ids of B slots sorted by estimated cost (rows x columns of the tile), largest first; ties
// keep the natural order (n-block fastest) so concurrently running CTAs share A tiles in L2.
// pair = true: items of the cluster kernel, one per pair of adjacent n-blocks.
std::vector<unsigned> cost_order(int B, int v, int NT, bool pair) {
  const int  yb = (v + PZ_BM - 1) / PZ_BM, nb = (v + NT - 1) / NT, nn = pair ? (nb + 1) / 2 : nb;
  const long n  = (long) B * 3 * v * yb * nn;
  std::vector<unsigned> ids(n);
  std::iota(ids.begin(), ids.end(), 0u);
  auto cols = [&](int b) { return b < nb ? std::min(NT, v - b * NT) : 0; };
  auto cost = [&](unsigned id) {
    const int n_b = id % nn, y_b = (id / nn) % yb;
    const int rows = std::min(PZ_BM, v - y_b * PZ_BM);
    return rows * (pair ? cols(2 * n_b) + cols(2 * n_b + 1) : cols(n_b));
  };
  std::stable_sort(ids.begin(), ids.end(), [&](unsigned a, unsigned b) { return cost(a) > cost(b); });
  return ids;
}

// Items per triplet slot of one launch.
long items_per_slot(int v, int NT, bool pair) {
  const int yb = (v + PZ_BM - 1) / PZ_BM, nb = (v + NT - 1) / NT;
  return 3L * v * yb * (pair ? (nb + 1) / 2 : nb);
}

template<int S>
cudaError_t launch_pair(const PzParams& p, int ncl, cudaStream_t st) {
  constexpr int NT = PzPick<S>::NT, ST = PzPick<S>::ST, KC = PzPick<S>::KC;
  using Cfg        = PzCfg<S, NT, ST, KC>;
  cudaError_t e = cudaFuncSetAttribute(oz_pair_kernel<S, NT, ST, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  if(e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id               = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim              = dim3(2 * ncl, 1, 1);
  cfg.blockDim             = dim3(PZ_THREADS, 1, 1);
  cfg.dynamicSmemBytes     = Cfg::SMEM;
  cfg.stream               = st;
  cfg.attrs                = attr;
  cfg.numAttrs             = 1;
  e = cudaLaunchKernelEx(&cfg, oz_pair_kernel<S, NT, ST, KC>, p);
  if(e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_pair_any(int S, const PzParams& p, int ncl, cudaStream_t st) {
  switch(S) {
    case 1: return launch_pair<1>(p, ncl, st);
    case 2: return launch_pair<2>(p, ncl, st);
    case 3: return launch_pair<3>(p, ncl, st);
    case 4: return launch_pair<4>(p, ncl, st);
    case 5: return launch_pair<5>(p, ncl, st);
  }
  return cudaErrorInvalidValue;
}

// Co-resident two-CTA clusters of the cluster kernel for S planes (0: cannot run).
template<int S>
int pair_clusters() {
  constexpr int NT = PzPick<S>::NT, ST = PzPick<S>::ST, KC = PzPick<S>::KC;
  using Cfg        = PzCfg<S, NT, ST, KC>;
  if(cudaFuncSetAttribute(oz_pair_kernel<S, NT, ST, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM) !=
     cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int sm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id               = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim              = dim3(2 * (sm / 2), 1, 1);
  cfg.blockDim             = dim3(PZ_THREADS, 1, 1);
  cfg.dynamicSmemBytes     = Cfg::SMEM;
  cfg.attrs                = attr;
  cfg.numAttrs             = 1;
  int n = 0;
  if(cudaOccupancyMaxActiveClusters(&n, oz_pair_kernel<S, NT, ST, KC>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int pair_clusters_any(int S) {
  switch(S) {
    case 1: return pair_clusters<1>();
    case 2: return pair_clusters<2>();
    case 3: return pair_clusters<3>();
    case 4: return pair_clusters<4>();
    case 5: return pair_clusters<5>();
  }
  return 0;
}

} // namespace

ccsdt_status ccsdt_handle::ensure_batch(int S, int B) {
  const long long v3 = (long long) v * v * v;
  const int       NT = pz_nt(S);
  if(!NT) return fail(CCSDT_E_INVALID, "no persistent configuration for this slice count");
  if(bt_B != B) {
    if(bt_F) cudaFree(bt_F);
    if(bt_part) cudaFree(bt_part);
    bt_F = nullptr;
    bt_part = nullptr;
    if(cudaMalloc((void**) &bt_F, sizeof(float2) * 3 * v3 * B) != cudaSuccess ||
       cudaMalloc((void**) &bt_part, sizeof(double) * 6 * kTiledBlocks * B) != cudaSuccess) {
      cudaGetLastError();
      if(bt_F) cudaFree(bt_F);
      bt_F = nullptr;
      return fail(CCSDT_E_OOM, "batch scratch: cudaMalloc failed");
    }
    bt_B = B;
    bt_order_key = -1;
  }
  const int key = (S * 100000 + B) * 2 + (pz_pair ? 1 : 0);
  if(bt_order_key != key) {
    auto ids = cost_order(B, v, NT, pz_pair);
    if(bt_order) cudaFree(bt_order);
    bt_order = nullptr;
    if(cudaMalloc((void**) &bt_order, ids.size() * sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "work-queue table: cudaMalloc failed");
    }
    if(cudaMemcpy(bt_order, ids.data(), ids.size() * sizeof(unsigned), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(CCSDT_E_CUDA, "work-queue table upload");
    bt_nitems    = (unsigned) ids.size();
    bt_order_key = key;
  }
  if(!bt_ctrl) { // [0] queue l-sum, [1] queue d-sum, [2] batch base
    if(cudaMalloc((void**) &bt_ctrl, 4 * sizeof(int)) != cudaSuccess) {
      bt_ctrl = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "batch counters");
    }
  }
  return CCSDT_OK;
}

// One full wave of the tiled energy kernels (resident CTAs per SM x SMs), capped at
// kTiledBlocks: a grid-stride loop over more CTAs than fit at once would leave a partial wave.
int ccsdt_handle::energy_grid() {
  if(energy_grid_ > 0) return energy_grid_;
  int sm = 0, per = 0, per1 = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, energy_tiled_batch_kernel, ET_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, energy_tiled_kernel, ET_THREADS, 0);
  per          = std::min(per, per1);
  energy_grid_ = std::max(1, std::min(kTiledBlocks, std::max(1, per) * std::max(1, sm)));
  cudaGetLastError();
  return energy_grid_;
}

// Launch the sequence of one batch of `nslots` triplets starting at the device base counter.
ccsdt_status ccsdt_handle::launch_batch(int S, int nslots, int nitems_override, bool advance, float* tails,
                                        double* sens) {
  // the B-side TMA box must be exactly the kernel's N tile, or the loads overrun the smem slot
  if(!tmaps_ready || tmaps_S != S || tmaps_NT != pz_nt(S) || tmaps_KC != pz_kc(S))
    return fail(CCSDT_E_STATE, "tensor maps do not match the persistent kernel's tile");
  int sm = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  PzParams p;
  static_assert(sizeof(p.maps) == sizeof(tmaps), "the persistent kernel takes every map");
  std::memcpy(p.maps, tmaps, sizeof(p.maps));
  p.tri = bt_tri, p.base = bt_ctrl + 2, p.nslots = nslots, p.o = o, p.v = v, p.kp_v = kp_v, p.kp_o = kp_o;
  p.F = bt_F;
  p.order = bt_order, p.nitems = (unsigned) nitems_override, p.err = d_err, p.tail = tails;
  const int  NT  = pz_nt(S);
  const long per = items_per_slot(v, NT, pz_pair);
  if(nitems_override <= 0) p.nitems = (unsigned) (per * nslots);
  // the cost-ordered table was built for bt_B slots; a smaller last batch has its own table
  const bool partial = nslots != bt_B;
  cudaError_t e = cudaSuccess;
  if(partial) p.order = bt_order_partial;
  cudaEvent_t tv[3] = {nullptr, nullptr, nullptr};
  if(phase_timing && !capturing && !profiling) {
    while(tev.size() < tev_used + 3) {
      cudaEvent_t ev = nullptr;
      if(cudaEventCreate(&ev) != cudaSuccess) return fail(CCSDT_E_CUDA, "phase-timing event");
      tev.push_back(ev);
    }
    for(int q = 0; q < 3; q++) tv[q] = tev[tev_used + q];
    tev_used += 3;
    tev_slots.push_back(nslots);
  }
  // one launch: every tile of the three partial arrays with its l-sum and d-sum terms
  p.queue = reinterpret_cast<unsigned*>(bt_ctrl);
  if(tv[0]) cudaEventRecord(tv[0], stream);
  e = cudaMemsetAsync(p.queue, 0, sizeof(unsigned), stream);
  if(profiling) {
    cudaEventRecord(prof_ev[0], stream);
    cudaEventRecord(prof_ev[1], stream); // no separate l-sum phase
  }
  if(e == cudaSuccess)
    e = pz_pair ? launch_pair_any(S, p, (int) std::min<long>(pz_pair_clusters, (long) p.nitems), stream)
                : launch_pz_any(S, p, sm, stream);
  launches++;
  if(profiling) cudaEventRecord(prof_ev[2], stream);
  if(tv[1]) cudaEventRecord(tv[1], stream);
  if(e == cudaSuccess) {
    BatchEnergyArgs ea;
    ea.base_args = TiledEnergyArgs{nullptr, nullptr, nullptr, oovv_f, t1_f, eo, ev, (const int3*) e_tiles, e_ntiles,
                                   o, v, 0, 0, 0, nullptr, sens != nullptr};
    ea.tri = bt_tri, ea.base = bt_ctrl + 2, ea.F = bt_F, ea.part = bt_part;
    const int G = std::min(e_ntiles, energy_grid());
    energy_tiled_batch_kernel<<<dim3(G, nslots), ET_THREADS, 0, stream>>>(ea);
    if(profiling) cudaEventRecord(prof_ev[3], stream);
    reduce_parts_batch_kernel<<<nslots, 256, 0, stream>>>(bt_part, G, bt_tri, bt_ctrl + 2, etrip, sens);
    if(advance) advance_base_kernel<<<1, 32, 0, stream>>>(bt_ctrl + 2, nslots);
    if(profiling) cudaEventRecord(prof_ev[4], stream);
    if(tv[2]) cudaEventRecord(tv[2], stream);
    launches += 2 + (advance ? 1 : 0);
    e = cudaGetLastError();
  }
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

// Run triplets tri[3 n] at S digit planes through the persistent kernels; results -> etrip.
// out_map (optional): output index of each listed triplet (etrip, tails, sens); default t.
ccsdt_status ccsdt_handle::run_batched(int S, long n, const int* tri, bool use_graph, float* tails, double* sens,
                                       const int* out_map) {
  ccsdt_status s;
  tev_used = 0; // events of a batch that failed earlier are not read
  tev_slots.clear();
  // the two-CTA cluster kernel when its clusters can be resident (and not switched off for a test)
  if(S >= 1 && S <= 5 && pair_clusters_by_S[S] < 0) pair_clusters_by_S[S] = pair_clusters_any(S);
  pz_pair_clusters = (S >= 1 && S <= 5) ? pair_clusters_by_S[S] : 0;
  pz_pair          = !force_single_cta && pz_pair_clusters > 0;
  if((s = ensure_slices(std::max(S, slices_ready), 0)) || (s = ensure_tmaps(S, pz_nt(S), pz_kc(S)))) return s;
  // table of non-zero triplets (i < k); i = j = k contributes exactly zero
  std::vector<int> tab;
  for(long t = 0; t < n; t++) {
    const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    const int out = out_map ? out_map[t] : (int) t;
    if(i == k) {
      if(cudaMemsetAsync(etrip + 2 * (long) out, 0, 2 * sizeof(double), stream) != cudaSuccess)
        return fail(CCSDT_E_CUDA, "memset");
      continue;
    }
    tab.insert(tab.end(), {i, j, k, out});
  }
  const long m = (long) tab.size() / 4;
  if(m == 0) return CCSDT_OK;
  const int B = (int) std::min<long>(batch_slots, m);
  if((s = ensure_batch(S, B))) return s;
  if(bt_tri_cap < m) {
    if(bt_tri) cudaFree(bt_tri);
    bt_tri = nullptr;
    if(cudaMalloc((void**) &bt_tri, tab.size() * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "triplet table");
    }
    bt_tri_cap = m;
  }
  // natural-order table for a partial last batch
  const int  NT  = pz_nt(S);
  const long per = items_per_slot(v, NT, pz_pair);
  const long rem = m % B;
  if(rem) {
    auto ids = cost_order((int) rem, v, NT, pz_pair);
    if(bt_order_partial) cudaFree(bt_order_partial);
    bt_order_partial = nullptr;
    if(cudaMalloc((void**) &bt_order_partial, ids.size() * sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "partial work-queue table");
    }
    if(cudaMemcpyAsync(bt_order_partial, ids.data(), ids.size() * sizeof(unsigned), cudaMemcpyHostToDevice, stream) !=
       cudaSuccess)
      return fail(CCSDT_E_CUDA, "partial table upload");
  }
  if(cudaMemcpyAsync(bt_tri, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
     cudaMemsetAsync(bt_ctrl + 2, 0, sizeof(int), stream) != cudaSuccess)
    return fail(CCSDT_E_CUDA, "triplet table upload");
  // table upload must finish before the host vector goes away
  if(cudaStreamSynchronize(stream) != cudaSuccess) return fail(CCSDT_E_CUDA, "sync");
  const long full = m / B;
  if(full > 0) {
    if(use_graph && full > 1 && !profiling) {
      cudaGraph_t     g  = nullptr;
      cudaGraphExec_t ge = nullptr;
      if(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(CCSDT_E_CUDA, "stream capture begin");
      capturing      = true;
      s              = launch_batch(S, B, 0, true, tails, sens);
      capturing      = false;
      cudaError_t ce = cudaStreamEndCapture(stream, &g);
      if(s) {
        if(g) cudaGraphDestroy(g);
        return s;
      }
      if(ce != cudaSuccess || cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
        if(g) cudaGraphDestroy(g);
        cudaGetLastError();
        return fail(CCSDT_E_CUDA, "graph capture / instantiate");
      }
      for(long b = 0; b < full; b++)
        if(cudaGraphLaunch(ge, stream) != cudaSuccess) {
          cudaGraphExecDestroy(ge);
          cudaGraphDestroy(g);
          return fail(CCSDT_E_CUDA, "graph launch");
        }
      launches += (full - 1) * 4; // contraction, energy, reduction, base advance per replay
      graph_replays += full;
      cudaGraphExecDestroy(ge);
      cudaGraphDestroy(g);
    } else {
      for(long b = 0; b < full; b++)
        if((s = launch_batch(S, B, 0, true, tails, sens))) return s;
    }
  }
  if(rem) {
    if((s = launch_batch(S, (int) rem, (int) (per * rem), true, tails, sens))) return s;
  }
  return collect_phase_times();
}

// Adds the timed batches' phase durations to the running totals (waits for the stream).
ccsdt_status ccsdt_handle::collect_phase_times() {
  if(tev_used == 0) return CCSDT_OK;
  if(cudaStreamSynchronize(stream) != cudaSuccess) return fail(CCSDT_E_CUDA, "phase-timing sync");
  for(size_t b = 0; b < tev_slots.size(); b++)
    for(int q = 0; q < 2; q++) {
      float ms = 0;
      if(cudaEventElapsedTime(&ms, tev[3 * b + q], tev[3 * b + q + 1]) != cudaSuccess)
        return fail(CCSDT_E_CUDA, "phase-timing elapsed time");
      phase_ms[q] += ms;
    }
  phase_batches += (long) tev_slots.size();
  for(int n: tev_slots) phase_triplets += n;
  tev_used = 0;
  tev_slots.clear();
  return CCSDT_OK;
}
