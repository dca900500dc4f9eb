// Batched, persistent split-precision (T): host orchestration.
//
// The non-zero triplets of a call (i < k) go into a device table (i, j, k, output index).  A batch
// of B triplets runs as: work-queue reset, one persistent contraction launch (every tile of the
// three partial arrays with its l-sum and d-sum terms), tiled energy of the B triplets,
// per-triplet reduction, advance of the device batch base.  With opts->use_graph that sequence is
// captured once per call into a CUDA graph and replayed for every full batch (the per-launch
// phase-timing events are not recorded inside the capture); the remainder batch is launched
// directly.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ccsdt_internal.cuh"
#include "energy_tiled.cuh"
#include "energy_tma.cuh"
#include "fp64_kernels.cuh"
#include "oz_persist.cuh"
#include "pz_confs.h"

using namespace ccsdt;

namespace {

// Item ids of B slots sorted by estimated cost, largest first.  The cost is the tile's row count
// (its A tile), not rows x columns: the items of one A tile - its n-blocks, the last of which may
// be narrower - then stay adjacent in the natural order (n-block fastest), run at the same time on
// neighbouring CTAs and read that A tile from L2 after the first load.  Ordering by rows x columns
// moved the narrow last n-block of every A tile to the end of the queue, long after the tile had
// left L2, and cost one more DRAM read of it.
std::vector<unsigned> cost_order(int B, int v, int NT) {
  const int  yb = (v + PZ_BM - 1) / PZ_BM, nb = (v + NT - 1) / NT;
  const long n  = (long) B * 3 * v * yb * nb;
  std::vector<unsigned> ids(n);
  std::iota(ids.begin(), ids.end(), 0u);
  auto cost = [&](unsigned id) {
    const int y_b = (id / nb) % yb;
    return std::min(PZ_BM, v - y_b * PZ_BM);
  };
  std::stable_sort(ids.begin(), ids.end(), [&](unsigned a, unsigned b) { return cost(a) > cost(b); });
  return ids;
}

// Items per triplet slot of one launch.
long items_per_slot(int v, int NT) {
  return 3L * v * ((v + PZ_BM - 1) / PZ_BM) * ((v + NT - 1) / NT);
}

} // namespace

namespace ccsdt {
cudaError_t pz_launch_single_a(int conf, const PzParams& p, int grid, cudaStream_t st);
cudaError_t pz_launch_single_b(int conf, const PzParams& p, int grid, cudaStream_t st);
cudaError_t pz_launch_single_c(int conf, const PzParams& p, int grid, cudaStream_t st);

cudaError_t pz_launch_single(int conf, const PzParams& p, int grid, cudaStream_t st) {
  return conf < kPzSplit ? pz_launch_single_a(conf, p, grid, st)
         : conf < kPzSplit2 ? pz_launch_single_b(conf, p, grid, st)
                            : pz_launch_single_c(conf, p, grid, st);
}
} // namespace ccsdt

// The configuration in use for S digit planes: the one the autotuner kept, else the default.
int ccsdt_handle::pz_conf_index(int S) const {
  if(S < 1 || S > OZ_MAX_SLICES) return -1;
  return pz_conf_idx[S] >= 0 ? pz_conf_idx[S] : pz_default_conf(S);
}

ccsdt_status ccsdt_handle::ensure_batch(int S, int B) {
  const long long v3 = (long long) v * v * v;
  const int conf = pz_conf_index(S);
  if(conf < 0) return fail(CCSDT_E_INVALID, "no persistent configuration for this slice count");
  const int NT = kPzConfs[conf].NT;
  if(bt_B != B) {
    if(bt_F) cudaFree(bt_F);
    if(bt_part) cudaFree(bt_part);
    bt_F = nullptr;
    bt_part = nullptr;
    bt_B = 0; // until both buffers exist
    if(dev_malloc((void**) &bt_F, sizeof(float2) * 3 * v3 * B) != cudaSuccess ||
       dev_malloc((void**) &bt_part, sizeof(double) * 6 * kTiledBlocks * B) != cudaSuccess) {
      cudaGetLastError();
      if(bt_F) cudaFree(bt_F);
      bt_F = nullptr;
      return fail(CCSDT_E_OOM, "batch scratch: cudaMalloc failed");
    }
    bt_B = B;
    bt_order_key = -1;
  }
  const int key = (conf * 8 + S) * 100000 + B;
  if(bt_order_key != key) {
    auto ids = cost_order(B, v, NT);
    if(bt_order) cudaFree(bt_order);
    bt_order     = nullptr;
    bt_order_key = -1; // until the new table is in place
    if(dev_malloc((void**) &bt_order, ids.size() * sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "work-queue table: cudaMalloc failed");
    }
    if(cudaMemcpy(bt_order, ids.data(), ids.size() * sizeof(unsigned), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(CCSDT_E_CUDA, "work-queue table upload");
    bt_nitems    = (unsigned) ids.size();
    bt_order_key = key;
  }
  if(!bt_ctrl) { // [0] queue l-sum, [1] queue d-sum, [2] batch base
    if(dev_malloc((void**) &bt_ctrl, 4 * sizeof(int)) != cudaSuccess) {
      bt_ctrl = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "batch counters");
    }
  }
  return CCSDT_OK;
}

// One full wave of the tiled energy kernels (resident CTAs per SM x SMs), capped at
// kTiledBlocks: a grid-stride loop over more CTAs than fit at once would leave a partial wave.
int ccsdt_handle::energy_grid(bool f32) {
  int& g = f32 ? energy_grid_f32_ : energy_grid_;
  if(g > 0) return g;
  int sm = 0, per = 0, per1 = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  if(f32) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, energy_tiled_batch_kernel<float>, ET_THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, energy_tiled_kernel<float>, ET_THREADS, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, energy_tiled_batch_kernel<float2>, ET_THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, energy_tiled_kernel<float2>, ET_THREADS, 0);
  }
  per = std::min(per, per1);
  g = std::max(1, std::min(kTiledBlocks, std::max(1, per) * std::max(1, sm)));
  cudaGetLastError();
  return g;
}

// Grid of one resident wave of the TMA energy kernel (element type, box stages); sets the kernel's
// dynamic shared-memory limit first (the boxes exceed the default 48 KB).
template<typename TP, int NST>
static int tma_energy_wave(int sm) {
  int per = 0;
  cudaFuncSetAttribute(energy_tma_batch_kernel<TP, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) em_smem_bytes<TP, NST>());
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, energy_tma_batch_kernel<TP, NST>, EM_THREADS,
                                                em_smem_bytes<TP, NST>());
  cudaGetLastError();
  return std::max(1, std::min(kTiledBlocks, std::max(1, per) * std::max(1, sm)));
}

// kind: 0 float-float, 1 FP32, 2 FP64 partial arrays
int ccsdt_handle::energy_tma_grid(int kind, int nst) {
  int& g = energy_tma_grid_[kind + 3 * (nst - 1)];
  if(g > 0) return g;
  int sm = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  g = kind == 1   ? (nst == 2 ? tma_energy_wave<float, 2>(sm) : tma_energy_wave<float, 1>(sm))
      : kind == 2 ? tma_energy_wave<double, 1>(sm)
                  : (nst == 2 ? tma_energy_wave<float2, 2>(sm) : tma_energy_wave<float2, 1>(sm));
  return g;
}

// Launch the sequence of one batch of `nslots` triplets starting at the device base counter.
ccsdt_status ccsdt_handle::launch_batch(int S, int nslots, int nitems_override, bool advance, float* tails,
                                        double* sens) {
  // the B-side TMA box must be exactly the kernel's N tile, or the loads overrun the smem slot
  const int conf = pz_conf_index(S);
  if(conf < 0 || !tmaps_ready || tmaps_S != S || tmaps_NT != kPzConfs[conf].NT || tmaps_KC != kPzConfs[conf].KC)
    return fail(CCSDT_E_STATE, "tensor maps do not match the persistent kernel's tile");
  int sm = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  PzParams p;
  static_assert(sizeof(p.maps) == sizeof(tmaps), "the persistent kernel takes every map");
  std::memcpy(p.maps, tmaps, sizeof(p.maps));
  p.tri = bt_tri, p.base = bt_ctrl + 2, p.nslots = nslots, p.o = o, p.v = v, p.kp_v = kp_v, p.kp_o = kp_o;
  p.F = bt_F;
  const bool f64 = p_storage == 3, f32 = !f64 && p_f32(S);
  p.f32_out      = f32;
  p.f64_out      = f64;
  last_p_f32     = f32;
  last_p_f64     = f64;
  if(f64 && !ensure_pmap(false))
    return fail(CCSDT_E_INVALID, "FP64 partial arrays need an even v (the energy reads them through TMA)");
  p.ovvv_slot    = ovvv_direct ? d_slab_of : nullptr;
  p.order = bt_order, p.nitems = (unsigned) nitems_override, p.err = d_err, p.tail = tails;
  // windows in multiples of 64 whatever the configuration's K chunk, so every configuration folds
  // the same windows and the energies stay bit-identical across configurations
  p.wst        = pz_window_k(S, 64) / kPzConfs[conf].KC;
  if(test_window_k > 0) p.wst = std::max(1, std::min(p.wst, test_window_k / kPzConfs[conf].KC));
  // the testing limit applies to the kernel whose loads the test withholds (the contraction's
  // unless the energy's are)
  p.spin       = test_spin_limit && test_skip_loads != 2 ? test_spin_limit : sm100::kSpinLimit;
  p.skip_loads = test_skip_loads == 1;
  const int  NT  = kPzConfs[conf].NT;
  const long per = items_per_slot(v, NT);
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
  if(e == cudaSuccess) e = pz_launch_single(conf, p, sm, stream);
  launches++;
  if(profiling) cudaEventRecord(prof_ev[2], stream);
  if(tv[1]) cudaEventRecord(tv[1], stream);
  if(e == cudaSuccess) {
    int G = 0;
    if(f64 || (test_energy_passes != 1 && ensure_pmap(f32))) {
      // the partial arrays staged by TMA, eighteen 8 x 8 x 8 boxes per work unit
      TmaEnergyArgs ta;
      ta.pmap = pmap, ta.oovv = oovv_f, ta.t1 = t1_f, ta.oovv_d = oovv, ta.t1_d = t1, ta.eo = eo, ta.ev = ev;
      ta.tiles = (const int3*) e_tiles;
      ta.ntiles = e_ntiles, ta.o = o, ta.v = v, ta.tri = bt_tri, ta.base = bt_ctrl + 2, ta.part = bt_part;
      ta.want_sens = sens != nullptr, ta.err = d_err;
      ta.spin       = test_spin_limit && test_skip_loads == 2 ? test_spin_limit : sm100::kSpinLimit;
      ta.skip_loads = test_skip_loads == 2;
      // box stages: two for FP32 boxes (2 CTAs / SM), one for float-float boxes (2 CTAs / SM rather
      // than 1), the faster of the two for each element type on GB300; knob 2 takes the other
      const int nst_default = f32 ? 2 : 1;
      const int nst         = f64 ? 1 : test_energy_passes == 2 ? 3 - nst_default : nst_default;
      G                     = std::min(e_ntiles, energy_tma_grid(f64 ? 2 : f32 ? 1 : 0, nst));
      const dim3 grid(G, nslots);
      if(f64) energy_tma_batch_kernel<double, 1><<<grid, EM_THREADS, em_smem_bytes<double, 1>(), stream>>>(ta);
      else if(f32 && nst == 2)
        energy_tma_batch_kernel<float, 2><<<grid, EM_THREADS, em_smem_bytes<float, 2>(), stream>>>(ta);
      else if(f32) energy_tma_batch_kernel<float, 1><<<grid, EM_THREADS, em_smem_bytes<float, 1>(), stream>>>(ta);
      else if(nst == 2)
        energy_tma_batch_kernel<float2, 2><<<grid, EM_THREADS, em_smem_bytes<float2, 2>(), stream>>>(ta);
      else energy_tma_batch_kernel<float2, 1><<<grid, EM_THREADS, em_smem_bytes<float2, 1>(), stream>>>(ta);
    } else {
      BatchEnergyArgs ea;
      ea.base_args = TiledEnergyArgs{nullptr, nullptr, nullptr, oovv_f, t1_f, eo, ev, (const int3*) e_tiles, e_ntiles,
                                     o, v, 0, 0, 0, nullptr, sens != nullptr};
      ea.tri = bt_tri, ea.base = bt_ctrl + 2, ea.F = bt_F, ea.part = bt_part;
      G = std::min(e_ntiles, energy_grid(f32));
      if(f32) energy_tiled_batch_kernel<float><<<dim3(G, nslots), ET_THREADS, 0, stream>>>(ea);
      else energy_tiled_batch_kernel<float2><<<dim3(G, nslots), ET_THREADS, 0, stream>>>(ea);
    }
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
  const int conf = pz_conf_index(S);
  if(conf < 0) return fail(CCSDT_E_INVALID, "no persistent configuration for this slice count");
  if((s = ensure_slices(std::max(S, slices_ready), 0)) || (s = ensure_tmaps(S, kPzConfs[conf].NT, kPzConfs[conf].KC))) return s;
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
  long m = (long) tab.size() / 4;
  if(m == 0) return CCSDT_OK;
  int B = (int) std::min<long>(batch_slots, m);
  if(ovvv_direct) {
    // Cholesky-direct mode: triplets by blocks of occupied indices, and batches whose slabs fit
    // the cache together (3 per triplet at most)
    B = std::max(1, std::min(B, (int) (ovvv_nslab / 3)));
    std::vector<int> ijk(3 * m);
    for(long t = 0; t < m; t++)
      for(int q = 0; q < 3; q++) ijk[3 * t + q] = tab[4 * t + q];
    const std::vector<long> ord = ccsdt::slab_order(ijk.data(), m, (int) ovvv_nslab);
    std::vector<int>        sorted(tab.size());
    for(long t = 0; t < m; t++)
      for(int q = 0; q < 4; q++) sorted[4 * t + q] = tab[4 * ord[t] + q];
    tab.swap(sorted);
    use_graph = false; // every batch may form slabs first
  }
  // the slabs batch b reads (direct mode), formed before its launch
  auto slabs_for = [&](long b0, long cnt) -> ccsdt_status {
    if(!ovvv_direct) return CCSDT_OK;
    std::vector<int> need;
    for(long t = b0; t < b0 + cnt; t++)
      for(int q = 0; q < 3; q++) need.push_back(tab[4 * t + q]);
    return ensure_ovvv(need.data(), (int) need.size(), true);
  };
  if((s = ensure_batch(S, B))) return s;
  if(bt_tri_cap < m) {
    if(bt_tri) cudaFree(bt_tri);
    bt_tri     = nullptr;
    bt_tri_cap = 0; // until the new table is in place
    if(dev_malloc((void**) &bt_tri, tab.size() * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "triplet table");
    }
    bt_tri_cap = m;
  }
  // natural-order table for a partial last batch
  const int  NT  = kPzConfs[conf].NT;
  const long per = items_per_slot(v, NT);
  const long rem = m % B;
  if(rem) {
    auto ids = cost_order((int) rem, v, NT);
    if(bt_order_partial) cudaFree(bt_order_partial);
    bt_order_partial = nullptr;
    if(dev_malloc((void**) &bt_order_partial, ids.size() * sizeof(unsigned)) != cudaSuccess) {
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
        if((s = slabs_for(b * B, B)) || (s = launch_batch(S, B, 0, true, tails, sens))) return s;
    }
  }
  if(rem) {
    if((s = slabs_for(full * B, rem)) || (s = launch_batch(S, (int) rem, (int) (per * rem), true, tails, sens)))
      return s;
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

// Times every compiled configuration for S digit planes on one triplet of this system (the
// contraction launch, CUDA events on the handle's stream, second of two runs) and keeps the
// fastest for the handle's later calls.  Every configuration gives bit-identical energies.
ccsdt_status ccsdt_handle::autotune(int S, double* ms, int* n, int* chosen) {
  if(S < 1 || S > OZ_MAX_SLICES) return fail(CCSDT_E_INVALID, "autotune: slices must be 1 to 8");
  if(!uploaded) return fail(CCSDT_E_STATE, "autotune before a successful upload");
  std::vector<int> cands;
  for(int c = 0; c < kPzNConfs; c++)
    if(kPzConfs[c].S == S) cands.push_back(c);
  if(n) *n = (int) cands.size();
  if(o < 2) { // no triplet with i < k: nothing to time, keep the default
    pz_tuned[S] = true;
    if(chosen) *chosen = 0;
    return CCSDT_OK;
  }
  ccsdt_status s;
  if((s = ensure_scratch()) || (s = ensure_triplet_slots(1)) || (s = ensure_slices(std::max(S, slices_ready), 0)))
    return s;
  if(!d_err) return fail(CCSDT_E_STATE, "autotune: device error flag missing");
  if(cudaMemsetAsync(d_err, 0, sizeof(int), stream) != cudaSuccess) return fail(CCSDT_E_CUDA, "autotune: memset");
  const int tri[3] = {0, o / 2, o - 1};
  // the phase timers serve the measurement; the caller's accumulated phase times are kept
  const bool   pt = phase_timing;
  const double saved[3] = {phase_ms[0], phase_ms[1], phase_ms[2]};
  const long   sb = phase_batches, st = phase_triplets;
  phase_timing     = true;
  int    best   = -1;
  double best_t = 0.0;
  for(size_t q = 0; q < cands.size() && !s; q++) {
    pz_conf_idx[S] = cands[q];
    double t = 0.0;
    for(int rep = 0; rep < 2 && !s; rep++) {
      phase_ms[0] = phase_ms[1] = phase_ms[2] = 0.0;
      s = run_batched(S, 1, tri, false, nullptr, nullptr, nullptr);
      t = phase_ms[0];
    }
    if(ms) ms[q] = t;
    if(!s && (best < 0 || t < best_t)) best = (int) q, best_t = t;
  }
  phase_timing     = pt;
  for(int q = 0; q < 3; q++) phase_ms[q] = saved[q];
  phase_batches  = sb;
  phase_triplets = st;
  if(!s) s = check_device_error();
  if(s) {
    pz_conf_idx[S] = -1;
    return s;
  }
  pz_conf_idx[S] = cands[best];
  pz_tuned[S]    = true;
  if(chosen) *chosen = best;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_tile_configs(int slices, int* n, int* nt_st_kc) {
  if(!n) return CCSDT_E_INVALID;
  int m = 0;
  for(int c = 0; c < kPzNConfs; c++)
    if(kPzConfs[c].S == slices) {
      if(nt_st_kc) {
        nt_st_kc[3 * m]     = kPzConfs[c].NT;
        nt_st_kc[3 * m + 1] = kPzConfs[c].ST;
        nt_st_kc[3 * m + 2] = kPzConfs[c].KC;
      }
      m++;
    }
  *n = m;
  return m ? CCSDT_OK : CCSDT_E_INVALID;
}

extern "C" ccsdt_status ccsdt_autotune(ccsdt_handle* h, int slices, double* ms, int* n, int* chosen) {
  if(!h) return CCSDT_E_INVALID;
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  return h->autotune(slices, ms, n, chosen);
}

extern "C" ccsdt_status ccsdt_set_tile_config(ccsdt_handle* h, int slices, int index) {
  if(!h) return CCSDT_E_INVALID;
  if(slices < 1 || slices > OZ_MAX_SLICES)
    return h->fail(CCSDT_E_INVALID, "ccsdt_set_tile_config: slices must be 1 to 8");
  int m = 0;
  for(int c = 0; c < kPzNConfs; c++)
    if(kPzConfs[c].S == slices) {
      if(m == index) {
        h->pz_conf_idx[slices] = c;
        h->pz_tuned[slices]    = true;
        return CCSDT_OK;
      }
      m++;
    }
  return h->fail(CCSDT_E_INVALID, "ccsdt_set_tile_config: no configuration " + std::to_string(index));
}

extern "C" ccsdt_status ccsdt_debug_set_wait_test(ccsdt_handle* h, unsigned spin_limit, int skip_loads) {
  if(!h) return CCSDT_E_INVALID;
  h->test_spin_limit = spin_limit;
  if(skip_loads < 0 || skip_loads > 2) return CCSDT_E_INVALID;
  h->test_skip_loads = skip_loads;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_debug_set_energy_kernel(ccsdt_handle* h, int passes) {
  if(!h || passes < 0 || passes > 2) return CCSDT_E_INVALID;
  h->test_energy_passes = passes;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_debug_set_window(ccsdt_handle* h, int k) {
  if(!h || k < 0) return CCSDT_E_INVALID;
  h->test_window_k = k;
  return CCSDT_OK;
}
