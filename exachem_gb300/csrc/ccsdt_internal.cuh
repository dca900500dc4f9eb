// Handle internals shared by the C-ABI translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ccsdt.h"
#include "ovvv_slabs.h"

namespace ccsdt {
struct OzBatch;
// BF16-digit Ozaki GEMMs (mma.sync kernel) of up to three jobs on a stream, and its tile count
cudaError_t oz_gemm_bf16(const OzBatch& b, int njobs, long long max_tiles, cudaStream_t st);
long long   oz_gemm_tiles(long long M, long long N);
// Every device allocation of the handle-based paths goes through here: cudaMalloc, except that a
// testing countdown (ccsdt_debug_fail_alloc) can make the n-th call fail as an out-of-memory
// cudaMalloc would (*p = nullptr, cudaErrorMemoryAllocation), so the error paths can be exercised.
cudaError_t dev_malloc(void** p, size_t bytes);
} // namespace ccsdt

constexpr int kEnergyBlocks = 1216; // 8 x 152 SMs
constexpr int kTiledBlocks  = 1216; // upper bound of the tiled energy's persistent grid

struct ccsdt_handle {
  int              device = 0, o = 0, v = 0;
  std::vector<int> occ_tiles, vir_tiles;
  cudaStream_t     stream = nullptr, own_stream = nullptr;
  cudaEvent_t      prof_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  bool             profiling  = false;
  cudaEvent_t      ev0 = nullptr, ev1 = nullptr;

  // resident inputs (C-ABI layouts) and kappa-contiguous copies
  double *eo = nullptr, *ev = nullptr, *t1 = nullptr, *t2 = nullptr, *oovv = nullptr,
         *ooov = nullptr, *ovvv = nullptr, *t2h = nullptr, *ooovh = nullptr;
  unsigned long long* d_count = nullptr;
  bool                uploaded = false;
  int                 slices_ready = 0;

  // per-triplet scratch
  double *P12 = nullptr, *P34 = nullptr, *P56 = nullptr, *part = nullptr, *res = nullptr;
  double* etrip     = nullptr;
  long    etrip_cap = 0;

  // split-precision state: digit planes (BF16 or INT8), exponents, FP32 copies, ff scratch
  std::vector<void*> slice_bufs;
  int                slice_variant = -1, kp_v = 0, kp_o = 0;
  void *             sl_t2 = nullptr, *sl_t2h = nullptr, *sl_ovvv = nullptr, *sl_ooovh = nullptr;
  int *              ex_t2 = nullptr, *ex_t2h = nullptr, *ex_ovvv = nullptr, *ex_ooovh = nullptr;
  long long          pl_t2 = 0, pl_t2h = 0, pl_ovvv = 0, pl_ooovh = 0;
  float *            oovv_f = nullptr, *t1_f = nullptr;
  float2 *           F12 = nullptr, *F34 = nullptr, *F56 = nullptr;
  // tcgen05 path: TMA maps over the digit planes (built once per slicing) and an error flag
  CUtensorMap        tmaps[9];
  bool               tmaps_ready = false;
  int                tmaps_S     = 0, tmaps_NT = 0, tmaps_KC = 0;
  int*               d_err       = nullptr;
  int*               e_tiles     = nullptr; // sorted virtual block triples of the tiled energy
  int                e_ntiles    = 0;
  double*            e_part      = nullptr;
  // a-posteriori estimate slots of the triplet being run (nullptr: not collected)
  float*             cur_tail    = nullptr;
  double*            cur_sens    = nullptr;

  long        launches       = 0;
  double      last_err_bound = 0.0;
  std::string err;

  std::vector<double*> owned;
  std::vector<void*>   owned_bytes;

  // Cholesky-direct mode (ccsdt_upload_cholesky_direct): (ia|bc) formed slab by slab (one occupied
  // index: v^3 values) from the vectors into `ovvv`, which then holds ovvv_nslab slots
  bool              ovvv_direct = false;
  long long         ovvv_nslab  = 0;         // slabs `ovvv` holds (o outside the direct mode)
  int               n_chol      = 0;
  double *          chol_ov = nullptr, *chol_vv = nullptr; // L[i][a][Q], L[b][c][Q] (direct mode)
  ccsdt::SlabCache  slabs;
  std::vector<char> slab_sliced;             // the slot's digit planes are current
  std::vector<char> slab_exact;              // the slot's slab was formed in FP64 (else by an Ozaki GEMM)
  bool              slab_split_build = true; // split-path calls form slabs from digit planes of the vectors
  long              slab_forms  = 0;         // slabs formed since the upload (re-formations included)
  void*             chol_planes = nullptr;   // BF16 digit planes of L_ov and L_vv (+ row exponents)
  long long         chol_kq     = 0;         // their padded Q extent
  int*              d_slab_of   = nullptr;   // index -> slot table read by the contraction kernel
  // makes the slabs of need[0..n) resident (formed and, with planes, sliced into digit planes)
  // and the device table current; a no-op outside the direct mode
  ccsdt_status      ensure_ovvv(const int* need, int n, bool planes);
  const double*     ovvv_slab(int x) const {
    return ovvv + (long long) (ovvv_direct ? slabs.slot(x) : x) * v * v * v;
  }

  ~ccsdt_handle();
  ccsdt_status fail(ccsdt_status s, const std::string& msg);
  ccsdt_status alloc(double** p, size_t n);
  ccsdt_status ensure_scratch();
  // nslab < 0: every array whole (ovvv = o slabs of v^3); nslab >= 3: the Cholesky-direct mode,
  // ovvv a cache of nslab slabs formed from the vectors as the triplets need them
  ccsdt_status ensure_inputs(long long nslab = -1);
  ccsdt_status finish_inputs(const char* who);
  // device-side retile of spin-orbital tile blocks (ccsdt_upload_blocks)
  double*      blk_stage = nullptr;    // device staging of a call's block data
  long long    blk_stage_cap = 0;      // doubles
  int*         blk_meta = nullptr;     // per block: 4 tile ids + 2 offset words
  long         blk_meta_cap = 0;
  int*         blk_tiles = nullptr;    // occupied / virtual tile offsets and extents
  bool         blocks_open = false;    // between ccsdt_upload_begin and ccsdt_upload_end
  ccsdt_status ensure_triplet_slots(long n);
  ccsdt_status run_triplet_fp64(int i, int j, int k, double* eout);
  ccsdt_status run_fp64_list(long n, const int* tri_host);
  ccsdt_status run_list(const ccsdt_opts* opts, long n, const int* tri_host);
  ccsdt_status run_split(const ccsdt_opts* opts, long n, const int* tri_host);
  ccsdt_status ensure_slices(int S, int variant);
  ccsdt_status run_triplet_split(int i, int j, int k, int S, int variant, double* eout);
  ccsdt_status ensure_tmaps(int S, int NT, int KC);
  ccsdt_status run_triplet_tc(int i, int j, int k, int S, double* eout);
  bool         tc_eligible(int S, int variant) const; // per-triplet tcgen05 kernel
  bool         pz_eligible(int S, int variant) const; // persistent tcgen05 kernel
  double*      part_buf() { return part; }
  ccsdt_status launch_energy_tiled(int i, int j, int k, double* eout, bool f32 = false);
  ccsdt_status run_triplet_S(int i, int j, int k, int S, double* eout);
  // learned slice count
  ccsdt_status run_learned(const ccsdt_opts* opts, long n, const int* tri_host);
  double       truncation_estimate(float tail_sq, double sens) const;
  ccsdt_status features(long n, const int* tri_dev, float* feats_dev);
  ccsdt_status ensure_stats();
  std::vector<float> model;          // MLP parameters (host copy); empty = no model
  void*              model_bf16 = nullptr;
  int*               st_slab = nullptr, *st_pair = nullptr, *st_hole = nullptr; // exponent statistics
  int                stats_for = -1;  // slicing generation the statistics belong to
  int                slice_gen = 0;
  // batched persistent path
  float2*   bt_F = nullptr;          // P arrays of the batch slots
  bool      last_batched = false;    // the last split-precision call ran the persistent path
  bool      last_p_f32   = false;    // ... and stored its partial arrays in FP32
  bool      last_p_f64   = false;    // ... or in FP64
  int       p_storage    = 0;        // the call's opts->p_storage
  // FP32 partial arrays for S <= kPF32MaxS digit planes unless the call asks otherwise
  static constexpr int kPF32MaxS = 3;
  bool p_f32(int S) const { return p_storage == 2 || (p_storage == 0 && S <= kPF32MaxS); }
  double*   bt_part = nullptr;
  int       bt_B = 0, bt_order_key = -1;
  unsigned* bt_order = nullptr, *bt_order_partial = nullptr;
  unsigned  bt_nitems = 0;
  int*      bt_ctrl = nullptr;       // queue counters and batch base
  int*      bt_tri = nullptr;        // triplet table (i, j, k, output index)
  long      bt_tri_cap = 0;
  int       batch_slots = 4;         // triplets per batch
  unsigned  test_spin_limit = 0;     // testing: bounded-wait poll limit of the persistent kernel (0: default)
  int       test_skip_loads = 0;     // testing: the persistent kernel issues no TMA loads
  int       test_window_k = 0;       // testing: shorter exact K windows than the slice count allows
  // persistent-contraction configuration per S (index into kPzConfs, -1 = the default), set by
  // the autotuner or ccsdt_set_tile_config; tuned[S]: the autotuner has run for S
  int          pz_conf_idx[9] = {-1, -1, -1, -1, -1, -1, -1, -1, -1};
  bool         pz_tuned[9]    = {false, false, false, false, false, false, false, false, false};
  int          pz_conf_index(int S) const;
  ccsdt_status autotune(int S, double* ms, int* n, int* chosen);
  long      graph_replays = 0;
  ccsdt_status ensure_batch(int S, int B);
  ccsdt_status launch_batch(int S, int nslots, int nitems_override, bool advance, float* tails, double* sens);
  ccsdt_status run_batched(int S, long n, const int* tri, bool use_graph, float* tails, double* sens,
                           const int* out_map = nullptr);
  // per-call statistics of the learned mode
  double             learned_mean_slices = 0.0;
  long               learned_fallbacks   = 0;
  double             learned_cost_products = 0.0; // digit-plane products run, incl. escalations
  ccsdt_status check_device_error();
  bool         force_mma_sync = false; // use the mma.sync slice kernel even where tcgen05 applies
  bool         fp64_ff_energy = false; // testing: FP64 contractions, then the float-float energy
  bool         fp64_unfused   = false; // the two-stage FP64 path (partial arrays in HBM, then the energy)
  bool         w_debug        = false; // ccsdt_debug_triplet_w is running
  int*         fx_tiles       = nullptr; // work units of the fused FP64 kernel
  int          fx_ntiles = 0, fx_grid = 0;
  ccsdt_status ensure_fused_tiles();
  ccsdt_status run_triplet_fp64_fused(int i, int j, int k, double* eout);
  // live per-phase timing of the batched path: 3 events per batch, read after the call
  bool                     phase_timing = false, capturing = false;
  std::vector<cudaEvent_t> tev;
  size_t                   tev_used = 0;
  std::vector<int>         tev_slots;
  double                   phase_ms[3]   = {0, 0, 0}; // contraction, energy + reduction, unused
  long                     phase_batches = 0, phase_triplets = 0;
  ccsdt_status collect_phase_times();
  int          energy_grid_ = 0, energy_grid_f32_ = 0; // resident CTAs of the tiled energy kernels
  int          energy_grid(bool f32 = false);            // (one full wave)
  // TMA map over the batch's partial arrays for energy_tma_batch_kernel (rebuilt when the batch
  // scratch or the element type changes); false when the layout does not suit TMA
  CUtensorMap  pmap;
  const void*  pmap_base = nullptr;
  int          pmap_B = 0, pmap_f32 = -1;
  int          energy_tma_grid_[6] = {0, 0, 0, 0, 0, 0};
  int          test_energy_passes = 0; // testing: 1 = the pass-by-pass energy kernel even where TMA
                                       // suits, 2 = the TMA kernel with the other number of box stages
  bool         ensure_pmap(bool f32);
  int          energy_tma_grid(int kind, int nst);
};
