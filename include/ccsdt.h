/*
 * ccsdt.h - C ABI of the GB300 CCSD(T) perturbative-triples library (closed shell; open shell
 * through ccsdt_energy_spin_orbital).
 *
 * This is the drop-in boundary for ExaChem's fused (T) driver:
 *
 *   std::tuple<T,T,double,double> CCSD_T_Fused_Driver<T>::execute(
 *       ChemEnv&, ExecutionContext&, std::vector<int>& k_spin, const TiledIndexSpace& MO,
 *       Tensor<T>& d_t1, Tensor<T>& d_t2, V2Tensors<T>& d_v2, std::vector<T>& k_evl_sorted,
 *       T hf_ccsd_energy, bool is_restricted, LRUCache x6, bool seq_h3b, bool tilesize_opt)
 *   (exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:73-81, 91-546; called from ccsd_t.cpp:253-256)
 *
 * which takes T1/T2, the V2 integral blocks, orbital energies and the triples tile
 * layout and returns (E[T], E(T), work seconds, total seconds).  The C++ adapter in
 * include/exachem_compat/ccsd_t_fused_driver.hpp keeps that signature and calls the
 * functions below.  Everything here uses plain pointers and sizes; no exceptions,
 * no exit(): every call returns a ccsdt_status and ccsdt_last_error() explains it.
 *
 * Closed-shell spatial layouts (row-major, chemist notation; o occupied, v virtual):
 *   eps_occ[o], eps_vir[v]                 orbital energies (Eh)
 *   t1[o][v]          t1[i][a]             = t_i^a
 *   t2[o][o][v][v]    t2[i][j][a][b]       = t_ij^ab        (ExaChem t2_abab(a,b,i,j))
 *   oovv[o][o][v][v]  oovv[i][j][a][b]     = (ia|jb)        (alpha-beta block of v2ijab)
 *   ooov[o][o][o][v]  ooov[i][j][k][a]     = (ij|ka)        (Coulomb part of v2ijka)
 *   ovvv[o][v][v][v]  ovvv[i][a][b][c]     = (ia|bc)        (Coulomb part of v2iabc)
 * The spin-orbital blocks ExaChem passes are the antisymmetrised combinations of these
 * (exachem/cholesky/v2tensors.cpp:67-86, exachem/cc/ccsd/cd_ccsd_cs_ann.cpp:949-973).
 */
#ifndef CCSDT_GB300_H
#define CCSDT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CCSDT_OK           = 0,
  CCSDT_E_INVALID    = 1, /* bad argument (null pointer, negative size, unknown mode)      */
  CCSDT_E_BAD_LAYOUT = 2, /* tile layout inconsistent with o / v                            */
  CCSDT_E_OOM        = 3, /* device or host allocation failed                               */
  CCSDT_E_NONFINITE  = 4, /* NaN or Inf in the inputs or in the result                      */
  CCSDT_E_TIMEOUT    = 5, /* a bounded device-side wait gave up                             */
  CCSDT_E_CUDA       = 6, /* CUDA runtime / driver error                                    */
  CCSDT_E_STATE      = 7  /* call out of order (e.g. energy before upload)                  */
} ccsdt_status;

/* Precision of the triples contractions. */
typedef enum {
  CCSDT_MODE_FP64    = 0, /* FP64 DMMA tensor-core contractions, FP64 energy (the drop-in) */
  CCSDT_MODE_OZAKI   = 1, /* split-precision: BF16 slices on tcgen05, float-float recombination */
  CCSDT_MODE_LEARNED = 2  /* split-precision with a per-triplet slice count from the MLP   */
} ccsdt_mode;

/* The triples tile layout: occupied and virtual tile extents (ragged allowed).
 * ExaChem's MO space repeats these for alpha and beta (cholesky_2e.cpp:230-285). */
typedef struct {
  int        o, v;
  int        n_occ_tiles;
  const int* occ_tiles; /* extents, sum == o */
  int        n_vir_tiles;
  const int* vir_tiles; /* extents, sum == v */
} ccsdt_layout;

typedef struct {
  int    mode;          /* ccsdt_mode                                                         */
  int    slices;        /* Ozaki digit planes per operand (1..8) for CCSDT_MODE_OZAKI         */
  int    slice_kind;    /* 0: BF16 digits on the tensor cores (FP32 accumulation),            */
                        /* 1: INT8 digits (INT32 accumulation)                                */
  int    use_graph;     /* capture the per-call launch sequence in a CUDA graph               */
  int    shard_index;   /* process triplets t with t % shard_count == shard_index; the        */
  int    shard_count;   /* caller sums the partial energies (0 or 1 = every triplet)          */
  double energy_budget; /* LEARNED: accept when 3 sum_t sigma_t <= budget x sum_t |E(T)_t|   */
                        /* (sigma_t: estimated error of triplet t; default 1e-8)              */
  int    budget_triplets; /* ignored (the linear acceptance test needs no share for a call that */
                          /* is part of a larger computation); kept for the struct layout       */
  int    test_kernel;     /* testing: 0 default, 1 mma.sync slice kernel, 2 per-triplet tcgen05, */
                          /* 3 FP64 contractions with the split path's float-float energy,       */
                          /* 5 (FP64 mode) the two-stage FP64 path: partial arrays, then energy  */
  int    autotune;        /* 1: ccsdt_energy / ccsdt_triplet_energies run ccsdt_autotune for each
                             slice count they use, once per handle, before the timed work      */
  int    p_storage;       /* split path: element type of the triples' partial arrays between the
                             contraction and the energy: 0 FP32 for 1..3 digit planes (their
                             rounding, unbiased and averaged over a triplet's v^3 elements, moves
                             E(T) by ~1e-11 relative, far below the truncation of 3 planes),
                             float-float from 4 planes on; 1 float-float always; 2 FP32 always;
                             3 FP64: the digit levels folded and the terms summed in FP64, the
                             energy's W, denominator division and compensated sums in FP64
                             (needs an even v)                                                 */
  int    reserved[2];
} ccsdt_opts;

typedef struct {
  double e_bracket_T;      /* E[T]                                                            */
  double e_paren_T;        /* E(T)                                                            */
  double abs_err_bound;    /* LEARNED: 3-sigma a-posteriori estimate of |E(T) - E(T)_fp64|     */
  double seconds;          /* device time of the call                                         */
  double flops_executed;   /* 2 x multiply-adds of the contractions (FP64-equivalent)         */
  double flops_ref_equiv;  /* the reference's own spin-orbital op count for this layout       */
  long   n_triplets;       /* occupied triplets i <= j <= k processed                         */
  long   n_tasks_ref;      /* tile-block tasks the reference would run for this layout        */
} ccsdt_result;

typedef struct ccsdt_handle ccsdt_handle;

/* Create a handle bound to CUDA device `device` for the given layout; -1 = the calling
 * thread's current device (the one the host runtime selected for this rank). */
ccsdt_status ccsdt_create(ccsdt_handle** out, const ccsdt_layout* layout, int device);

/* Copy the inputs into handle-owned device memory.  `on_device` = 0: host pointers
 * (pinned or pageable), 1: device pointers on the handle's device.  Checks finiteness. */
ccsdt_status ccsdt_upload(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                          const double* t1, const double* t2, const double* oovv,
                          const double* ooov, const double* ovvv, int on_device);

/* The occupied triplets i <= j <= k of one shard, in the order ccsdt_energy runs them: the
 * t-th triplet of the lexicographic list belongs to shard t mod shard_count.  Host-only (no
 * device work).  tri = NULL returns the count in *n; otherwise tri[3 * *n] receives them.
 * Replaces the reference's dynamic task split over ranks (a global atomic counter,
 * ac->fetch_add at ccsd_t_fused_driver.hpp:172,456): every triplet of a closed-shell run costs
 * the same 12 v^3 (o + v) flops, so a static split is balanced and needs no counter. */
ccsdt_status ccsdt_shard_triplets(int o, int shard_index, int shard_count, long* n, int* tri);

/* Device-side retile of ExaChem's spin-orbital tile blocks: instead of gathering the spatial
 * arrays of ccsdt_upload on the host, hand over the blocks as Tensor::get returns them (row-major
 * in the tensor's index order); the library copies them to the device and scatters them into its
 * arrays with one kernel (the gathers at ccsd_t_all_fused_doubles1.hpp:216-246,
 * ccsd_t_all_fused_doubles2.hpp:211-239,335-343 transpose each block on the host).
 *   ccsdt_upload_begin(h, eps_occ, eps_vir, t1, on_device)   small inputs; the four-index arrays zeroed
 *   ccsdt_upload_blocks(h, kind, n, tiles[4n], offsets[n], data, data_len, on_device)   any number
 *   ccsdt_upload_end(h)                                      finiteness check, repacks; ready
 * tiles: per block the positions of its four tiles in the layout's occupied / virtual tile lists
 * (alpha tiles; beta blocks are not needed for the closed shell), in the block's index order;
 * offsets: element offset of each block in data (data_len doubles).  Blocking (the caller may
 * reuse its buffers when the call returns).  No counterpart as a call in the reference. */
typedef enum {
  CCSDT_BLOCKS_T2   = 0, /* t2(a_alpha, b_beta, i_alpha, j_beta) block (A, B, I, J), [a][b][i][j]      */
  CCSDT_BLOCKS_OOVV = 1, /* v2ijab(i_a, j_b, a_a, b_b) = (ia|jb) block (I, J, A, B), [i][j][a][b]     */
  CCSDT_BLOCKS_OOOV = 2, /* v2ijka(i_a, k_b, j_a, a_b) = (ij|ka) block (I, K, J, A), [i][k][j][a]     */
  CCSDT_BLOCKS_OVVV = 3  /* v2iabc(i_a, b_b, a_a, c_b) = (ia|bc) block (I, B, A, C), [i][b][a][c]     */
} ccsdt_block_kind;
ccsdt_status ccsdt_upload_begin(ccsdt_handle* h, const double* eps_occ, const double* eps_vir, const double* t1,
                                int on_device);
ccsdt_status ccsdt_upload_blocks(ccsdt_handle* h, int kind, long n, const int* tiles, const long long* offsets,
                                 const double* data, long long data_len, int on_device);
ccsdt_status ccsdt_upload_end(ccsdt_handle* h);

/* Inputs with the integral blocks built on the device from spatial Cholesky vectors
 * L[p][q][Q] (the alpha-alpha block of the reference's cholVpr, symmetric in p, q):
 *   chol_oo[o][o][n_chol], chol_ov[o][v][n_chol], chol_vv[v][v][n_chol]  (row-major, Q fastest)
 *   oovv = (ia|jb), ooov = (ij|ka), ovvv = (ia|bc) = sum_Q L L       (FP64 DMMA GEMMs)
 * eps_occ, eps_vir, t1, t2 as in ccsdt_upload.  Replaces exachem/cholesky/v2tensors.cpp:66-88
 * (setupV2Tensors: v2ijab / v2ijka / v2iabc) for the blocks the closed-shell (T) reads, so the
 * o v^3 ovvv block never crosses the host link.  Blocking; non-finite inputs -> CCSDT_E_NONFINITE. */
ccsdt_status ccsdt_upload_cholesky(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                   const double* t1, const double* t2, int n_chol, const double* chol_oo,
                                   const double* chol_ov, const double* chol_vv, int on_device);

/* Cholesky-direct inputs: as ccsdt_upload_cholesky, but (ia|bc) is never held whole.  The handle
 * keeps chol_ov and chol_vv on the device and forms (ia|bc) one occupied index at a time (a slab:
 * all a, b, c; one DMMA GEMM of v x v^2 x n_chol) into a cache of max_ovvv_slabs slabs of v^3
 * doubles, as the triplets need them: the calls visit their triplets by blocks of max_ovvv_slabs / 3
 * occupied indices, the least recently used slab not needed by the current batch makes room, and
 * the split path slices each slab into digit planes when it is formed.  Systems whose o v^3
 * (ia|bc) exceeds the device memory then run, at the cost of forming slabs more than once
 * (ccsdt_ovvv_slab_builds); max_ovvv_slabs >= o forms each slab once.  Energies equal those of
 * ccsdt_upload_cholesky on the same vectors.  max_ovvv_slabs >= 3 (clamped to o); the split path
 * needs the persistent tcgen05 kernel (BF16 digits) and runs batches of at most max_ovvv_slabs / 3
 * triplets; CCSDT_MODE_LEARNED is not available in this mode (CCSDT_E_INVALID). */
ccsdt_status ccsdt_upload_cholesky_direct(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                          const double* t1, const double* t2, int n_chol, const double* chol_oo,
                                          const double* chol_ov, const double* chol_vv, int on_device,
                                          int max_ovvv_slabs);
/* (ia|bc) slabs formed since the last upload (the Cholesky-direct mode; 0 otherwise).  FP64 calls
 * form slabs with FP64 DMMA GEMMs; split-path calls form them as Ozaki GEMMs of six BF16 digit
 * planes of the vectors (relative error ~1e-12 of the slab's scale, far below the split (T)'s own),
 * and an FP64 call re-forms in FP64 any such slab it reads. */
long ccsdt_ovvv_slab_builds(const ccsdt_handle* h);
/* Testing: split-path calls form slabs with FP64 DMMA too (split = 0) or from digit planes (1, the
 * default). */
ccsdt_status ccsdt_debug_set_slab_build(ccsdt_handle* h, int split);
/* Testing, host only: the direct mode's visiting order (order[n]: triplet ids) and the number of
 * slabs it forms for triplets tri[3 n] run in batches of `batch` with max_ovvv_slabs slots;
 * CCSDT_E_STATE if a batch ever found a slab it needs missing. */
ccsdt_status ccsdt_debug_slab_schedule(int o, int max_ovvv_slabs, int batch, long n, const int* tri, long* order,
                                       long* builds);

/* Tile configurations of the persistent split-precision contraction (tcgen05 path, slices 1-8):
 *   ccsdt_tile_configs     lists the compiled ones for `slices`: *n of them, {N tile, pipeline
 *                          stages, K chunk} each in nt_st_kc[3 n] (nullable); index 0 is the default;
 *   ccsdt_autotune         times each on one triplet of the handle's system (CUDA events around the
 *                          contraction launch), keeps the fastest for the handle's later calls with
 *                          that slice count; ms[n] (nullable) the times, *chosen (nullable) the index;
 *   ccsdt_set_tile_config  selects one by index (testing, or a stored autotune result).
 * Every configuration gives bit-identical energies: the digit-level sums are exact integers
 * whatever the tiling, and each element's float-float fold does not depend on the tile.  The
 * reference has no counterpart (its kernels have fixed tile shapes). */
ccsdt_status ccsdt_tile_configs(int slices, int* n, int* nt_st_kc);
ccsdt_status ccsdt_autotune(ccsdt_handle* h, int slices, double* ms, int* n, int* chosen);
ccsdt_status ccsdt_set_tile_config(ccsdt_handle* h, int slices, int index);

/* Full (T): E[T] and E(T) over every occupied triplet of the shard in opts.  Blocking. */
ccsdt_status ccsdt_energy(ccsdt_handle* h, const ccsdt_opts* opts, ccsdt_result* out);

/* Per-triplet contributions for an explicit list tri[3n] (each i <= j <= k < o):
 * e_bracket[t], e_paren[t] receive host doubles.  Used for sampled parity checks. */
ccsdt_status ccsdt_triplet_energies(ccsdt_handle* h, const ccsdt_opts* opts, long n,
                                    const int* tri, double* e_bracket, double* e_paren);

/* Launch all further work of this handle on `stream` (a cudaStream_t on the handle's
 * device; NULL restores the handle's own stream).  Lets a caller time the calls with
 * CUDA events on its own stream.  No counterpart in the reference (it used one pooled
 * stream per rank, ccsd_t_all_fused.hpp:108). */
ccsdt_status ccsdt_set_stream(ccsdt_handle* h, void* stream);

/* Live per-phase device timing of the batched split-precision path (the persistent tcgen05
 * kernel).  on != 0 starts the accumulation (and zeroes it): CUDA events on the handle's
 * stream around the contraction launch (l-sum and d-sum terms) and around the energy launches
 * of every batch, read when the call returns.  ccsdt_phase_times gives the accumulated
 * milliseconds ms3 = {contraction, energy, 0} and the numbers of batches and triplets they
 * cover.  Batches replayed from a CUDA graph are not timed.  No counterpart in the reference
 * (its timers are host-side, ccsd_t.cpp). */
ccsdt_status ccsdt_set_phase_timing(ccsdt_handle* h, int on);
ccsdt_status ccsdt_phase_times(const ccsdt_handle* h, double* ms3, long* batches, long* triplets);

/* Device milliseconds of each phase of one triplet (i <= j <= k), measured with CUDA
 * events on the handle's stream: out_ms[0] l-sum contractions, [1] d-sum contractions,
 * [2] energy, [3] reduction.  Profiling aid; no counterpart in the reference. */
ccsdt_status ccsdt_profile_triplet(ccsdt_handle* h, const ccsdt_opts* opts, int i, int j, int k,
                                   double* out_ms);

/* Connected triples W_abc (v^3 doubles, [a][b][c], host memory) of one triplet
 * i <= j <= k, i < k, in the precision `opts` selects.  Verification aid: no counterpart
 * in the reference, whose t3 blocks stay internal (ccsd_t_all_fused_cpu.hpp:103-170). */
ccsdt_status ccsdt_debug_triplet_w(ccsdt_handle* h, const ccsdt_opts* opts, int i, int j, int k,
                                   double* w_host);

/* Testing the failure paths (no counterpart in the reference, whose errors end the process:
 * the exit(100) macros of ccsd_t_common.hpp:26-41).
 *   ccsdt_debug_fail_alloc: the nth device allocation the library makes from now on (any handle,
 *     any call) fails as an out-of-memory cudaMalloc would; 0 switches this off.  *attempts
 *     (nullable) receives the number of allocations attempted since the previous call.  The
 *     calls that meet the failure return CCSDT_E_OOM and leave their handle destroyable.
 *   ccsdt_debug_set_wait_test: the split-precision persistent kernel's bounded waits give up after
 *     spin_limit polls (0: the default limit), and with skip_loads = 1 it announces each stage's
 *     bytes but issues no TMA load, so its stage waits run out: the call returns CCSDT_E_TIMEOUT,
 *     the kernel having released its tensor memory, and the handle stays usable.  skip_loads = 2
 *     does the same to the TMA energy kernel (the limit then applies to its waits): it announces
 *     each work unit's box bytes without loading them, its threads stop after their first wait
 *     runs out, and the call returns CCSDT_E_TIMEOUT. */
ccsdt_status ccsdt_debug_fail_alloc(long nth, long* attempts);
ccsdt_status ccsdt_debug_set_wait_test(ccsdt_handle* h, unsigned spin_limit, int skip_loads);

/* Testing: the persistent split-precision kernel accumulates each contraction in windows of at most
 * k (rounded down to its K chunk, at least one chunk) instead of the longest window whose digit-level
 * sums stay exact for the slice count (0: that default).  Shorter windows are exact too; they
 * exercise the window-by-window fold that long contractions (v beyond the exact window) need. */
ccsdt_status ccsdt_debug_set_window(ccsdt_handle* h, int k);

/* Testing: the persistent split-precision path's energy kernel.  0 (default): the partial arrays
 * staged into shared memory by TMA tensor loads where their row pitch allows (v % 4 == 0 for FP32
 * partial arrays, v even for float-float), else the pass-by-pass kernel; 1: the pass-by-pass
 * kernel always (threads load the partial arrays and sum them into swizzled cubes); 2: the TMA
 * kernel with the other number of box stages (by default two for FP32 partial arrays - the next
 * unit's boxes load while the current one is evaluated - and one for float-float ones, where
 * two stages would leave one CTA per SM). */
ccsdt_status ccsdt_debug_set_energy_kernel(ccsdt_handle* h, int passes);

/* Number of kernel launches issued by the last ccsdt_energy / ccsdt_triplet_energies. */
long ccsdt_last_launch_count(const ccsdt_handle* h);

/* Reference-equivalent op count and task count for a layout (restricted, i.e. RHF):
 * the sum over tile-block tasks of 2 x product of sizes per enabled contraction, as
 * exachem/cc/ccsd_t/fused_common.hpp:34-261 counts it.  Pure host arithmetic. */
ccsdt_status ccsdt_reference_op_count(const ccsdt_layout* layout, double* ops, long* tasks);

/* The same count over MO tiles occ_a | occ_b | virt_a | virt_b of their own (open shell), with
 * is_restricted as the reference driver takes it (1: the two restricted spin filters; 0: none). */
ccsdt_status ccsdt_reference_op_count_so(int n_occ_a, const int* occ_a, int n_occ_b, const int* occ_b,
                                         int n_vir_a, const int* vir_a, int n_vir_b, const int* vir_b,
                                         int is_restricted, double* ops, long* tasks);

/* Allocation-free FP64 (T) for small problems.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc - a host runtime whose device memory is owned by
 * a pooled allocator (ExaChem's TAMM reserves the device through its RMM pool, so a
 * cudaMalloc beside it fails or fragments the pool), or a service held to a fixed device
 * budget.  All pointers are device pointers on the current device: the inputs in the
 * layouts above and `energies`, which receives {E[T], E(T)}.  Work is queued on `stream` (a
 * cudaStream_t, NULL = legacy default stream) and is complete when that stream is.
 * Every intermediate lives in one fixed device array of about 6.0 MB defined in the
 * library, which each GPU that loads the library keeps until the process exits; sizes
 * beyond o = 12 or v = 48 are rejected with CCSDT_E_INVALID.  The first call on a device
 * looks up that array's device address (make that first call before any stream capture)
 * and keeps it for the rest of the process: do not use this entry point across a
 * cudaDeviceReset.  All calls share the array: calls that overlap on the GPU race and give
 * wrong results, so order them on one stream or synchronise between them.  It calls no
 * cudaMalloc, cudaFree or allocating library routine. */
ccsdt_status ccsdt_energy_noalloc(int o, int v, const double* eps_occ, const double* eps_vir,
                                  const double* t1, const double* t2, const double* oovv,
                                  const double* ooov, const double* ovvv, double* energies,
                                  void* stream);

/* ---- open-shell (UHF) (T) over spin orbitals ------------------------------------------
 * ExaChem's fused driver with is_restricted = false (ccsd_t_fused_driver.hpp:383-392, the
 * spin filter and factor; its inputs come from ccsd_t.cpp:253-256).  Spin orbitals in
 * ExaChem's MO order: occupied alpha (oa) | occupied beta (ob), virtual alpha (va) | virtual
 * beta (vb); O = oa + ob, V = va + vb.  Dense row-major arrays in the index order of
 * ExaChem's tensors (exachem/cholesky/v2tensors.cpp:67-86 for the V2 blocks):
 *   eps_occ[O], eps_vir[V]      orbital energies
 *   t1[V][O]                    t1(a, i)
 *   t2[V][V][O][O]              t2(a, b, i, j)
 *   v2ijab[O][O][V][V]          <ij||ab>
 *   v2ijka[O][O][O][V]          <ij||ka>
 *   v2iabc[O][V][V][V]          <ia||bc>
 * Elements of spin-forbidden blocks are never read (they may hold anything).  FP64 DMMA
 * contractions over the spin-allowed blocks only; energies[0] = E[T], energies[1] = E(T)
 * (host memory).  on_device = 1: the arrays are device pointers on the current device; the
 * call first waits for all work already submitted to that device (cudaDeviceSynchronize), so
 * inputs still being written by the caller's kernels or copies on any stream are complete
 * before they are read; 0: host pointers, copied in by the call.  shard_index / shard_count: the call takes the
 * occupied triplets i < j < k with t % shard_count == shard_index (t counts them in
 * lexicographic order) and returns that part of the energies (shard_count 0 or 1: all).
 * seconds (may be NULL) receives the device time of the call, copies included.
 * Restricted (RHF) inputs in this form give the closed-shell energies. */
ccsdt_status ccsdt_energy_spin_orbital(int oa, int ob, int va, int vb, const double* eps_occ,
                                       const double* eps_vir, const double* t1, const double* t2,
                                       const double* v2ijab, const double* v2ijka,
                                       const double* v2iabc, int on_device, int shard_index,
                                       int shard_count, double* energies, double* seconds);

/* The same open-shell (T) with split-precision contractions: every operand of the spin-block
 * GEMMs cut into `slices` (1..6) BF16 digit planes carrying their rows' power-of-two scales (one
 * set per spin of the contraction index), exact FP32 level sums on the tensor cores (mma.sync),
 * float-float blocks; the energy is the FP64 one of ccsdt_energy_spin_orbital.  Arguments and
 * results as there. */
ccsdt_status ccsdt_energy_spin_orbital_split(int oa, int ob, int va, int vb, const double* eps_occ,
                                             const double* eps_vir, const double* t1, const double* t2,
                                             const double* v2ijab, const double* v2ijka,
                                             const double* v2iabc, int on_device, int shard_index,
                                             int shard_count, int slices, double* energies, double* seconds);

/* Testing: the contraction plan of triplet i < j < k of an open-shell system (pure host logic).
 * of[9]: for permutation p (ijk, jik, kji) and position q ((a; b c), (b; a c), (c; b a)) the
 * block the energy reads at of[3p + q], -1 where it is zero; blocks[14 b + ...] for b < *nblk:
 * x0, y0, z0, nx, ny, nz, has_d, d_k, d_a, d_b, has_s, s_k, s_a, s_b - block
 * X[x - x0][(y - y0) nz + z - z0] = - sum_e tt[d_a + x' V + e] vv[d_b + y' V^2 + z' V + e]
 * - sum_m uu[s_a + x' O + m] t2[s_b + y' V O^2 + z' O^2 + m], with tt[j][k][a][e] = t2(a,e,j,k),
 * vv[i][b][c][e] = <ie||bc>, uu[j][k][a][m] = <jk||ma>. */
ccsdt_status ccsdt_debug_spin_orbital_plan(int oa, int ob, int va, int vb, int i, int j, int k, int* of,
                                           long long* blocks, int* nblk);

/* ---- learned slice count (no counterpart in the reference) --------------------------
 * A 12 -> 64 -> 64 -> 7 MLP (ReLU, softmax over slice counts 2..8) predicts, per occupied
 * triplet, the smallest digit-plane count that keeps the triplet's energy error under a
 * budget.  Parameters are CCSDT_MLP_NPARAM floats: W1[64][12] b1[64] W2[64][64] b2[64]
 * W3[7][64] b3[7].  Training runs on the GPU in FP32 (hand-written forward/backward and
 * Adam kernels); inference runs in BF16.  All pointers below are host pointers. */
#define CCSDT_MLP_IN 12
#define CCSDT_MLP_HIDDEN 64
#define CCSDT_MLP_OUT 7
#define CCSDT_MLP_NPARAM (64 * 12 + 64 + 64 * 64 + 64 + 7 * 64 + 7)

/* grad = d(mean cross-entropy)/d(params) over n samples X[n][12] with labels 0..6 (slice
 * count - 2); *loss = the mean cross-entropy. */
ccsdt_status ccsdt_mlp_grad(const float* params, const float* X, const int* labels, int n, float* grad,
                            float* loss);

/* Adam training for `epochs` passes over shuffled minibatches of `batch`; init != 0 first
 * draws a seeded He-uniform initialisation into params.  params is updated in place. */
ccsdt_status ccsdt_mlp_train(const float* X, const int* labels, int n, int epochs, int batch, float lr,
                             unsigned seed, int init, float* params, float* final_loss);

/* BF16 inference: slices[s] = 2 + argmax of the logits (logits[n][7] optional). */
ccsdt_status ccsdt_mlp_predict(const float* params, const float* X, int n, int* slices, float* logits);

/* The 12 features of each triplet (host array feats[n][12]) the slice-count model reads. */
ccsdt_status ccsdt_triplet_features(ccsdt_handle* h, long n, const int* tri, float* feats);

/* Install (params != NULL, CCSDT_MLP_NPARAM floats) or clear the model CCSDT_MODE_LEARNED uses.
 * In that mode opts->slices is the full count used for the fallback (default 5) and
 * opts->energy_budget the relative per-triplet budget of the a-posteriori check. */
ccsdt_status ccsdt_set_slice_model(ccsdt_handle* h, const float* params);

/* Per-triplet energies at opts->slices digit planes (CCSDT_MODE_OZAKI, BF16 digits, 1..8
 * planes) together with the a-posteriori estimate est[t] of |E(T)_t - E(T)_t,fp64| that the
 * LEARNED mode checks against its budget: the estimated standard deviation of the triplet's
 * truncation error, from the last kept level's terms and the energy's sensitivity (a statistical
 * estimate, not a rigorous bound).  e_bracket may be NULL. */
ccsdt_status ccsdt_triplet_error_estimates(ccsdt_handle* h, const ccsdt_opts* opts, long n, const int* tri,
                                           double* e_bracket, double* e_paren, double* est);

/* Statistics of the last LEARNED call: mean predicted slice count, number of escalations (when
 * the total misses the budget, the triplets with the largest estimates are rerun one count
 * higher, up to opts->slices), and the digit-plane products actually run, sum over triplets of
 * S (S + 1) / 2 per run (any may be NULL). */
ccsdt_status ccsdt_learned_stats(const ccsdt_handle* h, double* mean_slices, long* fallbacks, double* products);

void        ccsdt_destroy(ccsdt_handle* h);
const char* ccsdt_last_error(const ccsdt_handle* h);
const char* ccsdt_status_string(ccsdt_status s);

#ifdef __cplusplus
}
#endif
#endif /* CCSDT_GB300_H */
