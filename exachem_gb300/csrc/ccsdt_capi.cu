// C ABI of the GB300 closed-shell (T) library: handle, upload, energy.
//
// Replaces the per-task orchestration of ExaChem's fused driver
// (exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:91-546 and ccsd_t_all_fused.hpp:77-286):
// instead of gathering spin-orbital blocks on the host and copying them per task, every
// input stays resident in HBM and each occupied triplet i <= j <= k is one unit of work.
#include <cuda_runtime.h>

#include <atomic>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"
#include "fused_fp64.cuh"

using namespace ccsdt;

namespace {

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e__ = (call);                                                                      \
    if(e__ != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
  } while(0)

// the same inside ccsdt_handle methods
#define CK_H(call)                                                                                 \
  do {                                                                                             \
    cudaError_t e__ = (call);                                                                      \
    if(e__ != cudaSuccess) return fail(CCSDT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
  } while(0)

int multiplicity(int i, int j, int k) {
  if(i == j && j == k) return 1;
  if(i == j || j == k || i == k) return 3;
  return 6;
}

} // namespace

ccsdt_status ccsdt_handle::fail(ccsdt_status s, const std::string& msg) {
  err = msg;
  return s;
}

namespace {
std::atomic<long> g_alloc_countdown{0}; // > 0: the call that brings it to 0 fails
std::atomic<long> g_alloc_attempts{0};
} // namespace

cudaError_t ccsdt::dev_malloc(void** p, size_t bytes) {
  g_alloc_attempts.fetch_add(1);
  if(g_alloc_countdown.load() > 0 && g_alloc_countdown.fetch_sub(1) == 1) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  const cudaError_t e = cudaMalloc(p, bytes);
  if(e != cudaSuccess) *p = nullptr;
  return e;
}

extern "C" ccsdt_status ccsdt_debug_fail_alloc(long nth, long* attempts) {
  if(nth < 0) return CCSDT_E_INVALID;
  if(attempts) *attempts = g_alloc_attempts.exchange(0);
  g_alloc_countdown.store(nth);
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::alloc(double** p, size_t n) {
  if(n == 0) n = 1;
  cudaError_t e = ccsdt::dev_malloc((void**) p, n * sizeof(double));
  if(e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(CCSDT_E_OOM, std::string("cudaMalloc of ") + std::to_string(n * sizeof(double)) +
                               " bytes failed: " + cudaGetErrorString(e));
  }
  owned.push_back(*p);
  return CCSDT_OK;
}

ccsdt_handle::~ccsdt_handle() {
  cudaSetDevice(device);
  for(void* p: owned) cudaFree(p);
  for(void* p: owned_bytes) cudaFree(p);
  for(void* p: slice_bufs) cudaFree(p);
  for(void* p: {(void*) bt_F, (void*) bt_part, (void*) bt_order, (void*) bt_order_partial, (void*) bt_ctrl, (void*) bt_tri,
                (void*) chol_ov, (void*) chol_vv, (void*) d_slab_of, chol_planes})
    if(p) cudaFree(p);
  if(ev0) cudaEventDestroy(ev0);
  if(ev1) cudaEventDestroy(ev1);
  for(auto& e: prof_ev)
    if(e) cudaEventDestroy(e);
  for(auto& e: tev)
    if(e) cudaEventDestroy(e);
  if(blk_stage) cudaFree(blk_stage);
  if(blk_meta) cudaFree(blk_meta);
  if(own_stream) cudaStreamDestroy(own_stream);
}

// Device arrays of the inputs (allocated once per handle).
ccsdt_status ccsdt_handle::ensure_inputs(long long nslab) {
  const size_t    o = this->o, v = this->v;
  const size_t    n_t2 = o * o * v * v, n_ooov = o * o * o * v;
  const long long want = nslab < 0 ? (long long) o : nslab;
  uploaded    = false;
  ovvv_direct = nslab >= 0;
  if(!ovvv_direct)
    for(double** p: {&chol_ov, &chol_vv}) // a previous direct-mode upload's vectors
      if(*p) {
        cudaFree(*p);
        *p = nullptr;
      }
  if(ovvv && ovvv_nslab != want) { // the other mode's ovvv: a different number of slabs
    cudaFree(ovvv);
    owned.erase(std::remove(owned.begin(), owned.end(), ovvv), owned.end());
    ovvv = nullptr;
  }
  // allocate each array still missing (a call that failed part-way may have left some)
  auto need = [&](double** p, size_t n) { return *p ? CCSDT_OK : alloc(p, n); };
  ccsdt_status s;
  if((s = need(&eo, o)) || (s = need(&ev, v)) || (s = need(&t1, o * v)) || (s = need(&t2, n_t2)) ||
     (s = need(&oovv, n_t2)) || (s = need(&ooov, n_ooov)) || (s = need(&ovvv, (size_t) want * v * v * v)) ||
     (s = need(&t2h, n_t2)) || (s = need(&ooovh, n_ooov)))
    return s;
  ovvv_nslab = want;
  if(d_count) return CCSDT_OK;
  if(ccsdt::dev_malloc((void**) &d_count, sizeof(unsigned long long)) != cudaSuccess) {
    d_count = nullptr;
    cudaGetLastError();
    return fail(CCSDT_E_OOM, "cudaMalloc of the error counter failed");
  }
  owned_bytes.push_back(d_count);
  return CCSDT_OK;
}

// After the inputs are in place: finiteness of every input, the kappa-contiguous copies for the
// l-sum contractions, and the handle marked ready (digit planes of earlier inputs dropped).
ccsdt_status ccsdt_handle::finish_inputs(const char* who) {
  const size_t o = this->o, v = this->v;
  struct {
    const double* p;
    size_t        n;
  } in[] = {{eo, o}, {ev, v}, {t1, o * v}, {t2, o * o * v * v}, {oovv, o * o * v * v}, {ooov, o * o * o * v},
            // the direct mode forms ovvv later from the vectors, which are checked instead
            {ovvv_direct ? chol_ov : ovvv, ovvv_direct ? o * v * (size_t) n_chol : o * v * v * v},
            {ovvv_direct ? chol_vv : nullptr, ovvv_direct ? v * v * (size_t) n_chol : 0}};
  CK_H(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream));
  for(auto& c: in) {
    if(!c.p) continue;
    nonfinite_count_kernel<<<1024, 256, 0, stream>>>(c.p, (long long) c.n, d_count);
    CK_H(cudaGetLastError());
  }
  transpose_mid_kernel<<<2048, 256, 0, stream>>>(t2, t2h, (int) o, (int) o, (long long) (v * v));
  CK_H(cudaGetLastError());
  transpose_mid_kernel<<<1024, 256, 0, stream>>>(ooov, ooovh, (int) o, (int) o, (long long) (o * v));
  CK_H(cudaGetLastError());
  unsigned long long bad = 0;
  CK_H(cudaMemcpyAsync(&bad, d_count, sizeof(bad), cudaMemcpyDeviceToHost, stream));
  CK_H(cudaStreamSynchronize(stream));
  uploaded = false;
  if(bad) return fail(CCSDT_E_NONFINITE, std::string(who) + ": " + std::to_string(bad) + " non-finite input values");
  uploaded     = true;
  slices_ready = 0;
  slabs.reset(o, ovvv_direct ? (int) ovvv_nslab : 0);
  slab_sliced.assign(ovvv_direct ? ovvv_nslab : 0, 0);
  slab_exact.assign(ovvv_direct ? ovvv_nslab : 0, 0);
  slab_forms = 0;
  if(chol_planes) { // digit planes of earlier vectors
    cudaFree(chol_planes);
    chol_planes = nullptr;
  }
  return CCSDT_OK;
}

extern "C" {

const char* ccsdt_status_string(ccsdt_status s) {
  switch(s) {
    case CCSDT_OK: return "ok";
    case CCSDT_E_INVALID: return "invalid argument";
    case CCSDT_E_BAD_LAYOUT: return "bad tile layout";
    case CCSDT_E_OOM: return "out of memory";
    case CCSDT_E_NONFINITE: return "non-finite value";
    case CCSDT_E_TIMEOUT: return "device wait timed out";
    case CCSDT_E_CUDA: return "CUDA error";
    case CCSDT_E_STATE: return "call out of order";
  }
  return "unknown status";
}

const char* ccsdt_last_error(const ccsdt_handle* h) { return h ? h->err.c_str() : "null handle"; }

long ccsdt_last_launch_count(const ccsdt_handle* h) { return h ? h->launches : -1; }

ccsdt_status ccsdt_create(ccsdt_handle** out, const ccsdt_layout* L, int device) {
  if(!out || !L) return CCSDT_E_INVALID;
  *out = nullptr;
  if(L->o <= 0 || L->v <= 0 || L->n_occ_tiles <= 0 || L->n_vir_tiles <= 0 || !L->occ_tiles ||
     !L->vir_tiles)
    return CCSDT_E_INVALID;
  long so = 0, sv = 0;
  for(int t = 0; t < L->n_occ_tiles; t++) {
    if(L->occ_tiles[t] <= 0) return CCSDT_E_BAD_LAYOUT;
    so += L->occ_tiles[t];
  }
  for(int t = 0; t < L->n_vir_tiles; t++) {
    if(L->vir_tiles[t] <= 0) return CCSDT_E_BAD_LAYOUT;
    sv += L->vir_tiles[t];
  }
  if(so != L->o || sv != L->v) return CCSDT_E_BAD_LAYOUT;
  int ndev = 0;
  if(device == -1 && cudaGetDevice(&device) != cudaSuccess) device = -2; // the caller's current device
  if(cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return CCSDT_E_CUDA;
  }
  ccsdt_handle* h = new ccsdt_handle();
  h->device       = device;
  h->o            = L->o;
  h->v            = L->v;
  h->occ_tiles.assign(L->occ_tiles, L->occ_tiles + L->n_occ_tiles);
  h->vir_tiles.assign(L->vir_tiles, L->vir_tiles + L->n_vir_tiles);
  if(cudaSetDevice(device) != cudaSuccess ||
     cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
     cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return CCSDT_E_CUDA;
  }
  for(auto& e: h->prof_ev)
    if(cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      delete h;
      return CCSDT_E_CUDA;
    }
  h->stream = h->own_stream;
  *out      = h;
  return CCSDT_OK;
}

ccsdt_status ccsdt_set_stream(ccsdt_handle* h, void* stream) {
  if(!h) return CCSDT_E_INVALID;
  h->stream = stream ? (cudaStream_t) stream : h->own_stream;
  return CCSDT_OK;
}

ccsdt_status ccsdt_set_phase_timing(ccsdt_handle* h, int on) {
  if(!h) return CCSDT_E_INVALID;
  h->phase_timing = on != 0;
  for(double& m: h->phase_ms) m = 0;
  h->phase_batches = h->phase_triplets = 0;
  return CCSDT_OK;
}

ccsdt_status ccsdt_phase_times(const ccsdt_handle* h, double* ms3, long* batches, long* triplets) {
  if(!h || !ms3) return CCSDT_E_INVALID;
  for(int q = 0; q < 3; q++) ms3[q] = h->phase_ms[q];
  if(batches) *batches = h->phase_batches;
  if(triplets) *triplets = h->phase_triplets;
  return CCSDT_OK;
}

void ccsdt_destroy(ccsdt_handle* h) { delete h; }

ccsdt_status ccsdt_upload(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                          const double* t1, const double* t2, const double* oovv,
                          const double* ooov, const double* ovvv, int on_device) {
  if(!h) return CCSDT_E_INVALID;
  if(!eps_occ || !eps_vir || !t1 || !t2 || !oovv || !ooov || !ovvv)
    return h->fail(CCSDT_E_INVALID, "ccsdt_upload: null input pointer");
  CK(cudaSetDevice(h->device));
  ccsdt_status s;
  if((s = h->ensure_inputs())) return s;
  h->blocks_open = false;
  const size_t o = h->o, v = h->v;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  struct {
    double*       dst;
    const double* src;
    size_t        n;
  } cp[] = {{h->eo, eps_occ, o},          {h->ev, eps_vir, v},          {h->t1, t1, o * v},
            {h->t2, t2, o * o * v * v},   {h->oovv, oovv, o * o * v * v}, {h->ooov, ooov, o * o * o * v},
            {h->ovvv, ovvv, o * v * v * v}};
  for(auto& c: cp) CK(cudaMemcpyAsync(c.dst, c.src, c.n * sizeof(double), kind, h->stream));
  return h->finish_inputs("ccsdt_upload");
}

} // extern "C"

// ------------------------------------------------------------------------------------------
// FP64 path: per triplet, hole GEMMs (initialise P12/P34/P56), particle GEMMs (accumulate),
// energy, partial reduction.

ccsdt_status ccsdt_handle::ensure_scratch() {
  const size_t v = this->v;
  ccsdt_status s;
  // each buffer on its own: a call that failed part-way may have left some of them
  auto need = [&](double** p, size_t n) { return *p ? CCSDT_OK : alloc(p, n); };
  if((s = need(&P12, v * v * v)) || (s = need(&P34, v * v * v)) || (s = need(&P56, v * v * v)) ||
     (s = need(&part, 4 * (size_t) kEnergyBlocks)) || (s = need(&res, 2)))
    return s;
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::ensure_triplet_slots(long n) {
  if(etrip_cap >= n) return CCSDT_OK;
  double*      p = nullptr;
  ccsdt_status s = alloc(&p, 2 * (size_t) n);
  if(s) return s;
  etrip     = p;
  etrip_cap = n;
  return CCSDT_OK;
}

// The sorted 8-wide virtual block triples (work units of the fused FP64 kernel), built once.
ccsdt_status ccsdt_handle::ensure_fused_tiles() {
  if(fx_tiles) return CCSDT_OK;
  const int        nb = (v + ET_B - 1) / ET_B;
  std::vector<int> host;
  for(int X = 0; X < nb; X++)
    for(int Y = X; Y < nb; Y++)
      for(int Z = Y; Z < nb; Z++) host.insert(host.end(), {X, Y, Z});
  int* d = nullptr;
  if(ccsdt::dev_malloc((void**) &d, host.size() * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return fail(CCSDT_E_OOM, "fused FP64 work units");
  }
  owned_bytes.push_back(d);
  if(cudaMemcpy(d, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(CCSDT_E_CUDA, "fused FP64 work-unit upload");
  fx_tiles  = d;
  fx_ntiles = (int) (host.size() / 3);
  int sm = 0, per = 0;
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, t3_fused_fp64_kernel, FX_THREADS, 0);
  cudaGetLastError();
  fx_grid = std::max(1, std::min(kEnergyBlocks, std::max(1, per) * std::max(1, sm)));
  return CCSDT_OK;
}

// One triplet on the fused FP64 kernel: contractions, the triples block kept on chip, energy.
ccsdt_status ccsdt_handle::run_triplet_fp64_fused(int i, int j, int k, double* eout) {
  ccsdt_status s;
  if((s = ensure_fused_tiles())) return s;
  FusedArgs fa{t2,        t2h, ovvv_slab(i), ovvv_slab(j), ovvv_slab(k), ooovh, oovv, t1, eo, ev, (const int3*) fx_tiles,
               fx_ntiles, o,   v,            i,            j,            k,     part};
  const int G = std::min(fx_ntiles, fx_grid);
  if(profiling) {
    cudaEventRecord(prof_ev[0], stream);
    cudaEventRecord(prof_ev[1], stream); // contractions and energy are one launch
  }
  t3_fused_fp64_kernel<<<G, FX_THREADS, 0, stream>>>(fa);
  if(profiling) {
    cudaEventRecord(prof_ev[2], stream);
    cudaEventRecord(prof_ev[3], stream);
  }
  reduce_parts_kernel<<<1, E_THREADS, 0, stream>>>(part, G, multiplicity(i, j, k) / 9.0, eout);
  if(profiling) cudaEventRecord(prof_ev[4], stream);
  launches += 2;
  const cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("fused FP64 launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::run_triplet_fp64(int i, int j, int k, double* eout) {
  // the fused kernel unless the partial arrays themselves are wanted (W debugging aid, the
  // float-float energy test) or a test asks for the two-stage path
  if(!fp64_unfused && !fp64_ff_energy) return run_triplet_fp64_fused(i, j, k, eout);
  const long long o = this->o, v = this->v, v2 = v * v, v3 = v2 * v;
  // ---- l-sum (hole) contractions: C[(pair)][single] = -sum_l t(pair, l) (..l|..)
  GemmBatch hb{};
  auto      t2h_of = [&](int x) { return t2h + (long long) x * v2 * o; };                // [(a,b)][l]
  auto      ooh_of = [&](int y, int z) { return ooovh + ((long long) y * o + z) * v * o; }; // [c][l]
  const RowMap pair_nat = plain_rows(o), pair_swp = swapped_pair_rows((int) v, o), single = plain_rows(o);
  // P12[(a,c)][b]: -t_il^{ac} (kl|jb) - t_kl^{ca} (il|jb)
  hb.job[0] = GemmJob{{GemmTerm{t2h_of(i), pair_nat, ooh_of(k, j), single, (int) o, -1.0},
                       GemmTerm{t2h_of(k), pair_swp, ooh_of(i, j), single, (int) o, -1.0}},
                      2, P12, v2, v, 0.0};
  // P34[(b,a)][c]: -t_il^{ab} (jl|kc) - t_jl^{ba} (il|kc)
  hb.job[1] = GemmJob{{GemmTerm{t2h_of(i), pair_swp, ooh_of(j, k), single, (int) o, -1.0},
                       GemmTerm{t2h_of(j), pair_nat, ooh_of(i, k), single, (int) o, -1.0}},
                      2, P34, v2, v, 0.0};
  // P56[(c,b)][a]: -t_jl^{bc} (kl|ia) - t_kl^{cb} (jl|ia)
  hb.job[2] = GemmJob{{GemmTerm{t2h_of(j), pair_swp, ooh_of(k, i), single, (int) o, -1.0},
                       GemmTerm{t2h_of(k), pair_nat, ooh_of(j, i), single, (int) o, -1.0}},
                      2, P56, v2, v, 0.0};
  if(profiling) cudaEventRecord(prof_ev[0], stream);
  {
    long long tiles = ((v2 + D_BM - 1) / D_BM) * ((v + D_BN - 1) / D_BN);
    if(tiles > 0x7fffffffLL) return fail(CCSDT_E_INVALID, "too many GEMM tiles");
    dmma_gemm_kernel<<<dim3((unsigned) tiles, 1, 3), D_THREADS, 0, stream>>>(hb);
    launches++;
  }
  // ---- d-sum (particle) contractions: C[single][(pair)] += sum_d t(single, d) (pair|d)
  GemmBatch pb{};
  auto      t2_of   = [&](int x, int y) { return t2 + ((long long) x * o + y) * v2; }; // [a][d]
  auto      ovvv_of = [&](int z) { return ovvv_slab(z); };                              // [(g,b)][d]
  const RowMap arow = plain_rows(v), bnat = plain_rows(v), bswp = swapped_pair_rows((int) v, v);
  // P12[a][(c,b)] += t_ij^{ad} (kc|bd) + t_ik^{ad} (jb|cd)
  pb.job[0] = GemmJob{{GemmTerm{t2_of(i, j), arow, ovvv_of(k), bnat, (int) v, 1.0},
                       GemmTerm{t2_of(i, k), arow, ovvv_of(j), bswp, (int) v, 1.0}},
                      2, P12, v, v2, 1.0};
  // P34[b][(a,c)] += t_ji^{bd} (kc|ad) + t_jk^{bd} (ia|cd)
  pb.job[1] = GemmJob{{GemmTerm{t2_of(j, i), arow, ovvv_of(k), bswp, (int) v, 1.0},
                       GemmTerm{t2_of(j, k), arow, ovvv_of(i), bnat, (int) v, 1.0}},
                      2, P34, v, v2, 1.0};
  // P56[c][(b,a)] += t_ki^{cd} (jb|ad) + t_kj^{cd} (ia|bd)
  pb.job[2] = GemmJob{{GemmTerm{t2_of(k, i), arow, ovvv_of(j), bnat, (int) v, 1.0},
                       GemmTerm{t2_of(k, j), arow, ovvv_of(i), bswp, (int) v, 1.0}},
                      2, P56, v, v2, 1.0};
  if(profiling) cudaEventRecord(prof_ev[1], stream);
  {
    long long tiles = ((v + D_BM - 1) / D_BM) * ((v2 + D_BN - 1) / D_BN);
    dmma_gemm_kernel<<<dim3((unsigned) tiles, 1, 3), D_THREADS, 0, stream>>>(pb);
    launches++;
  }
  if(profiling) cudaEventRecord(prof_ev[2], stream);
  if(fp64_ff_energy) { // testing: the same P arrays through the split path's float-float energy
    if(!F12 || !F34 || !F56) return fail(CCSDT_E_STATE, "float-float energy buffers missing");
    if(p_storage == 2) { // ... or its FP32 energy, from the arrays rounded to FP32
      to_f32_kernel<<<2048, 256, 0, stream>>>(P12, reinterpret_cast<float*>(F12), v3);
      to_f32_kernel<<<2048, 256, 0, stream>>>(P34, reinterpret_cast<float*>(F34), v3);
      to_f32_kernel<<<2048, 256, 0, stream>>>(P56, reinterpret_cast<float*>(F56), v3);
    } else {
      to_ff_kernel<<<2048, 256, 0, stream>>>(P12, F12, v3);
      to_ff_kernel<<<2048, 256, 0, stream>>>(P34, F34, v3);
      to_ff_kernel<<<2048, 256, 0, stream>>>(P56, F56, v3);
    }
    launches += 3;
    return launch_energy_tiled(i, j, k, eout, p_storage == 2);
  }
  EnergyArgs ea{P12, P34, P56, oovv, t1, eo, ev, (int) o, (int) v, i, j, k, part};
  energy_fp64_kernel<<<kEnergyBlocks, E_THREADS, 0, stream>>>(ea);
  if(profiling) cudaEventRecord(prof_ev[3], stream);
  reduce_parts_kernel<<<1, E_THREADS, 0, stream>>>(part, kEnergyBlocks, multiplicity(i, j, k) / 9.0, eout);
  if(profiling) cudaEventRecord(prof_ev[4], stream);
  launches += 2;
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

static bool valid_opts(const ccsdt_opts* o) {
  return o && (o->mode == CCSDT_MODE_FP64 || o->mode == CCSDT_MODE_OZAKI || o->mode == CCSDT_MODE_LEARNED) &&
         o->p_storage >= 0 && o->p_storage <= 3;
}

// opts->autotune: the slice counts this call can use on the persistent tcgen05 path, each tuned
// once per handle (before the caller's timed work)
static ccsdt_status autotune_for(ccsdt_handle* h, const ccsdt_opts* opts) {
  if(!opts->autotune || opts->mode == CCSDT_MODE_FP64 || opts->slice_kind != 0 || opts->test_kernel != 0)
    return CCSDT_OK;
  const int lo = opts->mode == CCSDT_MODE_LEARNED ? 1 : opts->slices, hi = std::min(opts->slices, 8);
  for(int S = std::max(lo, 1); S <= hi; S++)
    if(!h->pz_tuned[S]) {
      ccsdt_status s = h->autotune(S, nullptr, nullptr, nullptr);
      if(s) return s;
    }
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::run_list(const ccsdt_opts* opts, long n, const int* tri_host) {
  ccsdt_status s;
  if((s = ensure_scratch()) || (s = ensure_triplet_slots(n))) return s;
  launches  = 0;
  p_storage = opts->p_storage;
  if(opts->mode != CCSDT_MODE_FP64) return run_split(opts, n, tri_host);
  fp64_unfused = opts->test_kernel == 5 || w_debug; // testing: the two-stage FP64 path
  return run_fp64_list(n, tri_host);
}

// The FP64 path over a triplet list; results at etrip[2 t].  In the Cholesky-direct mode the
// triplets run by blocks of occupied indices, each after its three (ia|bc) slabs are resident.
ccsdt_status ccsdt_handle::run_fp64_list(long n, const int* tri_host) {
  ccsdt_status            s;
  const std::vector<long> ord =
    ovvv_direct ? ccsdt::slab_order(tri_host, n, (int) ovvv_nslab) : std::vector<long>();
  for(long u = 0; u < n; u++) {
    const long t = ovvv_direct ? ord[u] : u;
    const int  i = tri_host[3 * t], j = tri_host[3 * t + 1], k = tri_host[3 * t + 2];
    if(i == k) {
      // i = j = k: W is symmetric in (a, b, c), so Z Y vanishes identically
      cudaError_t e = cudaMemsetAsync(etrip + 2 * t, 0, 2 * sizeof(double), stream);
      if(e != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(e));
      continue;
    }
    if((s = ensure_ovvv(&tri_host[3 * t], 3, false)) || (s = run_triplet_fp64(i, j, k, etrip + 2 * t))) return s;
  }
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_triplet_energies(ccsdt_handle* h, const ccsdt_opts* opts, long n,
                                               const int* tri, double* e_bracket, double* e_paren) {
  if(!h) return CCSDT_E_INVALID;
  if(!valid_opts(opts) || n < 0 || (n > 0 && (!tri || !e_bracket || !e_paren)))
    return h->fail(CCSDT_E_INVALID, "ccsdt_triplet_energies: bad arguments");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_triplet_energies before a successful ccsdt_upload");
  for(long t = 0; t < n; t++) {
    const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    if(!(0 <= i && i <= j && j <= k && k < h->o))
      return h->fail(CCSDT_E_INVALID, "triplet " + std::to_string(t) + " is not 0 <= i <= j <= k < o");
  }
  CK(cudaSetDevice(h->device));
  ccsdt_status s = autotune_for(h, opts);
  if(s) return s;
  s = h->run_list(opts, n, tri);
  if(s) return s;
  std::vector<double> buf(2 * (size_t) n);
  if(n) CK(cudaMemcpyAsync(buf.data(), h->etrip, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if(opts->mode != CCSDT_MODE_FP64 && (s = h->check_device_error())) return s;
  for(long t = 0; t < n; t++) {
    e_bracket[t] = buf[2 * t];
    e_paren[t]   = buf[2 * t + 1];
  }
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_shard_triplets(int o, int shard_index, int shard_count, long* n, int* tri) {
  if(o <= 0 || !n || shard_count < 1 || shard_index < 0 || shard_index >= shard_count) return CCSDT_E_INVALID;
  long tcount = 0, m = 0;
  for(int i = 0; i < o; i++)
    for(int j = i; j < o; j++)
      for(int k = j; k < o; k++, tcount++) {
        if(tcount % shard_count != shard_index) continue;
        if(tri) {
          tri[3 * m]     = i;
          tri[3 * m + 1] = j;
          tri[3 * m + 2] = k;
        }
        m++;
      }
  *n = m;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_energy(ccsdt_handle* h, const ccsdt_opts* opts, ccsdt_result* out) {
  if(!h) return CCSDT_E_INVALID;
  if(!valid_opts(opts) || !out) return h->fail(CCSDT_E_INVALID, "ccsdt_energy: bad arguments");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_energy before a successful ccsdt_upload");
  CK(cudaSetDevice(h->device));
  const int        o = h->o;
  const int        nsh = opts->shard_count > 1 ? opts->shard_count : 1;
  if(opts->shard_index < 0 || opts->shard_index >= nsh)
    return h->fail(CCSDT_E_INVALID, "ccsdt_energy: shard_index outside [0, shard_count)");
  long n = 0;
  ccsdt_shard_triplets(o, opts->shard_index, nsh, &n, nullptr);
  std::vector<int> tri(3 * (size_t) n);
  ccsdt_shard_triplets(o, opts->shard_index, nsh, &n, tri.data());
  ccsdt_status s = autotune_for(h, opts);
  if(s) return s;
  CK(cudaEventRecord(h->ev0, h->stream));
  s = h->run_list(opts, n, tri.data());
  if(s) return s;
  reduce_triplets_kernel<<<1, 32, 0, h->stream>>>(h->etrip, n, h->res);
  h->launches++;
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev1, h->stream));
  double r[2];
  CK(cudaMemcpyAsync(r, h->res, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if(opts->mode != CCSDT_MODE_FP64 && (s = h->check_device_error())) return s;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  std::memset(out, 0, sizeof(*out));
  out->e_bracket_T    = r[0];
  out->e_paren_T      = r[1];
  out->abs_err_bound  = h->last_err_bound;
  out->seconds        = ms * 1e-3;
  const double vv     = h->v;
  long nzero = 0; // i = j = k triplets are skipped (they contribute exactly zero)
  for(long t = 0; t < n; t++) nzero += tri[3 * t] == tri[3 * t + 2];
  out->flops_executed = (double) (n - nzero) * 12.0 * vv * vv * vv * (vv + o);
  out->n_triplets     = n;
  ccsdt_layout L{h->o, h->v, (int) h->occ_tiles.size(), h->occ_tiles.data(), (int) h->vir_tiles.size(),
                 h->vir_tiles.data()};
  double ops = 0;
  long   nt  = 0;
  if(ccsdt_reference_op_count(&L, &ops, &nt) == CCSDT_OK) {
    out->flops_ref_equiv = ops;
    out->n_tasks_ref     = nt;
  }
  if(!std::isfinite(r[0]) || !std::isfinite(r[1])) return h->fail(CCSDT_E_NONFINITE, "non-finite energy");
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_profile_triplet(ccsdt_handle* h, const ccsdt_opts* opts, int i, int j,
                                              int k, double* out_ms) {
  if(!h) return CCSDT_E_INVALID;
  if(!valid_opts(opts) || !out_ms || !(0 <= i && i <= j && j <= k && k < h->o) || i == k)
    return h->fail(CCSDT_E_INVALID, "ccsdt_profile_triplet: bad arguments (needs i <= j <= k, i < k)");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_profile_triplet before ccsdt_upload");
  CK(cudaSetDevice(h->device));
  const int tri[3] = {i, j, k};
  h->profiling     = true;
  ccsdt_status s   = h->run_list(opts, 1, tri);
  h->profiling     = false;
  if(s) return s;
  CK(cudaStreamSynchronize(h->stream));
  for(int q = 0; q < 4; q++) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->prof_ev[q], h->prof_ev[q + 1]));
    out_ms[q] = ms;
  }
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_debug_triplet_w(ccsdt_handle* h, const ccsdt_opts* opts, int i, int j, int k,
                                              double* w_host) {
  if(!h) return CCSDT_E_INVALID;
  if(!valid_opts(opts) || !w_host || !(0 <= i && i <= j && j <= k && k < h->o) || i == k)
    return h->fail(CCSDT_E_INVALID, "ccsdt_debug_triplet_w: bad arguments (needs i <= j <= k, i < k)");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_debug_triplet_w before ccsdt_upload");
  CK(cudaSetDevice(h->device));
  const int    tri[3] = {i, j, k};
  h->w_debug          = true; // the FP64 partial arrays must be written to HBM
  ccsdt_status s      = h->run_list(opts, 1, tri);
  h->w_debug          = false;
  if(s) return s;
  CK(cudaStreamSynchronize(h->stream));
  if(opts->mode != CCSDT_MODE_FP64 && (s = h->check_device_error())) return s;
  const size_t        v = h->v, n = v * v * v;
  std::vector<double> a(n), b(n), c(n);
  if(opts->mode == CCSDT_MODE_FP64) {
    CK(cudaMemcpy(a.data(), h->P12, n * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b.data(), h->P34, n * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(c.data(), h->P56, n * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    // the persistent path keeps slot 0's P12, P34, P56 consecutively in the batch scratch, as
    // float-float or FP32 elements
    std::vector<float2> f(n);
    const float2*       src[3] = {h->F12, h->F34, h->F56};
    const bool          f32    = h->last_batched && h->last_p_f32, f64 = h->last_batched && h->last_p_f64;
    if(h->last_batched)
      for(int q = 0; q < 3; q++)
        src[q] = f32 ? reinterpret_cast<const float2*>(reinterpret_cast<const float*>(h->bt_F) + q * n) : h->bt_F + q * n;
    for(int q = 0; q < 3; q++) {
      CK(cudaMemcpy(f.data(), src[q], n * (f32 ? sizeof(float) : sizeof(float2)), cudaMemcpyDeviceToHost));
      std::vector<double>& d = q == 0 ? a : q == 1 ? b : c;
      const float*         g = reinterpret_cast<const float*>(f.data());
      if(f64)
        std::memcpy(d.data(), f.data(), n * sizeof(double)); // FP64 elements, 8 bytes like float2
      else
        for(size_t e = 0; e < n; e++) d[e] = f32 ? (double) g[e] : (double) f[e].x + (double) f[e].y;
    }
  }
  // W_xyz = P12[x][z][y] + P34[y][x][z] + P56[z][y][x]
  for(size_t x = 0; x < v; x++)
    for(size_t y = 0; y < v; y++)
      for(size_t z = 0; z < v; z++)
        w_host[(x * v + y) * v + z] = a[(x * v + z) * v + y] + b[(y * v + x) * v + z] + c[(z * v + y) * v + x];
  return CCSDT_OK;
}
