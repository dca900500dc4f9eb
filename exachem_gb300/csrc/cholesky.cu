// Closed-shell integral blocks built on the device from Cholesky vectors.
//
// Restates exachem/cholesky/v2tensors.cpp:66-88 (setupV2Tensors: v2ijab, v2ijka, v2iabc from
// cholVpr) for the blocks the closed-shell (T) reads.  With spatial vectors L[p][q][Q] (symmetric
// in p, q: the alpha-alpha block of cholVpr) the alpha / alpha-beta blocks the gather takes lose
// their exchange terms by spin, and
//   oovv[i][j][a][b] = (ia|jb) = sum_Q L[i][a][Q] L[j][b][Q]      v2ijab(i_a, j_b, a_a, b_b)
//   ooov[i][j][k][a] = (ij|ka) = sum_Q L[i][j][Q] L[k][a][Q]      v2ijka(i_a, k_b, j_a, a_b)
//   ovvv[i][a][b][c] = (ia|bc) = sum_Q L[i][a][Q] L[b][c][Q]      v2iabc(i_a, b_b, a_a, c_b)
// Each block is one FP64 DMMA GEMM C = A B^T with Q contiguous in both operands.  ovvv and ooov
// land in their row-major layouts directly; (ia|jb) comes out as [(i,a)][(j,b)], is formed in the
// array that later holds the kappa-contiguous copy of t2 (free until the inputs are finished) and
// permuted into oovv.  The 60 GB ovvv of o=60 v=500 then never crosses PCIe: the caller hands
// over o v nQ + v^2 nQ + o^2 nQ doubles instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"
#include "ozaki.cuh"

using namespace ccsdt;

namespace {

// dst[i][j][a][b] = src[i][a][j][b]
__global__ void __launch_bounds__(256) swap_ia_jb_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                                        int o, int v) {
  const long long v2 = (long long) v * v, total = (long long) o * o * v2;
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < total;
      e += (long long) gridDim.x * blockDim.x) {
    const long long i = e / (o * v2), r = e % (o * v2), j = r / v2, ab = r % v2, a = ab / v, b = ab % v;
    dst[e] = src[((i * v + a) * o + j) * v + b];
  }
}

// C[M][N] = sum_Q A[m][Q] B[n][Q] (row-major, Q contiguous) on the handle's stream
cudaError_t gemm_abt(const double* A, const double* B, double* C, long long M, long long N, int K, cudaStream_t st) {
  GemmBatch g{};
  g.job[0].t[0] = GemmTerm{A, plain_rows(K), B, plain_rows(K), K, 1.0};
  g.job[0].nterms = 1;
  g.job[0].C      = C;
  g.job[0].M      = M;
  g.job[0].N      = N;
  g.job[0].beta   = 0.0;
  const long long tiles = ((M + D_BM - 1) / D_BM) * ((N + D_BN - 1) / D_BN);
  if(tiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
  dmma_gemm_kernel<<<dim3((unsigned) tiles, 1, 1), D_THREADS, 0, st>>>(g);
  return cudaGetLastError();
}

} // namespace

// nslab < 0: every block built whole; nslab >= 3: the Cholesky-direct mode (ovvv a cache of nslab
// slabs formed later by ensure_ovvv from persistent copies of L_ov and L_vv)
static ccsdt_status upload_cholesky(ccsdt_handle* h, const char* who, const double* eps_occ, const double* eps_vir,
                                    const double* t1, const double* t2, int n_chol, const double* chol_oo,
                                    const double* chol_ov, const double* chol_vv, int on_device, long long nslab) {
  if(!h) return CCSDT_E_INVALID;
  if(!eps_occ || !eps_vir || !t1 || !t2 || !chol_oo || !chol_ov || !chol_vv)
    return h->fail(CCSDT_E_INVALID, std::string(who) + ": null input pointer");
  if(n_chol <= 0) return h->fail(CCSDT_E_INVALID, std::string(who) + ": n_chol must be positive");
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  const long long o = h->o, v = h->v, nq = n_chol;
  // the direct mode's persistent vectors (dropped by any other upload)
  for(double** p: {&h->chol_ov, &h->chol_vv})
    if(*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  h->n_chol = 0;
  ccsdt_status s;
  if((s = h->ensure_inputs(nslab))) return s;
  h->blocks_open = false;
  h->uploaded    = false;
  if(nslab >= 0) {
    if(ccsdt::dev_malloc((void**) &h->chol_ov, o * v * nq * sizeof(double)) != cudaSuccess ||
       ccsdt::dev_malloc((void**) &h->chol_vv, v * v * nq * sizeof(double)) != cudaSuccess ||
       (!h->d_slab_of && ccsdt::dev_malloc((void**) &h->d_slab_of, o * sizeof(int)) != cudaSuccess)) {
      cudaGetLastError();
      return h->fail(CCSDT_E_OOM, std::string(who) + ": cudaMalloc of the Cholesky vectors failed");
    }
    h->n_chol = n_chol;
  }
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaError_t e = cudaSuccess;
  struct {
    double*       dst;
    const double* src;
    long long     n;
  } cp[] = {{h->eo, eps_occ, o}, {h->ev, eps_vir, v}, {h->t1, t1, o * v}, {h->t2, t2, o * o * v * v}};
  for(auto& c: cp)
    if(e == cudaSuccess) e = cudaMemcpyAsync(c.dst, c.src, c.n * sizeof(double), kind, h->stream);
  // the vectors on the device (copied from the host into one scratch allocation when needed)
  const double *L_oo = chol_oo, *L_ov = chol_ov, *L_vv = chol_vv;
  double*       scratch = nullptr;
  if(e == cudaSuccess && nslab >= 0) { // the direct mode keeps L_ov and L_vv
    e = cudaMemcpyAsync(h->chol_ov, chol_ov, o * v * nq * sizeof(double), kind, h->stream);
    if(e == cudaSuccess) e = cudaMemcpyAsync(h->chol_vv, chol_vv, v * v * nq * sizeof(double), kind, h->stream);
    L_ov = h->chol_ov, L_vv = h->chol_vv;
    if(e == cudaSuccess && !on_device) {
      if(ccsdt::dev_malloc((void**) &scratch, o * o * nq * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return h->fail(CCSDT_E_OOM, std::string(who) + ": cudaMalloc of the occupied-occupied vectors failed");
      }
      e    = cudaMemcpyAsync(scratch, chol_oo, o * o * nq * sizeof(double), cudaMemcpyHostToDevice, h->stream);
      L_oo = scratch;
    }
  } else if(e == cudaSuccess && !on_device) {
    const long long n_oo = o * o * nq, n_ov = o * v * nq, n_vv = v * v * nq;
    if(ccsdt::dev_malloc((void**) &scratch, (n_oo + n_ov + n_vv) * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return h->fail(CCSDT_E_OOM, "ccsdt_upload_cholesky: cudaMalloc of " +
                                     std::to_string((n_oo + n_ov + n_vv) * sizeof(double)) + " bytes for the vectors");
    }
    double* d_oo = scratch;
    double* d_ov = d_oo + n_oo;
    double* d_vv = d_ov + n_ov;
    e = cudaMemcpyAsync(d_oo, chol_oo, n_oo * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if(e == cudaSuccess) e = cudaMemcpyAsync(d_ov, chol_ov, n_ov * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if(e == cudaSuccess) e = cudaMemcpyAsync(d_vv, chol_vv, n_vv * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    L_oo = d_oo, L_ov = d_ov, L_vv = d_vv;
  }
  if(e == cudaSuccess && nslab < 0) e = gemm_abt(L_ov, L_vv, h->ovvv, o * v, v * v, (int) nq, h->stream); // (ia|bc)
  if(e == cudaSuccess) e = gemm_abt(L_oo, L_ov, h->ooov, o * o, o * v, (int) nq, h->stream); // (ij|ka)
  if(e == cudaSuccess) e = gemm_abt(L_ov, L_ov, h->t2h, o * v, o * v, (int) nq, h->stream);  // [(i,a)][(j,b)]
  if(e == cudaSuccess) {
    swap_ia_jb_kernel<<<2048, 256, 0, h->stream>>>(h->t2h, h->oovv, (int) o, (int) v);
    e = cudaGetLastError();
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if(scratch) cudaFree(scratch);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string(who) + ": " + cudaGetErrorString(e));
  return h->finish_inputs(who);
}

extern "C" ccsdt_status ccsdt_upload_cholesky(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                             const double* t1, const double* t2, int n_chol,
                                             const double* chol_oo, const double* chol_ov, const double* chol_vv,
                                             int on_device) {
  return upload_cholesky(h, "ccsdt_upload_cholesky", eps_occ, eps_vir, t1, t2, n_chol, chol_oo, chol_ov, chol_vv,
                         on_device, -1);
}

extern "C" ccsdt_status ccsdt_upload_cholesky_direct(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                                    const double* t1, const double* t2, int n_chol,
                                                    const double* chol_oo, const double* chol_ov,
                                                    const double* chol_vv, int on_device, int max_ovvv_slabs) {
  if(h && (max_ovvv_slabs < 3))
    return h->fail(CCSDT_E_INVALID, "ccsdt_upload_cholesky_direct: max_ovvv_slabs must be at least 3");
  if(h) max_ovvv_slabs = std::min(max_ovvv_slabs, std::max(h->o, 3));
  return upload_cholesky(h, "ccsdt_upload_cholesky_direct", eps_occ, eps_vir, t1, t2, n_chol, chol_oo, chol_ov,
                         chol_vv, on_device, max_ovvv_slabs);
}

namespace {
constexpr int kCholSlices = 6; // digit planes of the vectors for the split-path slab formation

// float-float values widened to FP64 in place (element e: 8 bytes either way)
__global__ void __launch_bounds__(256) ff_to_f64_inplace_kernel(void* p, long long n) {
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long) gridDim.x * blockDim.x) {
    const float2 f                     = reinterpret_cast<const float2*>(p)[e];
    reinterpret_cast<double*>(p)[e] = (double) f.x + (double) f.y;
  }
}
} // namespace

// Forms the missing slabs (index x into slot c: (x a|b c) = sum_Q L[x][a][Q] L[b][c][Q], a GEMM of
// v x v^2 x n_chol), slices them into the digit-plane slots when `planes`, and updates the device
// index -> slot table.  FP64 calls (planes false) form slabs with FP64 DMMA and re-form any
// resident slab that was not; split-path calls (planes true) form them, unless slab_split_build is
// off, as an Ozaki GEMM of kCholSlices BF16 digit planes of the vectors (mma.sync, exact FP32
// level sums, float-float result widened to FP64; relative error ~1e-12 of the slab's scale,
// far below the (T)'s own truncation at the slice counts the split path runs).  Stream-ordered: a
// slot is overwritten only after the kernels launched before on the handle's stream have finished
// reading it.
ccsdt_status ccsdt_handle::ensure_ovvv(const int* need, int n, bool planes) {
  if(!ovvv_direct) return CCSDT_OK;
  std::vector<std::pair<int, int>> todo;
  if(!slabs.require(need, n, todo))
    return fail(CCSDT_E_INVALID, "more distinct occupied indices at once than (ia|bc) slab slots");
  const long long vv = v, v3 = vv * vv * vv, oo = o;
  const bool      split_build = planes && slab_split_build;
  if(!planes) // FP64 calls read exact slabs only
    for(int q = 0; q < n; q++) {
      const int c = slabs.slot(need[q]);
      if(!slab_exact[c] && std::find_if(todo.begin(), todo.end(), [&](const std::pair<int, int>& t) {
                             return t.second == c;
                           }) == todo.end())
        todo.emplace_back(need[q], c);
    }
  if(split_build && !todo.empty() && !chol_planes) { // digit planes of L_ov and L_vv, once per upload
    chol_kq               = (n_chol + 31) / 32 * 32;
    const long long rows  = oo * vv + vv * vv;
    const size_t    bytes = (size_t) kCholSlices * rows * chol_kq * 2 + (size_t) rows * 4;
    if(ccsdt::dev_malloc(&chol_planes, bytes) != cudaSuccess) {
      chol_planes = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "(ia|bc) slab formation: digit planes of the Cholesky vectors");
    }
    auto*     pl   = static_cast<__nv_bfloat16*>(chol_planes);
    int*      exps = reinterpret_cast<int*>(static_cast<char*>(chol_planes) + (size_t) kCholSlices * rows * chol_kq * 2);
    oz_slice_rows_kernel<__nv_bfloat16><<<4096, 256, 0, stream>>>(chol_ov, oo * vv, n_chol, (int) chol_kq, kCholSlices,
                                                                   pl, rows * chol_kq, exps, n_chol);
    oz_slice_rows_kernel<__nv_bfloat16><<<4096, 256, 0, stream>>>(chol_vv, vv * vv, n_chol, (int) chol_kq, kCholSlices,
                                                                   pl + oo * vv * chol_kq, rows * chol_kq,
                                                                   exps + oo * vv, n_chol);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("Cholesky vector slicing: ") + cudaGetErrorString(e));
    launches += 2;
  }
  for(auto& xc: todo) {
    double*     slot = ovvv + xc.second * v3;
    cudaError_t e    = cudaSuccess;
    if(split_build) {
      const long long rows = oo * vv + vv * vv, plane = rows * chol_kq;
      auto*           pl   = static_cast<const __nv_bfloat16*>(chol_planes);
      OzBatch         b{};
      b.S      = kCholSlices;
      b.job[0] = OzJob{{OzTerm{pl + (long long) xc.first * vv * chol_kq, nullptr, oz_plain(), plane,
                               pl + oo * vv * chol_kq, nullptr, oz_plain(), plane, (int) chol_kq, 1.f}},
                       1, reinterpret_cast<float2*>(slot), vv, vv * vv, 0};
      e = oz_gemm_bf16(b, 1, oz_gemm_tiles(vv, vv * vv), stream);
      if(e == cudaSuccess) {
        ff_to_f64_inplace_kernel<<<4096, 256, 0, stream>>>(slot, v3);
        e = cudaGetLastError();
      }
      launches += 2;
    } else {
      e = gemm_abt(chol_ov + (long long) xc.first * vv * n_chol, chol_vv, slot, vv, vv * vv, n_chol, stream);
      launches++;
    }
    if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("(ia|bc) slab: ") + cudaGetErrorString(e));
    slab_sliced[xc.second] = 0;
    slab_exact[xc.second]  = !split_build;
    slab_forms++;
  }
  if(planes) {
    if(!sl_ovvv || slices_ready <= 0 || slice_variant != 0)
      return fail(CCSDT_E_STATE, "(ia|bc) slab planes asked for before the BF16 slicing");
    for(int q = 0; q < n; q++) {
      const int c = slabs.slot(need[q]);
      if(slab_sliced[c]) continue;
      oz_slice_rows_kernel<__nv_bfloat16><<<2048, 256, 0, stream>>>(
        ovvv + c * v3, vv * vv, v, kp_v, slices_ready, (__nv_bfloat16*) sl_ovvv + (long long) c * vv * vv * kp_v,
        pl_ovvv, ex_ovvv + (long long) c * vv * vv, vv);
      cudaError_t e = cudaGetLastError();
      if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("(ia|bc) slab slicing: ") + cudaGetErrorString(e));
      slab_sliced[c] = 1;
      launches++;
    }
  }
  if(!todo.empty()) { // pageable source: the copy is staged before the call returns
    const std::vector<int>& tab = slabs.slots();
    if(cudaMemcpyAsync(d_slab_of, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return fail(CCSDT_E_CUDA, "(ia|bc) slot table upload");
  }
  return CCSDT_OK;
}

extern "C" long ccsdt_ovvv_slab_builds(const ccsdt_handle* h) { return h ? h->slab_forms : -1; }

extern "C" ccsdt_status ccsdt_debug_set_slab_build(ccsdt_handle* h, int split) {
  if(!h || split < 0 || split > 1) return CCSDT_E_INVALID;
  h->slab_split_build = split != 0;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_debug_slab_schedule(int o, int max_ovvv_slabs, int batch, long n, const int* tri,
                                                 long* order, long* builds) {
  if(o <= 0 || max_ovvv_slabs < 3 || batch <= 0 || 3 * batch > max_ovvv_slabs || n < 0 || (n && (!tri || !order)) ||
     !builds)
    return CCSDT_E_INVALID;
  for(long t = 0; t < n; t++)
    if(!(0 <= tri[3 * t] && tri[3 * t] <= tri[3 * t + 1] && tri[3 * t + 1] <= tri[3 * t + 2] && tri[3 * t + 2] < o))
      return CCSDT_E_INVALID;
  const std::vector<long> ord = ccsdt::slab_order(tri, n, max_ovvv_slabs);
  ccsdt::SlabCache        cache;
  cache.reset(o, max_ovvv_slabs);
  std::vector<std::pair<int, int>> todo;
  for(long b0 = 0; b0 < n; b0 += batch) {
    std::vector<int> need;
    for(long t = b0; t < std::min(n, b0 + batch); t++)
      for(int q = 0; q < 3; q++) need.push_back(tri[3 * ord[t] + q]);
    if(!cache.require(need.data(), (int) need.size(), todo)) return CCSDT_E_STATE;
    for(int x: need)
      if(cache.slot(x) < 0 || cache.owner(cache.slot(x)) != x) return CCSDT_E_STATE;
  }
  for(long t = 0; t < n; t++) order[t] = ord[t];
  *builds = cache.builds();
  return CCSDT_OK;
}
