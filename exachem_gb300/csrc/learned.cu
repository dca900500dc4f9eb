// Learned per-triplet slice count: features, model storage and the LEARNED mode.
//
// No counterpart in the reference.  For every occupied triplet a small MLP (mlp.cu) reads 12
// features and predicts the digit-plane count S in 2..8 that keeps the triplet's energy error
// under a budget.  After the run an a-posteriori estimate is formed per triplet,
//     est = 6 * tail * 2^-6 * sqrt(sum_abc ((|Z| + |Y|) / |D|)^2)      (times m / 9)
// with `tail` the largest contribution of the last kept digit level (the dropped levels are
// each about 2^-7 of it) and the sum the first-order sensitivity of the energy to W.  A triplet
// whose estimate exceeds budget * |E_triplet| is recomputed with the full slice count.
// The element errors are treated as independent (a random walk): the sensitivity is the
// root of the summed squares, sqrt(sum_abc ((|Z| + |Y|) / |D|)^2), not the plain sum.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"

namespace {

constexpr int NF = CCSDT_MLP_IN;

// max / min of the row exponents in consecutive groups of `len` rows
__global__ void exp_stats_kernel(const int* __restrict__ e, long long len, int groups, int* __restrict__ out) {
  const int g = blockIdx.x;
  if(g >= groups) return;
  int mx = -1000000, mn = 1000000;
  for(long long r = threadIdx.x; r < len; r += blockDim.x) {
    const int x = e[(long long) g * len + r];
    mx = max(mx, x);
    mn = min(mn, x);
  }
  __shared__ int smx[256], smn[256];
  smx[threadIdx.x] = mx;
  smn[threadIdx.x] = mn;
  __syncthreads();
  for(int s = blockDim.x / 2; s > 0; s >>= 1) {
    if((int) threadIdx.x < s) {
      smx[threadIdx.x] = max(smx[threadIdx.x], smx[threadIdx.x + s]);
      smn[threadIdx.x] = min(smn[threadIdx.x], smn[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    out[2 * g]     = smx[0];
    out[2 * g + 1] = smn[0];
  }
}

// 12 features per triplet (exponents scaled by 1/8 to stay O(1)):
//  0 v/512   1 o/64   2..4 max row exponent of the (ia|bc) slabs i, j, k
//  5 max and 6 min row exponent over the six amplitude blocks t_xy, x,y in {i,j,k}
//  7 min row exponent of the three slabs   8 log10 min |D|   9 log10 max |D|
// 10 degeneracy (i==j) + (j==k)   11 max row exponent of the l-sum amplitudes t_x.^..
__global__ void features_kernel(const int* __restrict__ tri, long n, int o, int v, const int* __restrict__ slab,
                                const int* __restrict__ pair, const int* __restrict__ hole, const double* __restrict__ eo,
                                const double* __restrict__ ev, float* __restrict__ F) {
  const long t = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if(t >= n) return;
  const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
  const int x3[3] = {i, j, k};
  float*    f = F + t * NF;
  f[0] = v / 512.f;
  f[1] = o / 64.f;
  for(int q = 0; q < 3; q++) f[2 + q] = slab[2 * x3[q]] / 8.f;
  int pmax = -1000000, pmin = 1000000, smin = 1000000, hmax = -1000000;
  for(int a = 0; a < 3; a++) {
    smin = min(smin, slab[2 * x3[a] + 1]);
    hmax = max(hmax, hole[2 * x3[a]]);
    for(int b = 0; b < 3; b++) {
      if(a == b) continue;
      const int p = x3[a] * o + x3[b];
      pmax        = max(pmax, pair[2 * p]);
      pmin        = min(pmin, pair[2 * p + 1]);
    }
  }
  f[5]            = pmax / 8.f;
  f[6]            = pmin / 8.f;
  f[7]            = smin / 8.f;
  const double e3 = eo[i] + eo[j] + eo[k];
  f[8]            = (float) log10(fmax(3.0 * ev[0] - e3, 1e-300));
  f[9]            = (float) log10(fmax(3.0 * ev[v - 1] - e3, 1e-300));
  f[10]           = (float) ((i == j) + (j == k));
  f[11]           = hmax / 8.f;
}

} // namespace

// the BF16 inference kernel of mlp.cu, re-declared here for the LEARNED mode
void ccsdt_mlp_infer_device(const void* params_bf16, const float* X, long n, int* slices, cudaStream_t st);

ccsdt_status ccsdt_handle::ensure_stats() {
  if(stats_for == slice_gen) return CCSDT_OK;
  const long long o = this->o, v = this->v;
  auto need = [&](int** p, size_t n) -> ccsdt_status {
    if(*p) return CCSDT_OK;
    if(ccsdt::dev_malloc((void**) p, n * sizeof(int)) != cudaSuccess) {
      *p = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "exponent statistics: cudaMalloc failed");
    }
    owned_bytes.push_back(*p);
    return CCSDT_OK;
  };
  ccsdt_status s;
  if((s = need(&st_slab, 2 * o)) || (s = need(&st_pair, 2 * o * o)) || (s = need(&st_hole, 2 * o))) return s;
  exp_stats_kernel<<<(int) o, 256, 0, stream>>>(ex_ovvv, v * v, (int) o, st_slab);
  exp_stats_kernel<<<(int) (o * o), 256, 0, stream>>>(ex_t2, v, (int) (o * o), st_pair);
  exp_stats_kernel<<<(int) o, 256, 0, stream>>>(ex_t2h, v * v, (int) o, st_hole);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("exponent statistics: ") + cudaGetErrorString(e));
  stats_for = slice_gen;
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::features(long n, const int* tri_dev, float* feats_dev) {
  ccsdt_status s;
  if((s = ensure_stats())) return s;
  if(n > 0)
    features_kernel<<<(unsigned) ((n + 127) / 128), 128, 0, stream>>>(tri_dev, n, o, v, st_slab, st_pair, st_hole, eo,
                                                                      ev, feats_dev);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("features: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

namespace {
struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for(void* q: p) cudaFree(q);
  }
  template<typename T>
  T* get(size_t n) {
    void* q = nullptr;
    if(ccsdt::dev_malloc(&q, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    p.push_back(q);
    return static_cast<T*>(q);
  }
};
} // namespace

extern "C" ccsdt_status ccsdt_triplet_features(ccsdt_handle* h, long n, const int* tri, float* feats) {
  if(!h) return CCSDT_E_INVALID;
  if(n < 0 || (n > 0 && (!tri || !feats))) return h->fail(CCSDT_E_INVALID, "ccsdt_triplet_features: bad arguments");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_triplet_features before ccsdt_upload");
  for(long t = 0; t < n; t++)
    if(!(0 <= tri[3 * t] && tri[3 * t] <= tri[3 * t + 1] && tri[3 * t + 1] <= tri[3 * t + 2] && tri[3 * t + 2] < h->o))
      return h->fail(CCSDT_E_INVALID, "ccsdt_triplet_features: triplet out of order or range");
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  ccsdt_status s;
  if(h->slices_ready < 1 && (s = h->ensure_slices(1, 0))) return s;
  Scratch sc;
  int*    dt = sc.get<int>(3 * (size_t) n);
  float*  df = sc.get<float>((size_t) n * NF);
  if(!dt || !df) return h->fail(CCSDT_E_OOM, "features scratch");
  if(cudaMemcpyAsync(dt, tri, 3 * sizeof(int) * n, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return h->fail(CCSDT_E_CUDA, "features upload");
  if((s = h->features(n, dt, df))) return s;
  if(cudaMemcpyAsync(feats, df, sizeof(float) * NF * n, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
     cudaStreamSynchronize(h->stream) != cudaSuccess)
    return h->fail(CCSDT_E_CUDA, "features readback");
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_set_slice_model(ccsdt_handle* h, const float* params) {
  if(!h) return CCSDT_E_INVALID;
  if(!params) {
    h->model.clear();
    return CCSDT_OK;
  }
  for(int e = 0; e < CCSDT_MLP_NPARAM; e++)
    if(!std::isfinite(params[e])) return h->fail(CCSDT_E_NONFINITE, "slice model has non-finite parameters");
  h->model.assign(params, params + CCSDT_MLP_NPARAM);
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_learned_stats(const ccsdt_handle* h, double* mean_slices, long* fallbacks,
                                            double* products) {
  if(!h) return CCSDT_E_INVALID;
  if(mean_slices) *mean_slices = h->learned_mean_slices;
  if(fallbacks) *fallbacks = h->learned_fallbacks;
  if(products) *products = h->learned_cost_products;
  return CCSDT_OK;
}

// A-posteriori estimate of the standard deviation of a triplet's truncation error E_S - E_exact
// from the sum of squares of its last kept level's terms (tail_sq, over the 12 v^3 term values of
// the twelve contraction terms) and its sensitivity sens = (m/9)^2 sum_abc (18 Y^2 + 12 Z^2) / D^2
// (|dE/dW_abc|^2 with uncorrelated signs).  The dropped levels are ~2^-7 of the last kept one,
// with signs that do not correlate across the v^3 elements, so
//   sigma ~ kEstScale 2^-7 sqrt(sens tail_sq / v^3).
// A statistical estimate (random-walk model), not a rigorous bound; kEstScale is fitted to
// errors measured against the FP64 path (tests/test_learned.py checks that 3 sigma covers them).
double ccsdt_handle::truncation_estimate(float tail_sq, double sens) const {
  constexpr double kEstScale = 5.0;
  const double     v3         = (double) v * v * v;
  return kEstScale * std::ldexp(1.0, -7) * std::sqrt(sens * (double) tail_sq / v3);
}

extern "C" ccsdt_status ccsdt_triplet_error_estimates(ccsdt_handle* h, const ccsdt_opts* opts, long n, const int* tri,
                                                      double* e_bracket, double* e_paren, double* est) {
  if(!h) return CCSDT_E_INVALID;
  if(!opts || opts->mode != CCSDT_MODE_OZAKI || opts->p_storage < 0 || opts->p_storage > 3 || n < 0 ||
     (n && (!tri || !e_paren || !est)))
    return h->fail(CCSDT_E_INVALID, "ccsdt_triplet_error_estimates: needs CCSDT_MODE_OZAKI and output arrays");
  if(!h->uploaded) return h->fail(CCSDT_E_STATE, "ccsdt_triplet_error_estimates before ccsdt_upload");
  if(!h->pz_eligible(opts->slices, opts->slice_kind))
    return h->fail(CCSDT_E_INVALID, "error estimates need the tcgen05 path (BF16 digits, 1..8 planes)");
  for(long t = 0; t < n; t++) {
    const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    if(!(0 <= i && i <= j && j <= k && k < h->o)) return h->fail(CCSDT_E_INVALID, "triplet outside 0 <= i <= j <= k < o");
  }
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  if(n == 0) return CCSDT_OK;
  ccsdt_status s;
  if((s = h->ensure_triplet_slots(n)) || (s = h->ensure_slices(opts->slices, 0))) return s;
  Scratch sc;
  float*  dtail = sc.get<float>((size_t) n);
  double* dsens = sc.get<double>((size_t) n);
  if(!dtail || !dsens) return h->fail(CCSDT_E_OOM, "estimate scratch");
  if(cudaMemsetAsync(dtail, 0, sizeof(float) * n, h->stream) != cudaSuccess ||
     cudaMemsetAsync(dsens, 0, sizeof(double) * n, h->stream) != cudaSuccess ||
     cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream) != cudaSuccess)
    return h->fail(CCSDT_E_CUDA, "estimate scratch init");
  h->force_mma_sync   = false;
  h->p_storage = opts->p_storage;
  if((s = h->run_batched(opts->slices, n, tri, false, dtail, dsens))) return s;
  std::vector<double> E(2 * n), sens(n);
  std::vector<float>  tail(n);
  if(cudaMemcpyAsync(E.data(), h->etrip, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
     cudaMemcpyAsync(tail.data(), dtail, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
     cudaMemcpyAsync(sens.data(), dsens, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
     cudaStreamSynchronize(h->stream) != cudaSuccess)
    return h->fail(CCSDT_E_CUDA, "estimate readback");
  if((s = h->check_device_error())) return s;
  for(long t = 0; t < n; t++) {
    if(e_bracket) e_bracket[t] = E[2 * t];
    e_paren[t] = E[2 * t + 1];
    est[t]     = tri[3 * t] == tri[3 * t + 2] ? 0.0 : h->truncation_estimate(tail[t], sens[t]);
  }
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::run_learned(const ccsdt_opts* opts, long n, const int* tri) {
  if(model.size() != (size_t) CCSDT_MLP_NPARAM) return fail(CCSDT_E_STATE, "LEARNED mode needs ccsdt_set_slice_model");
  const int Sfull = opts->slices >= 2 && opts->slices <= 8 ? opts->slices : 5;
  ccsdt_status s;
  if((s = ensure_slices(Sfull, 0))) return s;
  Scratch sc;
  int*     dt    = sc.get<int>(3 * (size_t) n);
  float*   df    = sc.get<float>((size_t) n * NF);
  int*     dsl   = sc.get<int>((size_t) n);
  float*   dtail = sc.get<float>((size_t) n);
  double*  dsens = sc.get<double>((size_t) n);
  if(!dt || !df || !dsl || !dtail || !dsens) return fail(CCSDT_E_OOM, "learned-mode scratch");
  if(!model_bf16) {
    if(ccsdt::dev_malloc(&model_bf16, CCSDT_MLP_NPARAM * sizeof(__nv_bfloat16)) != cudaSuccess) {
      model_bf16 = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "model buffer");
    }
    owned_bytes.push_back(model_bf16);
  }
  std::vector<__nv_bfloat16> mb(CCSDT_MLP_NPARAM);
  for(int e = 0; e < CCSDT_MLP_NPARAM; e++) mb[e] = __float2bfloat16_rn(model[e]);
  if(cudaMemcpyAsync(model_bf16, mb.data(), mb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, stream) !=
       cudaSuccess ||
     cudaMemcpyAsync(dt, tri, 3 * sizeof(int) * n, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
     cudaMemsetAsync(dtail, 0, sizeof(float) * n, stream) != cudaSuccess ||
     cudaMemsetAsync(dsens, 0, sizeof(double) * n, stream) != cudaSuccess ||
     cudaMemsetAsync(d_err, 0, sizeof(int), stream) != cudaSuccess)
    return fail(CCSDT_E_CUDA, "learned-mode upload");
  if((s = features(n, dt, df))) return s;
  ccsdt_mlp_infer_device(model_bf16, df, n, dsl, stream);
  std::vector<int> S(n);
  if(cudaMemcpyAsync(S.data(), dsl, sizeof(int) * n, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
     cudaStreamSynchronize(stream) != cudaSuccess)
    return fail(CCSDT_E_CUDA, "learned-mode slice readback");
  // run the triplets at their predicted counts, one persistent batched pass per count (the
  // persistent tcgen05 path); results, tails and sensitivities land at each triplet's own index
  force_mma_sync = false;
  const bool graph = opts->use_graph != 0;
  double     ssum  = 0;
  auto       group = [&](int cnt, const std::vector<long>& ids, bool with_est) -> ccsdt_status {
    if(ids.empty()) return CCSDT_OK;
    std::vector<int> sub(3 * ids.size()), out(ids.size());
    for(size_t q = 0; q < ids.size(); q++) {
      for(int c = 0; c < 3; c++) sub[3 * q + c] = tri[3 * ids[q] + c];
      out[q] = (int) ids[q];
    }
    if(pz_eligible(cnt, 0))
      return run_batched(cnt, (long) ids.size(), sub.data(), graph, with_est ? dtail : nullptr,
                         with_est ? dsens : nullptr, out.data());
    for(size_t q = 0; q < ids.size(); q++) { // counts above the tcgen05 range: per-triplet slices
      const int i = sub[3 * q], j = sub[3 * q + 1], k = sub[3 * q + 2];
      const long t = ids[q];
      if(i == k) {
        if(cudaMemsetAsync(etrip + 2 * t, 0, 2 * sizeof(double), stream) != cudaSuccess)
          return fail(CCSDT_E_CUDA, "memset");
        continue;
      }
      cur_tail = with_est ? dtail + t : nullptr;
      cur_sens = with_est ? dsens + t : nullptr;
      ccsdt_status r = run_triplet_S(i, j, k, cnt, etrip + 2 * t);
      cur_tail = nullptr;
      cur_sens = nullptr;
      if(r) return r;
    }
    return CCSDT_OK;
  };
  // effective count: predictions the estimate cannot check (above the tcgen05 range, which
  // collects it) run at the full count directly
  for(long t = 0; t < n; t++) {
    S[t] = std::min(std::max(S[t], 2), Sfull);
    if(!pz_eligible(S[t], 0)) S[t] = Sfull;
  }
  for(int cnt = 2; cnt <= Sfull; cnt++) {
    std::vector<long> ids;
    for(long t = 0; t < n; t++)
      if(S[t] == cnt) ids.push_back(t);
    if((s = group(cnt, ids, true))) return s;
  }
  learned_mean_slices = 0;
  ssum                = 0; // digit-plane products actually run (S (S + 1) / 2 per run)
  long nz             = 0;
  for(long t = 0; t < n; t++)
    if(tri[3 * t] != tri[3 * t + 2]) {
      learned_mean_slices += S[t];
      ssum += S[t] * (S[t] + 1) / 2.0;
      nz++;
    }
  learned_mean_slices = nz ? learned_mean_slices / nz : 0.0;
  // Acceptance on the total: the call is accepted when 3 sum_t est_t <= budget x sum_t |E(T)_t|,
  // est_t the estimated standard deviation of triplet t's truncation error.  The errors are summed
  // linearly, not in quadrature: measured against FP64 at o=60 v=500, the triplets' truncation
  // errors share their sign often enough that the error of the sum is close to the sum of the
  // errors, and a quadrature test accepted two digit planes at a budget their whole-call error
  // exceeded 2.5-fold.  The linear test is the same for a call and for any part of it, so
  // batched calls need no share of the allowance.  Otherwise the triplets with the largest
  // estimates are rerun one count higher (each step divides a triplet's error by ~2^7) until the
  // prediction passes.
  std::vector<double> E(2 * n), sens(n), est(n, 0.0);
  std::vector<float>  tail(n);
  auto readback = [&]() -> ccsdt_status {
    if(cudaMemcpyAsync(E.data(), etrip, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
       cudaMemcpyAsync(tail.data(), dtail, sizeof(float) * n, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
       cudaMemcpyAsync(sens.data(), dsens, sizeof(double) * n, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
       cudaStreamSynchronize(stream) != cudaSuccess)
      return fail(CCSDT_E_CUDA, "learned-mode readback");
    for(long t = 0; t < n; t++)
      est[t] = (tri[3 * t] == tri[3 * t + 2] || !pz_eligible(S[t], 0)) ? 0.0 : truncation_estimate(tail[t], sens[t]);
    return CCSDT_OK;
  };
  if((s = readback())) return s;
  double abs_sum = 0;
  for(long t = 0; t < n; t++) abs_sum += std::fabs(E[2 * t + 1]);
  const double target = (opts->energy_budget > 0 ? opts->energy_budget : 1e-8) * abs_sum / 3.0; // on sum est
  learned_fallbacks   = 0;
  for(int round = 0; round < 16; round++) {
    double tot = 0;
    for(long t = 0; t < n; t++) tot += est[t];
    if(tot <= target) break;
    // greedy: largest estimates first, assuming a rerun one count higher leaves 2^-7 of the error
    std::vector<long> order;
    for(long t = 0; t < n; t++)
      if(est[t] > 0 && S[t] < Sfull) order.push_back(t);
    if(order.empty()) break;
    std::sort(order.begin(), order.end(), [&](long a, long b) { return est[a] > est[b]; });
    std::vector<long> redo;
    for(long t: order) {
      if(tot <= target) break;
      tot -= est[t] * (1.0 - std::ldexp(1.0, -7));
      redo.push_back(t);
    }
    learned_fallbacks += (long) redo.size();
    for(int cnt = 3; cnt <= Sfull; cnt++) {
      std::vector<long> ids;
      for(long t: redo)
        if(S[t] + 1 == cnt) ids.push_back(t);
      if(ids.empty()) continue;
      for(long t: ids) { // fresh estimate slots for the rerun
        ssum += cnt * (cnt + 1) / 2.0;
        if(cudaMemsetAsync(dtail + t, 0, sizeof(float), stream) != cudaSuccess ||
           cudaMemsetAsync(dsens + t, 0, sizeof(double), stream) != cudaSuccess)
          return fail(CCSDT_E_CUDA, "estimate reset");
      }
      if((s = group(cnt, ids, true))) return s;
    }
    for(long t: redo) S[t] += 1;
    if((s = readback())) return s;
  }
  double tot = 0;
  for(long t = 0; t < n; t++) tot += est[t];
  last_err_bound = 3.0 * tot;
  learned_cost_products = ssum;
  return CCSDT_OK;
}
