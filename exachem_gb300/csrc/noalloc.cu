// Allocation-free FP64 (T): the plain FP64 path run on a fixed, file-scope device scratch.
//
// For callers that cannot call cudaMalloc: a host runtime whose device memory is owned by a
// pooled allocator (ExaChem's TAMM runs on an RMM pool that takes the device up front, so a
// cudaMalloc beside it fails or fragments the pool), or a service held to a fixed device-memory
// budget.  The caller passes device inputs and a device output; every intermediate lives in
// `g_noalloc_scratch` below.
//
// Limits: o <= 12, v <= 48.  The scratch is NOALLOC_DOUBLES doubles (about 6.0 MB); every GPU
// that loads this library holds it until the process exits.  All calls share it: two calls that
// overlap on the GPU (different streams, or different host threads without ordering) race on it
// and give wrong results.  Nothing in it needs clearing between calls: each call writes every
// element it reads before reading it.  The first call on a device looks up the array's device
// address and keeps it for the process; after a cudaDeviceReset the module may load at another
// address, so the entry point must not be used across a device reset.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"

using namespace ccsdt;

namespace {

constexpr int       kOMax = 12, kVMax = 48;
constexpr long long kTriMax = (long long) kOMax * (kOMax + 1) * (kOMax + 2) / 6;
// layout of the scratch (in doubles)
constexpr long long kOffT2h   = 0;
constexpr long long kOffOoovh = kOffT2h + (long long) kOMax * kOMax * kVMax * kVMax;
constexpr long long kOffP12   = kOffOoovh + (long long) kOMax * kOMax * kOMax * kVMax;
constexpr long long kOffP34   = kOffP12 + (long long) kVMax * kVMax * kVMax;
constexpr long long kOffP56   = kOffP34 + (long long) kVMax * kVMax * kVMax;
constexpr long long kOffPart  = kOffP56 + (long long) kVMax * kVMax * kVMax;
constexpr long long kOffTrip  = kOffPart + 4LL * kEnergyBlocks;
constexpr long long NOALLOC_DOUBLES = kOffTrip + 2 * kTriMax;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex    g_mu;
double*       g_scratch_addr[kMaxDevices] = {};

int mult(int i, int j, int k) {
  if(i == j && j == k) return 1;
  if(i == j || j == k || i == k) return 3;
  return 6;
}

} // namespace

extern "C" ccsdt_status ccsdt_energy_noalloc(int o, int v, const double* eps_occ, const double* eps_vir,
                                             const double* t1, const double* t2, const double* oovv,
                                             const double* ooov, const double* ovvv, double* energies,
                                             void* stream) {
  if(o <= 0 || v <= 0 || o > kOMax || v > kVMax) return CCSDT_E_INVALID;
  if(!eps_occ || !eps_vir || !t1 || !t2 || !oovv || !ooov || !ovvv || !energies) return CCSDT_E_INVALID;
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return CCSDT_E_CUDA;
  }
  double* base = nullptr;
  {
    // first call on this device: device address of the scratch (host code must not use the
    // symbol itself, which is only a host-side stand-in)
    std::lock_guard<std::mutex> lock(g_mu);
    if(!g_scratch_addr[dev]) {
      void* p = nullptr;
      if(cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return CCSDT_E_CUDA;
      }
      g_scratch_addr[dev] = static_cast<double*>(p);
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long O = o, V = v, v2 = V * V, v3 = v2 * V;
  double *t2h = base + kOffT2h, *ooovh = base + kOffOoovh, *P12 = base + kOffP12, *P34 = base + kOffP34,
         *P56 = base + kOffP56, *part = base + kOffPart, *etrip = base + kOffTrip;

  transpose_mid_kernel<<<256, 256, 0, st>>>(t2, t2h, o, o, v2);
  transpose_mid_kernel<<<64, 256, 0, st>>>(ooov, ooovh, o, o, O * V);
  if(cudaGetLastError() != cudaSuccess) return CCSDT_E_CUDA;

  long ntri = 0;
  for(int i = 0; i < o; i++)
    for(int j = i; j < o; j++)
      for(int k = j; k < o; k++, ntri++) {
        double* eout = etrip + 2 * ntri;
        if(i == k) { // W symmetric in (a, b, c): the triplet contributes exactly zero
          if(cudaMemsetAsync(eout, 0, 2 * sizeof(double), st) != cudaSuccess) return CCSDT_E_CUDA;
          continue;
        }
        auto         t2h_of = [&](int x) { return t2h + (long long) x * v2 * O; };
        auto         ooh_of = [&](int y, int z) { return ooovh + ((long long) y * O + z) * V * O; };
        const RowMap pn = plain_rows(O), ps = swapped_pair_rows(v, O), sg = plain_rows(O);
        GemmBatch    hb{};
        hb.job[0] = GemmJob{{GemmTerm{t2h_of(i), pn, ooh_of(k, j), sg, o, -1.0},
                             GemmTerm{t2h_of(k), ps, ooh_of(i, j), sg, o, -1.0}}, 2, P12, v2, V, 0.0};
        hb.job[1] = GemmJob{{GemmTerm{t2h_of(i), ps, ooh_of(j, k), sg, o, -1.0},
                             GemmTerm{t2h_of(j), pn, ooh_of(i, k), sg, o, -1.0}}, 2, P34, v2, V, 0.0};
        hb.job[2] = GemmJob{{GemmTerm{t2h_of(j), ps, ooh_of(k, i), sg, o, -1.0},
                             GemmTerm{t2h_of(k), pn, ooh_of(j, i), sg, o, -1.0}}, 2, P56, v2, V, 0.0};
        const long long ht = ((v2 + D_BM - 1) / D_BM) * ((V + D_BN - 1) / D_BN);
        dmma_gemm_kernel<<<dim3((unsigned) ht, 1, 3), D_THREADS, 0, st>>>(hb);
        auto         t2_of   = [&](int x, int y) { return t2 + ((long long) x * O + y) * v2; };
        auto         ovvv_of = [&](int z) { return ovvv + (long long) z * v3; };
        const RowMap ar = plain_rows(V), bn = plain_rows(V), bs = swapped_pair_rows(v, V);
        GemmBatch    pb{};
        pb.job[0] = GemmJob{{GemmTerm{t2_of(i, j), ar, ovvv_of(k), bn, v, 1.0},
                             GemmTerm{t2_of(i, k), ar, ovvv_of(j), bs, v, 1.0}}, 2, P12, V, v2, 1.0};
        pb.job[1] = GemmJob{{GemmTerm{t2_of(j, i), ar, ovvv_of(k), bs, v, 1.0},
                             GemmTerm{t2_of(j, k), ar, ovvv_of(i), bn, v, 1.0}}, 2, P34, V, v2, 1.0};
        pb.job[2] = GemmJob{{GemmTerm{t2_of(k, i), ar, ovvv_of(j), bn, v, 1.0},
                             GemmTerm{t2_of(k, j), ar, ovvv_of(i), bs, v, 1.0}}, 2, P56, V, v2, 1.0};
        const long long pt = ((V + D_BM - 1) / D_BM) * ((v2 + D_BN - 1) / D_BN);
        dmma_gemm_kernel<<<dim3((unsigned) pt, 1, 3), D_THREADS, 0, st>>>(pb);
        EnergyArgs ea{P12, P34, P56, oovv, t1, eps_occ, eps_vir, o, v, i, j, k, part};
        energy_fp64_kernel<<<kEnergyBlocks, E_THREADS, 0, st>>>(ea);
        reduce_parts_kernel<<<1, E_THREADS, 0, st>>>(part, kEnergyBlocks, mult(i, j, k) / 9.0, eout);
        if(cudaGetLastError() != cudaSuccess) return CCSDT_E_CUDA;
      }
  reduce_triplets_kernel<<<1, 32, 0, st>>>(etrip, ntri, energies);
  if(cudaGetLastError() != cudaSuccess) return CCSDT_E_CUDA;
  return CCSDT_OK;
}
