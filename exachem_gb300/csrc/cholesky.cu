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

#include <string>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"

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

extern "C" ccsdt_status ccsdt_upload_cholesky(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                             const double* t1, const double* t2, int n_chol,
                                             const double* chol_oo, const double* chol_ov, const double* chol_vv,
                                             int on_device) {
  if(!h) return CCSDT_E_INVALID;
  if(!eps_occ || !eps_vir || !t1 || !t2 || !chol_oo || !chol_ov || !chol_vv)
    return h->fail(CCSDT_E_INVALID, "ccsdt_upload_cholesky: null input pointer");
  if(n_chol <= 0) return h->fail(CCSDT_E_INVALID, "ccsdt_upload_cholesky: n_chol must be positive");
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  ccsdt_status s;
  if((s = h->ensure_inputs())) return s;
  h->blocks_open = false;
  h->uploaded    = false;
  const long long o = h->o, v = h->v, nq = n_chol;
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
  if(e == cudaSuccess && !on_device) {
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
  if(e == cudaSuccess) e = gemm_abt(L_ov, L_vv, h->ovvv, o * v, v * v, (int) nq, h->stream); // (ia|bc)
  if(e == cudaSuccess) e = gemm_abt(L_oo, L_ov, h->ooov, o * o, o * v, (int) nq, h->stream); // (ij|ka)
  if(e == cudaSuccess) e = gemm_abt(L_ov, L_ov, h->t2h, o * v, o * v, (int) nq, h->stream);  // [(i,a)][(j,b)]
  if(e == cudaSuccess) {
    swap_ia_jb_kernel<<<2048, 256, 0, h->stream>>>(h->t2h, h->oovv, (int) o, (int) v);
    e = cudaGetLastError();
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if(scratch) cudaFree(scratch);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("ccsdt_upload_cholesky: ") + cudaGetErrorString(e));
  return h->finish_inputs("ccsdt_upload_cholesky");
}
