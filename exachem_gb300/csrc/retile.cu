// Device-side retile of ExaChem's spin-orbital tile blocks into the closed-shell spatial arrays.
//
// The reference's gathers fetch one tile block at a time with Tensor::get and transpose it on the
// host (ccsd_t_all_fused_doubles1.hpp:216-246, doubles2.hpp:211-239, 335-343, singles.hpp:196-313);
// a host-side gather of the whole input (75 GB at o=60 v=500) costs minutes.  Here the caller
// hands over the blocks exactly as Tensor::get returns them (row-major in the tensor's index
// order), many per call, and one kernel scatters them into the handle's arrays in HBM:
//   T2    block (A, B, I, J) of t2(a_alpha, b_beta, i_alpha, j_beta)     [a][b][i][j] -> t2[i][j][a][b]
//   OOVV  block (I, J, A, B) of v2ijab(i_a, j_b, a_a, b_b) = (ia|jb)      [i][j][a][b] -> oovv[i][j][a][b]
//   OOOV  block (I, K, J, A) of v2ijka(i_a, k_b, j_a, a_b) = (ij|ka)      [i][k][j][a] -> ooov[i][j][k][a]
//   OVVV  block (I, B, A, C) of v2iabc(i_a, b_b, a_a, c_b) = (ia|bc)      [i][b][a][c] -> ovvv[i][a][b][c]
// (the same index maps as the C++ adapter's host gather, gather_closed_shell).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"

using namespace ccsdt;

namespace {

struct RetileArgs {
  const double*    src;
  const int4*      tiles;   // per block: tile indices in the block's index order
  const long long* offs;    // per block: element offset in src
  const int*       tt;      // [occ offsets | occ extents | vir offsets | vir extents]
  int              nocc, nvir, kind, o, v;
  double*          dst;
};

// grid (blocks, chunks): CTA (b, y) writes elements y, y + chunks, ... (x 256 threads) of block b
__global__ void __launch_bounds__(256) retile_kernel(const __grid_constant__ RetileArgs A) {
  const int4      t   = A.tiles[blockIdx.x];
  const int*      oo  = A.tt;
  const int*      ot  = A.tt + A.nocc;
  const int*      vo  = A.tt + 2 * A.nocc;
  const int*      vt  = A.tt + 2 * A.nocc + A.nvir;
  const long long o = A.o, v = A.v;
  // extents of the block's four indices and the destination of element (q0, q1, q2, q3)
  int d0, d1, d2, d3;
  switch(A.kind) {
    case CCSDT_BLOCKS_T2: d0 = vt[t.x], d1 = vt[t.y], d2 = ot[t.z], d3 = ot[t.w]; break;
    case CCSDT_BLOCKS_OOVV: d0 = ot[t.x], d1 = ot[t.y], d2 = vt[t.z], d3 = vt[t.w]; break;
    case CCSDT_BLOCKS_OOOV: d0 = ot[t.x], d1 = ot[t.y], d2 = ot[t.z], d3 = vt[t.w]; break;
    default: d0 = ot[t.x], d1 = vt[t.y], d2 = vt[t.z], d3 = vt[t.w]; break;
  }
  const long long n    = (long long) d0 * d1 * d2 * d3;
  const double*   src  = A.src + A.offs[blockIdx.x];
  const long long step = (long long) gridDim.y * blockDim.x;
  for(long long e = (long long) blockIdx.y * blockDim.x + threadIdx.x; e < n; e += step) {
    const int q3 = (int) (e % d3), q2 = (int) ((e / d3) % d2), q1 = (int) ((e / ((long long) d3 * d2)) % d1),
              q0 = (int) (e / ((long long) d3 * d2 * d1));
    long long dst;
    switch(A.kind) {
      case CCSDT_BLOCKS_T2: // [a][b][i][j] -> t2[i][j][a][b]
        dst = (((oo[t.z] + q2) * o + oo[t.w] + q3) * v + vo[t.x] + q0) * v + vo[t.y] + q1;
        break;
      case CCSDT_BLOCKS_OOVV: // [i][j][a][b] -> oovv[i][j][a][b]
        dst = (((oo[t.x] + q0) * o + oo[t.y] + q1) * v + vo[t.z] + q2) * v + vo[t.w] + q3;
        break;
      case CCSDT_BLOCKS_OOOV: // [i][k][j][a] -> ooov[i][j][k][a]
        dst = (((oo[t.x] + q0) * o + oo[t.z] + q2) * o + oo[t.y] + q1) * v + vo[t.w] + q3;
        break;
      default: // [i][b][a][c] -> ovvv[i][a][b][c]
        dst = (((oo[t.x] + q0) * v + vo[t.z] + q2) * v + vo[t.y] + q1) * v + vo[t.w] + q3;
        break;
    }
    A.dst[dst] = src[e];
  }
}

} // namespace

extern "C" ccsdt_status ccsdt_upload_begin(ccsdt_handle* h, const double* eps_occ, const double* eps_vir,
                                          const double* t1, int on_device) {
  if(!h) return CCSDT_E_INVALID;
  if(!eps_occ || !eps_vir || !t1) return h->fail(CCSDT_E_INVALID, "ccsdt_upload_begin: null input pointer");
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  ccsdt_status s;
  if((s = h->ensure_inputs())) return s;
  const size_t o = h->o, v = h->v;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaError_t e = cudaMemcpyAsync(h->eo, eps_occ, o * sizeof(double), kind, h->stream);
  if(e == cudaSuccess) e = cudaMemcpyAsync(h->ev, eps_vir, v * sizeof(double), kind, h->stream);
  if(e == cudaSuccess) e = cudaMemcpyAsync(h->t1, t1, o * v * sizeof(double), kind, h->stream);
  // blocks not handed over stay zero
  if(e == cudaSuccess) e = cudaMemsetAsync(h->t2, 0, o * o * v * v * sizeof(double), h->stream);
  if(e == cudaSuccess) e = cudaMemsetAsync(h->oovv, 0, o * o * v * v * sizeof(double), h->stream);
  if(e == cudaSuccess) e = cudaMemsetAsync(h->ooov, 0, o * o * o * v * sizeof(double), h->stream);
  if(e == cudaSuccess) e = cudaMemsetAsync(h->ovvv, 0, o * v * v * v * sizeof(double), h->stream);
  if(e == cudaSuccess && !h->blk_tiles) { // tile offsets and extents of the layout
    std::vector<int> tt;
    for(int pass = 0; pass < 2; pass++) {
      const std::vector<int>& ext = pass == 0 ? h->occ_tiles : h->vir_tiles;
      int                     off = 0;
      for(int x: ext) tt.push_back(off), off += x;
      tt.insert(tt.end(), ext.begin(), ext.end());
    }
    if(ccsdt::dev_malloc((void**) &h->blk_tiles, tt.size() * sizeof(int)) != cudaSuccess) {
      h->blk_tiles = nullptr;
      cudaGetLastError();
      return h->fail(CCSDT_E_OOM, "tile table");
    }
    h->owned_bytes.push_back(h->blk_tiles);
    e = cudaMemcpy(h->blk_tiles, tt.data(), tt.size() * sizeof(int), cudaMemcpyHostToDevice);
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("ccsdt_upload_begin: ") + cudaGetErrorString(e));
  h->uploaded    = false;
  h->blocks_open = true;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_upload_blocks(ccsdt_handle* h, int kind, long n, const int* tiles,
                                           const long long* offsets, const double* data, long long data_len,
                                           int on_device) {
  if(!h) return CCSDT_E_INVALID;
  if(!h->blocks_open) return h->fail(CCSDT_E_STATE, "ccsdt_upload_blocks outside ccsdt_upload_begin / end");
  if(kind < CCSDT_BLOCKS_T2 || kind > CCSDT_BLOCKS_OVVV || n < 0 || (n && (!tiles || !offsets || !data)) ||
     data_len < 0)
    return h->fail(CCSDT_E_INVALID, "ccsdt_upload_blocks: bad arguments");
  if(n == 0) return CCSDT_OK;
  const int nocc = (int) h->occ_tiles.size(), nvir = (int) h->vir_tiles.size();
  // which of the four block indices are occupied (1) or virtual (0)
  static const int occ_pos[4][4] = {{0, 0, 1, 1}, {1, 1, 0, 0}, {1, 1, 1, 0}, {1, 0, 0, 0}};
  const int* op = occ_pos[kind];
  for(long b = 0; b < n; b++) {
    long long sz = 1;
    for(int q = 0; q < 4; q++) {
      const int t = tiles[4 * b + q], lim = op[q] ? nocc : nvir;
      if(t < 0 || t >= lim) return h->fail(CCSDT_E_INVALID, "ccsdt_upload_blocks: tile index outside the layout");
      sz *= op[q] ? h->occ_tiles[t] : h->vir_tiles[t];
    }
    if(offsets[b] < 0 || offsets[b] + sz > data_len)
      return h->fail(CCSDT_E_INVALID, "ccsdt_upload_blocks: block outside the data buffer");
  }
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  // per-block metadata, and the data itself in device memory
  const size_t meta_bytes = (size_t) n * (sizeof(int4) + sizeof(long long));
  if(h->blk_meta_cap < (long) meta_bytes) {
    if(h->blk_meta) cudaFree(h->blk_meta);
    h->blk_meta = nullptr;
    if(ccsdt::dev_malloc((void**) &h->blk_meta, meta_bytes) != cudaSuccess) {
      cudaGetLastError();
      h->blk_meta_cap = 0;
      return h->fail(CCSDT_E_OOM, "block metadata");
    }
    h->blk_meta_cap = (long) meta_bytes;
  }
  std::vector<unsigned char> meta(meta_bytes);
  std::memcpy(meta.data(), tiles, (size_t) n * sizeof(int4));
  std::memcpy(meta.data() + (size_t) n * sizeof(int4), offsets, (size_t) n * sizeof(long long));
  cudaError_t e = cudaMemcpyAsync(h->blk_meta, meta.data(), meta_bytes, cudaMemcpyHostToDevice, h->stream);
  const double* src = data;
  if(e == cudaSuccess && !on_device) {
    if(h->blk_stage_cap < data_len) {
      if(h->blk_stage) cudaFree(h->blk_stage);
      h->blk_stage = nullptr;
      if(ccsdt::dev_malloc((void**) &h->blk_stage, (size_t) data_len * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        h->blk_stage_cap = 0;
        return h->fail(CCSDT_E_OOM, "block staging buffer of " + std::to_string(data_len * 8) + " bytes");
      }
      h->blk_stage_cap = data_len;
    }
    e   = cudaMemcpyAsync(h->blk_stage, data, (size_t) data_len * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    src = h->blk_stage;
  }
  if(e == cudaSuccess) {
    RetileArgs a;
    a.src   = src;
    a.tiles = reinterpret_cast<const int4*>(h->blk_meta);
    a.offs  = reinterpret_cast<const long long*>(reinterpret_cast<const unsigned char*>(h->blk_meta) +
                                                (size_t) n * sizeof(int4));
    a.tt = h->blk_tiles, a.nocc = nocc, a.nvir = nvir, a.kind = kind, a.o = h->o, a.v = h->v;
    a.dst = kind == CCSDT_BLOCKS_T2 ? h->t2 : kind == CCSDT_BLOCKS_OOVV ? h->oovv : kind == CCSDT_BLOCKS_OOOV ? h->ooov : h->ovvv;
    const unsigned chunks = (unsigned) std::max<long>(1, std::min<long>(64, 4096 / std::max<long>(1, n)));
    retile_kernel<<<dim3((unsigned) n, chunks), 256, 0, h->stream>>>(a);
    h->launches++;
    e = cudaGetLastError();
  }
  // the caller may reuse its buffers as soon as the call returns
  if(e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("ccsdt_upload_blocks: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_upload_end(ccsdt_handle* h) {
  if(!h) return CCSDT_E_INVALID;
  if(!h->blocks_open) return h->fail(CCSDT_E_STATE, "ccsdt_upload_end without ccsdt_upload_begin");
  if(cudaSetDevice(h->device) != cudaSuccess) return h->fail(CCSDT_E_CUDA, "cudaSetDevice");
  h->blocks_open = false;
  return h->finish_inputs("ccsdt_upload_end");
}
