// Split-precision (T): Ozaki slice contractions on the tensor cores, float-float
// recombination and a float-float energy.  Same contraction plan as the FP64 path
// (three partial arrays P12 / P34 / P56 per triplet; l-sum GEMMs initialise them, d-sum
// GEMMs accumulate), with every GEMM run on digit planes.
//
// Two tensor-core variants of the slice products, selected by opts->slice_kind:
//   0: BF16 digits, mma.sync m16n8k16 with FP32 accumulation (exact per level, K <= 512)
//   1: INT8 digits, mma.sync m16n8k32 with INT32 accumulation (exact per level)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <string>

#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"
#include "energy_tiled.cuh"
#include "oz_tc.cuh"
#include "ozaki.cuh"

using namespace ccsdt;

namespace {

constexpr int OZ_BM = 64, OZ_BN = 64, OZ_THREADS = 256, OZ_LEVELS = 4, OZ_KWIN = 512;

template<typename T>
struct OzTraits;
template<>
struct OzTraits<__nv_bfloat16> {
  static constexpr int KC = 32;        // contraction elements per smem chunk
  static constexpr int KSTEP = 16;     // per mma
  using Acc = float;
};
template<>
struct OzTraits<int8_t> {
  static constexpr int KC = 64;
  static constexpr int KSTEP = 32;
  using Acc = int;
};

__device__ __forceinline__ void mma_k(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
               "{%8,%9}, {%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ void mma_k(int (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
               "{%8,%9}, {%0,%1,%2,%3};\n"
               : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragment loads from a [rows][ROWB bytes] smem tile.  For both variants the 32-bit word
// at (row, word w) holds 2 bf16 / 4 int8 consecutive along k; the m16n8k16 (bf16) and
// m16n8k32 (s8) fragments use words: a0 (g, t) a1 (g+8, t) a2 (g, t+4) a3 (g+8, t+4);
// b0 (n = g, t) b1 (g, t+4), with k-step offset ks words.
__device__ __forceinline__ uint32_t lds32(const unsigned char* base, int row, int word) {
  return *reinterpret_cast<const uint32_t*>(base + row * 80 + word * 4);
}

template<typename T>
__global__ void __launch_bounds__(OZ_THREADS) oz_gemm_kernel(const __grid_constant__ OzBatch batch) {
  using Tr  = OzTraits<T>;
  using Acc = typename Tr::Acc;
  const OzJob&    J       = batch.job[blockIdx.z];
  const int       S       = batch.S;
  if(J.nterms <= 0 || J.M <= 0 || J.N <= 0) return; // an unused job of the batch
  const long long tiles_n = (J.N + OZ_BN - 1) / OZ_BN;
  const long long m0 = (long long) (blockIdx.x / tiles_n) * OZ_BM, n0 = (long long) (blockIdx.x % tiles_n) * OZ_BN;
  if(m0 >= J.M || n0 >= J.N) return;

  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* As = smem;                               // [S][64 rows][80 B]
  unsigned char* Bs = smem + (size_t) S * OZ_BM * 80;     // [S][64 rows][80 B]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 2) * 32, wn = (warp & 3) * 16; // 2 x 4 warps, warp tile 32 x 16
  const int g = lane >> 2, t = lane & 3;

  ff out[2][2][4];
#pragma unroll
  for(int x = 0; x < 2; x++)
#pragma unroll
    for(int y = 0; y < 2; y++)
#pragma unroll
      for(int z = 0; z < 4; z++) out[x][y][z] = ff{0.f, 0.f};

  for(int term = 0; term < J.nterms; term++) {
    const OzTerm& T_ = J.t[term];
    // exponents of this thread's output rows / columns
    int ea[2][2], eb[2][2];
#pragma unroll
    for(int x = 0; x < 2; x++)
#pragma unroll
      for(int h = 0; h < 2; h++) {
        long long m = m0 + wm + x * 16 + g + h * 8;
        ea[x][h]    = m < J.M && T_.eA ? T_.eA[oz_rid(T_.ma, m)] : 0;
      }
#pragma unroll
    for(int y = 0; y < 2; y++)
#pragma unroll
      for(int e = 0; e < 2; e++) {
        long long n = n0 + wn + y * 8 + 2 * t + e;
        eb[y][e]    = n < J.N && T_.eB ? T_.eB[oz_rid(T_.mb, n)] : 0;
      }
    const T* Ab = static_cast<const T*>(T_.A);
    const T* Bb = static_cast<const T*>(T_.B);
    // loader: thread -> (row = tid / 4, 16-byte word group (tid % 4)) per plane
    const int       lr = tid >> 2, lq = tid & 3;
    const long long ma = m0 + lr, nb = n0 + lr;
    const bool      va = ma < J.M, vb = nb < J.N;
    const long long ra = va ? oz_rid(T_.ma, ma) * T_.Kp : 0, rb = vb ? oz_rid(T_.mb, nb) * T_.Kp : 0;

    for(int lvl0 = 2; lvl0 <= S + 1; lvl0 += OZ_LEVELS) {
      for(int kw = 0; kw < T_.Kp; kw += OZ_KWIN) {
        const int kend = min(T_.Kp, kw + OZ_KWIN);
        Acc       acc[OZ_LEVELS][2][2][4];
#pragma unroll
        for(int l = 0; l < OZ_LEVELS; l++)
#pragma unroll
          for(int x = 0; x < 2; x++)
#pragma unroll
            for(int y = 0; y < 2; y++)
#pragma unroll
              for(int z = 0; z < 4; z++) acc[l][x][y][z] = 0;
        for(int k0 = kw; k0 < kend; k0 += Tr::KC) {
          __syncthreads();
          for(int p = 0; p < S; p++) {
            // 64 bytes of row data per plane: 4 x 16 B, one per thread
            uint4 va4 = make_uint4(0, 0, 0, 0), vb4 = make_uint4(0, 0, 0, 0);
            if(va) va4 = *reinterpret_cast<const uint4*>(Ab + p * T_.planeA + ra + k0 + lq * (16 / sizeof(T)));
            if(vb) vb4 = *reinterpret_cast<const uint4*>(Bb + p * T_.planeB + rb + k0 + lq * (16 / sizeof(T)));
            *reinterpret_cast<uint4*>(As + ((size_t) p * OZ_BM + lr) * 80 + lq * 16) = va4;
            *reinterpret_cast<uint4*>(Bs + ((size_t) p * OZ_BN + lr) * 80 + lq * 16) = vb4;
          }
          __syncthreads();
#pragma unroll
          for(int ks = 0; ks < Tr::KC / Tr::KSTEP; ks++) {
            const int w0 = ks * 8; // 8 words (32 B) per k-step
            for(int q = 1; q <= S; q++) {
              const unsigned char* Bq = Bs + (size_t) (q - 1) * OZ_BN * 80;
              uint32_t             bf[2][2];
#pragma unroll
              for(int y = 0; y < 2; y++) {
                bf[y][0] = lds32(Bq, wn + y * 8 + g, w0 + t);
                bf[y][1] = lds32(Bq, wn + y * 8 + g, w0 + t + 4);
              }
              for(int p = 1; p <= S; p++) {
                const int l = p + q - lvl0;
                if(l < 0 || l >= OZ_LEVELS) continue;
                const unsigned char* Ap = As + (size_t) (p - 1) * OZ_BM * 80;
#pragma unroll
                for(int x = 0; x < 2; x++) {
                  uint32_t af[4];
                  af[0] = lds32(Ap, wm + x * 16 + g, w0 + t);
                  af[1] = lds32(Ap, wm + x * 16 + g + 8, w0 + t);
                  af[2] = lds32(Ap, wm + x * 16 + g, w0 + t + 4);
                  af[3] = lds32(Ap, wm + x * 16 + g + 8, w0 + t + 4);
#pragma unroll
                  for(int y = 0; y < 2; y++) {
                    // select the level accumulator without dynamic register indexing
#pragma unroll
                    for(int ll = 0; ll < OZ_LEVELS; ll++)
                      if(ll == l) mma_k(acc[ll][x][y], af, bf[y]);
                  }
                }
              }
            }
          }
        }
        // fold this window's levels into the float-float output (exact power-of-two scaling)
#pragma unroll
        for(int ll = 0; ll < OZ_LEVELS; ll++) {
          const int lev = lvl0 + ll;
          if(lev > S + 1) break;
#pragma unroll
          for(int x = 0; x < 2; x++)
#pragma unroll
            for(int y = 0; y < 2; y++)
#pragma unroll
              for(int z = 0; z < 4; z++) {
                const int   h = z >> 1, e = z & 1;
                const float sc = ldexpf(T_.sign, ea[x][h] + eb[y][e] - OZ_BITS * lev);
                out[x][y][z]   = ff_add_f(out[x][y][z], (float) acc[ll][x][y][z] * sc);
              }
        }
      }
    }
  }
  // C (+)= out
#pragma unroll
  for(int x = 0; x < 2; x++)
#pragma unroll
    for(int y = 0; y < 2; y++)
#pragma unroll
      for(int z = 0; z < 4; z++) {
        const int       h = z >> 1, e = z & 1;
        const long long m = m0 + wm + x * 16 + g + h * 8, n = n0 + wn + y * 8 + 2 * t + e;
        if(m >= J.M || n >= J.N) continue;
        float2* cp = J.C + m * J.N + n;
        ff      r  = out[x][y][z];
        if(J.accumulate) {
          float2 old = *cp;
          r          = ff_add(r, ff{old.x, old.y});
        }
        *cp = make_float2(r.hi, r.lo);
      }
}

__global__ void to_float_kernel(const double* x, float* y, long long n) {
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long) gridDim.x * blockDim.x)
    y[e] = (float) x[e];
}

int multiplicity(int i, int j, int k) {
  if(i == j && j == k) return 1;
  if(i == j || j == k || i == k) return 3;
  return 6;
}

template<typename T>
size_t oz_smem(int S) {
  return (size_t) S * (OZ_BM + OZ_BN) * 80;
}

} // namespace

// ------------------------------------------------------------------------------------ host
ccsdt_status ccsdt_handle::ensure_slices(int S, int variant) {
  if(S < 1 || S > OZ_MAX_SLICES) return fail(CCSDT_E_INVALID, "slices must be in 1..8");
  if(slices_ready >= S && slice_variant == variant) return CCSDT_OK;
  const long long o = this->o, v = this->v;
  const size_t    esz = variant == 0 ? 2 : 1;
  const int       kc  = 64; // TMA box width of the tcgen05 path; the mma.sync path steps 32 / 64
  const int       Kpv = (int) ((v + kc - 1) / kc * kc), Kpo = (int) ((o + kc - 1) / kc * kc);
  // drop old planes (only what this function allocates below; persistent buffers stay)
  cudaError_t se = cudaStreamSynchronize(stream);
  if(se != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(se));
  for(void* p: slice_bufs) cudaFree(p);
  slice_bufs.clear();
  sl_t2 = sl_t2h = sl_ovvv = sl_ooovh = nullptr;
  ex_t2 = ex_t2h = ex_ovvv = ex_ooovh = nullptr;
  oovv_f = t1_f = nullptr;
  F12 = F34 = F56 = nullptr;
  e_tiles = nullptr;
  slices_ready = 0;
  tmaps_ready  = false;
  auto grab = [&](void** p, size_t bytes) -> ccsdt_status {
    cudaError_t e = ccsdt::dev_malloc(p, bytes ? bytes : 1);
    if(e != cudaSuccess) {
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "slice planes: cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    slice_bufs.push_back(*p);
    return CCSDT_OK;
  };
  struct Src {
    const double* x;
    long long     R;
    int           K, Kp;
    void**        planes;
    int**         exps;
    long long*    plane;
  } src[4] = {{t2, o * o * v, (int) v, Kpv, &sl_t2, &ex_t2, &pl_t2},
              {t2h, o * v * v, (int) o, Kpo, &sl_t2h, &ex_t2h, &pl_t2h},
              {ovvv, ovvv_nslab * v * v, (int) v, Kpv, &sl_ovvv, &ex_ovvv, &pl_ovvv}, // slots in the direct mode
              {ooovh, o * o * v, (int) o, Kpo, &sl_ooovh, &ex_ooovh, &pl_ooovh}};
  ccsdt_status s;
  for(auto& q: src) {
    *q.plane = q.R * q.Kp;
    if((s = grab(q.planes, (size_t) S * q.R * q.Kp * esz)) || (s = grab((void**) q.exps, (size_t) q.R * sizeof(int))))
      return s;
    if(ovvv_direct && q.planes == &sl_ovvv) { // its slabs are sliced as they are formed (ensure_ovvv)
      std::fill(slab_sliced.begin(), slab_sliced.end(), 0);
      continue;
    }
    if(variant == 0)
      oz_slice_rows_kernel<__nv_bfloat16><<<4096, 256, 0, stream>>>(q.x, q.R, q.K, q.Kp, S, (__nv_bfloat16*) *q.planes,
                                                                     *q.plane, *q.exps, q.K);
    else
      oz_slice_rows_kernel<int8_t><<<4096, 256, 0, stream>>>(q.x, q.R, q.K, q.Kp, S, (int8_t*) *q.planes, *q.plane,
                                                             *q.exps, q.K);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("slicing: ") + cudaGetErrorString(e));
  }
  kp_v = Kpv;
  kp_o = Kpo;
  // FP32 copies for the energy's singles terms; ff scratch
  if((s = grab((void**) &oovv_f, (size_t) o * o * v * v * sizeof(float))) ||
     (s = grab((void**) &t1_f, (size_t) o * v * sizeof(float))) ||
     (s = grab((void**) &F12, (size_t) v * v * v * sizeof(float2))) ||
     (s = grab((void**) &F34, (size_t) v * v * v * sizeof(float2))) ||
     (s = grab((void**) &F56, (size_t) v * v * v * sizeof(float2))))
    return s;
  to_float_kernel<<<2048, 256, 0, stream>>>(oovv, oovv_f, o * o * v * v);
  to_float_kernel<<<64, 256, 0, stream>>>(t1, t1_f, o * v);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("to_float: ") + cudaGetErrorString(e));
  // energy work items: sorted triples of 8-wide virtual blocks
  {
    const int        nb = (int) ((v + ET_B - 1) / ET_B);
    std::vector<int> host;
    for(int X = 0; X < nb; X++)
      for(int Y = X; Y < nb; Y++)
        for(int Z = Y; Z < nb; Z++) {
          host.push_back(X);
          host.push_back(Y);
          host.push_back(Z);
        }
    e_ntiles = (int) (host.size() / 3);
    if((s = grab((void**) &e_tiles, host.size() * sizeof(int)))) return s;
    if(!e_part) {
      cudaError_t ce = ccsdt::dev_malloc((void**) &e_part, 6 * sizeof(double) * kTiledBlocks);
      if(ce != cudaSuccess) {
        e_part = nullptr;
        cudaGetLastError();
        return fail(CCSDT_E_OOM, "tiled energy partials: cudaMalloc failed");
      }
      owned_bytes.push_back(e_part);
    }
    cudaError_t ce = cudaMemcpyAsync(e_tiles, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    if(ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
    if(ce != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(ce));
  }
  if(!d_err) { // persistent: survives re-slicing
    cudaError_t ce = ccsdt::dev_malloc((void**) &d_err, sizeof(int));
    if(ce != cudaSuccess) {
      d_err = nullptr;
      cudaGetLastError();
      return fail(CCSDT_E_OOM, "error flag: cudaMalloc failed");
    }
    owned_bytes.push_back(d_err);
  }
  slices_ready  = S;
  slice_variant = variant;
  tmaps_ready   = false;
  slice_gen++;
  return CCSDT_OK;
}

namespace {

enum {
  MAP_OVVV_NAT = 0, MAP_OVVV_SWP = 1, MAP_T2 = 2, MAP_T2H_NAT = 3, MAP_T2H_SWP = 4, MAP_OOOVH = 5,
  // the persistent kernel's l-sum runs with the single index on the tile rows: ooovh as the
  // 128-row A operand, t2h pair rows as the NT-row B operand
  MAP_T2H_NAT_B = 6, MAP_T2H_SWP_B = 7, MAP_OOOVH_A = 8
};

// tcgen05 configurations: digit planes S -> columns per level NT (S NT <= 256, (S + 2) NT <= 512)
template<int S>
struct TcPick;
template<>
struct TcPick<1> {
  static constexpr int NT = 128, ST = 4;
};
template<>
struct TcPick<2> {
  static constexpr int NT = 128, ST = 3;
};
template<>
struct TcPick<3> {
  static constexpr int NT = 80, ST = 2;
};
template<>
struct TcPick<4> {
  static constexpr int NT = 64, ST = 2;
};
template<>
struct TcPick<5> {
  static constexpr int NT = 48, ST = 2;
};
int tc_nt(int S) {
  switch(S) {
    case 1: return TcPick<1>::NT;
    case 2: return TcPick<2>::NT;
    case 3: return TcPick<3>::NT;
    case 4: return TcPick<4>::NT;
    case 5: return TcPick<5>::NT;
  }
  return 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so that the library
// itself does not link libcuda (it must load on machines without a driver).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if(!fn) {
    void*                           p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
       q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// 5-D BF16 map: dims (k, d1, d2, d3, plane), strides in elements for d1..d3 and plane.
// kc: the box's K extent, 64 (128-byte rows, 128-byte swizzle) or 32 (64-byte rows, 64-byte swizzle)
bool encode_map(CUtensorMap* m, const void* base, int Kp, long long d1, long long d2, long long d3, int planes,
                long long s1, long long s2, long long s3, long long sp, int box1, int boxp, int kc) {
  if(boxp > planes || (kc != 64 && kc != 32) || Kp % kc) return false;
  cuuint64_t dims[5]    = {(cuuint64_t) Kp, (cuuint64_t) d1, (cuuint64_t) d2, (cuuint64_t) d3, (cuuint64_t) planes};
  cuuint64_t strides[4] = {(cuuint64_t) s1 * 2, (cuuint64_t) s2 * 2, (cuuint64_t) s3 * 2, (cuuint64_t) sp * 2};
  cuuint32_t box[5]     = {(cuuint32_t) kc, (cuuint32_t) box1, 1, 1, (cuuint32_t) boxp};
  cuuint32_t estr[5]    = {1, 1, 1, 1, 1};
  auto fn = encode_fn();
  if(!fn) return false;
  CUresult   r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides,
                                        box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                        kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

} // namespace

// TMA map over the batch scratch's partial arrays: dims (v, v, v, 3 bt_B) of FP32 or float-float
// (8-byte) elements, box 8 x 8 x 8 x 1, zero fill outside.  The row pitch must be a multiple of 16
// bytes; out-of-range box elements are filled with zeros.
bool ccsdt_handle::ensure_pmap(bool f32) {
  if(!bt_F || bt_B <= 0 || v < ET_B) return false;
  const long long es = f32 ? 4 : 8, vv = v;
  if((vv * es) % 16) return false;
  if(pmap_base == bt_F && pmap_B == bt_B && pmap_f32 == (int) f32) return true;
  pmap_base      = nullptr;
  auto fn        = encode_fn();
  if(!fn) return false;
  cuuint64_t dims[4]    = {(cuuint64_t) vv, (cuuint64_t) vv, (cuuint64_t) vv, (cuuint64_t) 3 * bt_B};
  cuuint64_t strides[3] = {(cuuint64_t) (vv * es), (cuuint64_t) (vv * vv * es), (cuuint64_t) (vv * vv * vv * es)};
  cuuint32_t box[4]     = {ET_B, ET_B, ET_B, 1};
  cuuint32_t estr[4]    = {1, 1, 1, 1};
  CUresult   r = fn(&pmap, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, bt_F, dims,
                    strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if(r != CUDA_SUCCESS) return false;
  pmap_base = bt_F, pmap_B = bt_B, pmap_f32 = (int) f32;
  return true;
}

// Tensor maps for S planes whose B-side box is NT rows of KC elements: NT and KC must equal the
// N tile and K chunk of the kernel that will use them (its shared-memory B slot holds exactly
// S x NT rows of 2 KC bytes).
ccsdt_status ccsdt_handle::ensure_tmaps(int S, int NT, int KC) {
  if(tmaps_ready && tmaps_S == S && tmaps_NT == NT && tmaps_KC == KC) return CCSDT_OK;
  if(S > slices_ready) return fail(CCSDT_E_STATE, "tensor maps asked for more planes than were sliced");
  if(NT <= 0 || NT > 256 || NT % 16) return fail(CCSDT_E_INVALID, "bad N tile for the tensor maps");
  const long long o = this->o, v = this->v, S_ = S;
  const int       P = slices_ready; // stored planes (extent); the box loads the first S
  const long long Kv = kp_v, Ko = kp_o;
  bool ok = true;
  // A side (pair rows, 128-row boxes): rows (z, x, y) natural = z v^2 + x v + y, swapped = z v^2 + y v + x
  // ovvv's occupied dimension: its slots in the direct mode (the kernel maps index -> slot)
  ok &= encode_map(&tmaps[MAP_OVVV_NAT], sl_ovvv, (int) Kv, v, v, ovvv_nslab, P, Kv, v * Kv, v * v * Kv, pl_ovvv, TC_BM,
                   (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_OVVV_SWP], sl_ovvv, (int) Kv, v, v, ovvv_nslab, P, v * Kv, Kv, v * v * Kv, pl_ovvv, TC_BM,
                   (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_T2H_NAT], sl_t2h, (int) Ko, v, v, o, P, Ko, v * Ko, v * v * Ko, pl_t2h, TC_BM, (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_T2H_SWP], sl_t2h, (int) Ko, v, v, o, P, v * Ko, Ko, v * v * Ko, pl_t2h, TC_BM, (int) S_, KC);
  // B side (single rows, NT-row boxes): t2 rows (xx, yy, a); ooovh rows (yy, zz, c)
  ok &= encode_map(&tmaps[MAP_T2], sl_t2, (int) Kv, v, o, o, P, Kv, v * Kv, o * v * Kv, pl_t2, NT, (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_OOOVH], sl_ooovh, (int) Ko, v, o, o, P, Ko, v * Ko, o * v * Ko, pl_ooovh, NT, (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_T2H_NAT_B], sl_t2h, (int) Ko, v, v, o, P, Ko, v * Ko, v * v * Ko, pl_t2h, NT, (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_T2H_SWP_B], sl_t2h, (int) Ko, v, v, o, P, v * Ko, Ko, v * v * Ko, pl_t2h, NT, (int) S_, KC);
  ok &= encode_map(&tmaps[MAP_OOOVH_A], sl_ooovh, (int) Ko, v, o, o, P, Ko, v * Ko, o * v * Ko, pl_ooovh, TC_BM, (int) S_, KC);
  if(!ok) return fail(CCSDT_E_CUDA, "cuTensorMapEncodeTiled failed for the digit planes");
  tmaps_ready = true;
  tmaps_S     = S;
  tmaps_NT    = NT;
  tmaps_KC    = KC;
  return CCSDT_OK;
}

template<int S>
static ccsdt_status launch_tc(ccsdt_handle* h, TcBatch& b) {
  constexpr int NT = TcPick<S>::NT, ST = TcPick<S>::ST;
  if(!h->tmaps_ready || h->tmaps_S != S || h->tmaps_NT != NT || h->tmaps_KC != 64)
    return h->fail(CCSDT_E_STATE, "tensor maps do not match the tcgen05 kernel's tile");
  using Cfg        = TcCfg<S, NT, ST>;
  const int    v   = h->v;
  const long long tiles = (long long) v * ((v + TC_BM - 1) / TC_BM) * ((v + NT - 1) / NT);
  cudaError_t e = cudaFuncSetAttribute(oz_tc_gemm_kernel<S, NT, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("tc smem attr: ") + cudaGetErrorString(e));
  oz_tc_gemm_kernel<S, NT, ST><<<dim3((unsigned) tiles, 1, 3), TC_THREADS, Cfg::SMEM, h->stream>>>(b);
  h->launches++;
  e = cudaGetLastError();
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("tc launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

static ccsdt_status launch_tc_any(ccsdt_handle* h, TcBatch& b, int S) {
  switch(S) {
    case 1: return launch_tc<1>(h, b);
    case 2: return launch_tc<2>(h, b);
    case 3: return launch_tc<3>(h, b);
    case 4: return launch_tc<4>(h, b);
    case 5: return launch_tc<5>(h, b);
  }
  return h->fail(CCSDT_E_INVALID, "no tcgen05 configuration for this slice count");
}

bool ccsdt_handle::tc_eligible(int S, int variant) const {
  return variant == 0 && S >= 1 && S <= 5 && kp_v <= 512 && kp_o <= 512 && !force_mma_sync;
}
// the persistent tcgen05 path: BF16 digits, 1..8 planes, any contraction length (exact K windows)
bool ccsdt_handle::pz_eligible(int S, int variant) const {
  return variant == 0 && S >= 1 && S <= OZ_MAX_SLICES && !force_mma_sync;
}

ccsdt_status ccsdt_handle::run_triplet_tc(int i, int j, int k, int S, double* eout) {
  ccsdt_status s;
  if((s = ensure_tmaps(S, tc_nt(S), 64))) return s;
  const long long v = this->v, v2 = v * v;
  // BF16 digit planes carry their rows' scales: no exponent tables
  auto hole = [&](int xx, bool nat, int yy, int zz) {
    return TcTerm{nat ? MAP_T2H_NAT : MAP_T2H_SWP, MAP_OOOVH, xx, zz, yy, nullptr, nat ? v : 1, nat ? 1 : v,
                  xx * v2, nullptr, kp_o, -1.f};
  };
  auto part = [&](int z, bool nat, int xx, int yy) {
    return TcTerm{nat ? MAP_OVVV_NAT : MAP_OVVV_SWP, MAP_T2, z, yy, xx, nullptr, nat ? v : 1, nat ? 1 : v,
                  z * v2, nullptr, kp_v, 1.f};
  };
  TcBatch b;
  std::memcpy(b.maps, tmaps, sizeof(b.maps)); // the first six maps
  b.v       = (int) v;
  b.xblocks = (int) v;
  b.err     = d_err;
  b.tail    = cur_tail;
  // l-sum: F[(pair)][single], pairs (a,c) / (b,a) / (c,b)
  b.job[0] = TcJob{{hole(i, true, k, j), hole(k, false, i, j)}, 2, F12, v, 1, 0};
  b.job[1] = TcJob{{hole(i, false, j, k), hole(j, true, i, k)}, 2, F34, v, 1, 0};
  b.job[2] = TcJob{{hole(j, false, k, i), hole(k, true, j, i)}, 2, F56, v, 1, 0};
  if(profiling) cudaEventRecord(prof_ev[0], stream);
  if((s = launch_tc_any(this, b, S))) return s;
  // d-sum: F[single][(pair)], pairs (c,b) / (a,c) / (b,a)
  b.job[0] = TcJob{{part(k, true, i, j), part(j, false, i, k)}, 2, F12, 1, v2, 1};
  b.job[1] = TcJob{{part(k, false, j, i), part(i, true, j, k)}, 2, F34, 1, v2, 1};
  b.job[2] = TcJob{{part(j, true, k, i), part(i, false, k, j)}, 2, F56, 1, v2, 1};
  if(profiling) cudaEventRecord(prof_ev[1], stream);
  if((s = launch_tc_any(this, b, S))) return s;
  if(profiling) cudaEventRecord(prof_ev[2], stream);
  if((s = launch_energy_tiled(i, j, k, eout))) return s;
  if(profiling) cudaEventRecord(prof_ev[4], stream);
  launches += 2;
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("tc energy launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

template<typename T>
static ccsdt_status launch_oz(ccsdt_handle* h, const OzBatch& b, long long M, long long N) {
  const long long tiles = ((M + OZ_BM - 1) / OZ_BM) * ((N + OZ_BN - 1) / OZ_BN);
  const size_t    sm    = oz_smem<T>(b.S);
  cudaError_t     e     = cudaFuncSetAttribute(oz_gemm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("smem attr: ") + cudaGetErrorString(e));
  oz_gemm_kernel<T><<<dim3((unsigned) tiles, 1, 3), OZ_THREADS, sm, h->stream>>>(b);
  h->launches++;
  e = cudaGetLastError();
  if(e != cudaSuccess) return h->fail(CCSDT_E_CUDA, std::string("oz_gemm launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

// BF16-digit Ozaki GEMMs of up to three jobs (grid z = njobs) on `st`, for translation units
// without the kernel (the open-shell split path)
cudaError_t ccsdt::oz_gemm_bf16(const OzBatch& b, int njobs, long long max_tiles, cudaStream_t st) {
  if(njobs < 1 || njobs > 3 || max_tiles <= 0 || max_tiles >= (1LL << 31)) return cudaErrorInvalidValue;
  const size_t sm = oz_smem<__nv_bfloat16>(b.S);
  cudaError_t  e  = cudaFuncSetAttribute(oz_gemm_kernel<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int) sm);
  if(e != cudaSuccess) return e;
  oz_gemm_kernel<__nv_bfloat16><<<dim3((unsigned) max_tiles, 1, (unsigned) njobs), OZ_THREADS, sm, st>>>(b);
  return cudaGetLastError();
}
long long ccsdt::oz_gemm_tiles(long long M, long long N) { return ((M + OZ_BM - 1) / OZ_BM) * ((N + OZ_BN - 1) / OZ_BN); }

ccsdt_status ccsdt_handle::run_triplet_split(int i, int j, int k, int S, int variant, double* eout) {
  const long long o = this->o, v = this->v, v2 = v * v;
  const size_t    esz = variant == 0 ? 2 : 1;
  auto at = [&](const void* base, long long elems) { return (const void*) ((const char*) base + elems * esz); };
  // l-sum: rows of t2h are (x, (a, b)), rows of ooovh are (y, z, c)
  // BF16 digit planes carry their rows' scales (no exponent tables); INT8 digits do not
  const bool int8 = variant != 0;
  auto t2h_t = [&](int x, OzRows m) {
    return std::make_tuple(at(sl_t2h, (long long) x * v2 * kp_o), int8 ? ex_t2h + (long long) x * v2 : nullptr, m);
  };
  auto ooh_t = [&](int y, int z) {
    return std::make_tuple(at(sl_ooovh, ((long long) y * o + z) * v * kp_o),
                           int8 ? ex_ooovh + ((long long) y * o + z) * v : nullptr);
  };
  auto hole = [&](int xa, OzRows ma, int yb, int zb) {
    auto [A, eA, mA] = t2h_t(xa, ma);
    auto [B, eB]     = ooh_t(yb, zb);
    return OzTerm{A, eA, mA, pl_t2h, B, eB, oz_plain(), pl_ooovh, kp_o, -1.f};
  };
  const OzRows nat = oz_plain(), swp = oz_swapped((int) v);
  OzBatch      hb{};
  hb.S      = S;
  hb.job[0] = OzJob{{hole(i, nat, k, j), hole(k, swp, i, j)}, 2, F12, v2, v, 0};
  hb.job[1] = OzJob{{hole(i, swp, j, k), hole(j, nat, i, k)}, 2, F34, v2, v, 0};
  hb.job[2] = OzJob{{hole(j, swp, k, i), hole(k, nat, j, i)}, 2, F56, v2, v, 0};
  ccsdt_status s;
  if(profiling) cudaEventRecord(prof_ev[0], stream);
  if((s = variant == 0 ? launch_oz<__nv_bfloat16>(this, hb, v2, v) : launch_oz<int8_t>(this, hb, v2, v))) return s;
  // d-sum: rows of t2 are (x, y, a), rows of ovvv are (z, c, b)
  auto part_t = [&](int x, int y, int z, OzRows mb) {
    const long long ra = ((long long) x * o + y) * v, rb = (long long) z * v2;
    return OzTerm{at(sl_t2, ra * kp_v), int8 ? ex_t2 + ra : nullptr, nat, pl_t2, at(sl_ovvv, rb * kp_v),
                  int8 ? ex_ovvv + rb : nullptr, mb, pl_ovvv, kp_v, 1.f};
  };
  OzBatch pb{};
  pb.S      = S;
  pb.job[0] = OzJob{{part_t(i, j, k, nat), part_t(i, k, j, swp)}, 2, F12, v, v2, 1};
  pb.job[1] = OzJob{{part_t(j, i, k, swp), part_t(j, k, i, nat)}, 2, F34, v, v2, 1};
  pb.job[2] = OzJob{{part_t(k, i, j, nat), part_t(k, j, i, swp)}, 2, F56, v, v2, 1};
  if(profiling) cudaEventRecord(prof_ev[1], stream);
  if((s = variant == 0 ? launch_oz<__nv_bfloat16>(this, pb, v, v2) : launch_oz<int8_t>(this, pb, v, v2))) return s;
  if(profiling) cudaEventRecord(prof_ev[2], stream);
  if((s = launch_energy_tiled(i, j, k, eout))) return s;
  if(profiling) cudaEventRecord(prof_ev[4], stream);
  launches += 2;
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("split launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::run_split(const ccsdt_opts* opts, long n, const int* tri) {
  last_batched     = false;
  last_err_bound   = 0.0; // only the LEARNED mode estimates its error
  if(opts->mode == CCSDT_MODE_LEARNED) {
    if(ovvv_direct) // its features read every occupied index's (ia|bc) exponent statistics
      return fail(CCSDT_E_INVALID, "the learned slice count needs the whole (ia|bc); not in the Cholesky-direct mode");
    return run_learned(opts, n, tri);
  }
  const int S       = opts->slices;
  const int variant = opts->slice_kind;
  if(variant != 0 && variant != 1) return fail(CCSDT_E_INVALID, "unknown slice variant");
  if(v > OZ_KWIN * 64) return fail(CCSDT_E_INVALID, "v too large for the split path");
  ccsdt_status s;
  if((s = ensure_slices(S, variant))) return s;
  if(!d_err || !F12 || !F34 || !F56 || !e_tiles || !e_part || !oovv_f || !t1_f)
    return fail(CCSDT_E_STATE, "split-precision buffers missing after slicing");
  // test knob opts->test_kernel: 0 persistent tcgen05 (default), 1 mma.sync slice kernel,
  // 2 per-triplet (non-persistent) tcgen05 kernel
  const int kernel_kind = opts->test_kernel;
  force_mma_sync        = kernel_kind == 1;
  cudaError_t e0 = cudaMemsetAsync(d_err, 0, sizeof(int), stream);
  if(e0 != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(e0));
  if(kernel_kind == 3) { // testing: FP64 contractions with the float-float energy (its own error)
    if((s = ensure_scratch())) return s;
    fp64_ff_energy = true;
    s              = run_fp64_list(n, tri);
    fp64_ff_energy = false;
    return s;
  }
  last_batched = kernel_kind == 0 && pz_eligible(S, variant);
  if(ovvv_direct && !last_batched)
    return fail(CCSDT_E_INVALID, "the Cholesky-direct mode runs the split path on the persistent tcgen05 kernel only "
                                 "(BF16 digits, default test_kernel)");
  if(last_batched) return run_batched(S, n, tri, opts->use_graph != 0, nullptr, nullptr);
  for(long t = 0; t < n; t++) {
    const int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    if(i == k) {
      cudaError_t e = cudaMemsetAsync(etrip + 2 * t, 0, 2 * sizeof(double), stream);
      if(e != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(e));
      continue;
    }
    if(tc_eligible(S, variant)) {
      if((s = run_triplet_tc(i, j, k, S, etrip + 2 * t))) return s;
    } else if((s = run_triplet_split(i, j, k, S, variant, etrip + 2 * t)))
      return s;
  }
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::check_device_error() {
  if(!d_err) return fail(CCSDT_E_STATE, "device error flag missing");
  int         flag = 0;
  cudaError_t e    = cudaMemcpyAsync(&flag, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  if(e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, cudaGetErrorString(e));
  if(flag) return fail(CCSDT_E_TIMEOUT, "a bounded device-side wait of the tcgen05 contraction gave up");
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::launch_energy_tiled(int i, int j, int k, double* eout, bool f32) {
  const int       G = std::min(e_ntiles, energy_grid(f32));
  TiledEnergyArgs ea{F12, F34, F56, oovv_f, t1_f, eo, ev, (const int3*) e_tiles, e_ntiles, o, v, i, j, k, e_part,
                     cur_sens != nullptr};
  if(f32) energy_tiled_kernel<float><<<G, ET_THREADS, 0, stream>>>(ea);
  else energy_tiled_kernel<float2><<<G, ET_THREADS, 0, stream>>>(ea);
  if(profiling) cudaEventRecord(prof_ev[3], stream);
  reduce_parts_parallel_kernel<<<1, 256, 0, stream>>>(e_part, G, multiplicity(i, j, k) / 9.0, eout, cur_sens);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return fail(CCSDT_E_CUDA, std::string("tiled energy launch: ") + cudaGetErrorString(e));
  return CCSDT_OK;
}

ccsdt_status ccsdt_handle::run_triplet_S(int i, int j, int k, int S, double* eout) {
  if(tc_eligible(S, 0)) return run_triplet_tc(i, j, k, S, eout);
  return run_triplet_split(i, j, k, S, 0, eout);
}
