// Split-precision contraction on the 5th-generation tensor cores (tcgen05 + TMA).
//
//   D[m][n] (+)= sum_terms sign_t 2^{eA_t(m) + eB_t(n)} sum_{l=2..S+1} 2^{-7 l} L_{t,l}[m][n]
//   L_{t,l}    = sum_{p+q=l} sum_k A_{t,p}[m,k] B_{t,q}[n,k]          (exact in FP32, K <= 512)
//
// m runs over pair rows (x, y) of the A operand: m = x * v + y, y in [0, v); n over the v
// rows of the B operand.  One CTA owns a 128 (m: fixed x, y0 .. y0+127) x NT (n) tile.
//
// Level trick: the S digit planes of one B tile sit next to each other in shared memory, so
// for A plane p a single MMA with N = (S+1-p) NT against planes 1..S+1-p of B writes the
// products (p, q) into TMEM column blocks p+q-2, i.e. every level l has its own FP32
// accumulator block, and a K-step costs S MMAs instead of S(S+1)/2.
//
// Warp roles (192 threads): warp 0 lane 0 issues the TMA loads, warp 1 lane 0 issues the
// MMAs, warps 2-5 (128 threads, one TMEM lane each) fold the levels into a float-float
// accumulator that also lives in TMEM, and write D at the end.
#pragma once

#include <cuda.h>

#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace ccsdt {

constexpr int TC_BM = 128, TC_KC = 64, TC_THREADS = 192;

struct TcTerm {
  int        mapA, mapB;         // indices into TcBatch::maps
  int        az;                 // A coordinate of the slab (dim 3); dims 1, 2 are the tile's (y, x)
  int        by, bx;             // B coordinates of the single rows (dims 2, 3 of map B)
  const int* eA;                 // exponent of A row: eA[rid] (nullptr: the digits carry it)
  long long  eA_x, eA_y;         // rid = eA_base + x * eA_x + y * eA_y
  long long  eA_base;
  const int* eB;                 // exponent of B row n: eB[n] (nullptr: the digits carry it)
  int        Kp;                 // contraction length (multiple of 64, <= 512)
  float      sign;
};

struct TcJob {
  TcTerm    t[2];
  int       nterms;
  float2*   C;       // D element (m, n) at C[m * csm + n * csn]
  long long csm, csn;
  int       accumulate;
};

struct TcBatch {
  CUtensorMap maps[6];
  TcJob       job[3];
  int         v;        // pair rows per x and single rows
  int         xblocks;  // x values (= v)
  int*        err;      // device error flag (set on a wait timeout)
  float*      tail;     // optional: += sum of squares of the last kept level's terms (a-posteriori estimate)
};

template<int S, int NT, int STAGES>
struct TcCfg {
  static constexpr int A_BYTES     = S * TC_BM * 128;       // S planes x 128 rows x 128 B
  static constexpr int B_BYTES     = S * NT * 128;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM        = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr int LVL_COLS    = S * NT;
  static constexpr int ACC_HI      = LVL_COLS, ACC_LO = LVL_COLS + NT;
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert((S + 2) * NT <= 512, "TMEM budget");
  static_assert(S * NT <= 256 && NT % 16 == 0, "MMA N limit");
};

template<int S, int NT, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1) oz_tc_gemm_kernel(const __grid_constant__ TcBatch P) {
  using C = TcCfg<S, NT, STAGES>;
  const TcJob& J = P.job[blockIdx.z];
  const int    v = P.v;
  const int    yblocks = (v + TC_BM - 1) / TC_BM, nblocks = (v + NT - 1) / NT;
  const int    tile = blockIdx.x;
  const int    nb = tile % nblocks, rest = tile / nblocks;
  const int    yb = rest % yblocks, x = rest / yblocks;
  if(x >= P.xblocks) return;
  const int y0 = yb * TC_BM, n0 = nb * NT;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full  = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* mma_done = empty + STAGES;   // MMAs of a term finished -> epilogue may read
  uint64_t* tmem_free = mma_done + 1;    // epilogue finished reading levels
  uint64_t* drain = tmem_free + 1;       // every MMA issued by this CTA has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if(threadIdx.x == 0) {
    for(int s = 0; s < STAGES; s++) {
      sm100::mbar_init(&full[s], 1);
      sm100::mbar_init(&empty[s], 1);
    }
    sm100::mbar_init(mma_done, 1);
    sm100::mbar_init(tmem_free, 128);
    sm100::mbar_init(drain, 1);
    *abort_flag = 0;
    sm100::mbar_fence_init();
  }
  if(warp == 1) {
    sm100::tmem_alloc(tmem_slot, C::TMEM_COLS);
    sm100::tmem_relinquish();
  }
  sm100::tc_fence_before();
  __syncthreads();
  sm100::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto fail = [&]() {
    *abort_flag = 1;
    if(P.err) atomicExch(P.err, 1);
  };

  if(warp == 0) {
    // ------------------------------------------------------------------ TMA producer
    if(lane == 0) {
      for(int m = 0; m < 6; m++) sm100::prefetch_tmap(&P.maps[m]);
      int it = 0;
      for(int t = 0; t < J.nterms && !*abort_flag; t++) {
        const TcTerm& T = J.t[t];
        for(int k0 = 0; k0 < T.Kp; k0 += TC_KC, it++) {
          const int s = it % STAGES, use = it / STAGES;
          if(use > 0 && !sm100::mbar_wait(&empty[s], (use - 1) & 1)) {
            fail();
            break;
          }
          unsigned char* a = smem + s * C::STAGE_BYTES;
          unsigned char* b = a + C::A_BYTES;
          sm100::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
          sm100::tma_load_5d(a, &P.maps[T.mapA], &full[s], k0, y0, x, T.az, 0);
          sm100::tma_load_5d(b, &P.maps[T.mapB], &full[s], k0, n0, T.by, T.bx, 0);
        }
      }
      // every issued stage must have landed before the CTA may exit (also on abort)
      for(int u = (it > STAGES ? it - STAGES : 0); u < it; u++)
        if(!sm100::mbar_wait(&full[u % STAGES], (u / STAGES) & 1)) fail();
    }
  } else if(warp == 1) {
    // ------------------------------------------------------------------ MMA issuer
    if(lane == 0) {
      int it = 0;
      for(int t = 0; t < J.nterms && !*abort_flag; t++) {
        const TcTerm& T = J.t[t];
        if(t > 0 && !sm100::mbar_wait(tmem_free, (t - 1) & 1)) { // levels drained by the epilogue
          fail();
          break;
        }
        sm100::tc_fence_after();
        for(int k0 = 0; k0 < T.Kp; k0 += TC_KC, it++) {
          const int s = it % STAGES, use = it / STAGES;
          if(!sm100::mbar_wait(&full[s], use & 1)) {
            fail();
            break;
          }
          sm100::tc_fence_after();
          const uint32_t a = sm100::smem_u32(smem + s * C::STAGE_BYTES);
          const uint32_t b = a + C::A_BYTES;
#pragma unroll
          for(int ks = 0; ks < TC_KC / 16; ks++) {
#pragma unroll
            for(int p = 1; p <= S; p++) {
              const uint64_t ad = sm100::desc_kmajor_sw128(a + (p - 1) * TC_BM * 128 + ks * 32);
              const uint64_t bd = sm100::desc_kmajor_sw128(b + ks * 32);
              const uint32_t id = sm100::idesc_bf16_f32(TC_BM, (S + 1 - p) * NT);
              const uint32_t first = (k0 == 0 && ks == 0 && p == 1) ? 0u : 1u;
              sm100::mma_bf16(tmem + (p - 1) * NT, ad, bd, id, first);
            }
          }
          sm100::mma_commit(&empty[s]); // smem stage reusable once these MMAs are done
        }
        sm100::mma_commit(mma_done);    // this term's levels are complete
      }
      // no MMA may still be writing TMEM when it is released (also on abort)
      sm100::mma_commit(drain);
      if(!sm100::mbar_wait(drain, 0)) fail();
    }
  } else {
    // ------------------------------------------------------------------ epilogue (128 threads)
    const int q   = warp & 3;                 // TMEM lane quarter of this warp
    const int row = q * 32 + lane;            // tile row = TMEM lane
    const int y   = y0 + row;
    const bool vrow = y < v;
    const long long m = (long long) x * v + y;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
    float          tsq       = 0.f; // sum of squares of this thread's last-level terms
    for(int t = 0; t < J.nterms; t++) {
      const TcTerm& T = J.t[t];
      // warp-uniform decision: the tcgen05.ld / st below are .sync.aligned
      const bool ok = __all_sync(0xffffffffu, sm100::mbar_wait(mma_done, t & 1) && !*abort_flag);
      if(!ok) {
        fail();
        break;
      }
      sm100::tc_fence_after();
      const int ea = vrow && T.eA ? T.eA[T.eA_base + (long long) x * T.eA_x + (long long) y * T.eA_y] : 0;
      const bool last = (t == J.nterms - 1);
      for(int c0 = 0; c0 < NT; c0 += 16) {
        float hi[16], lo[16];
        int   eb[16];
#pragma unroll
        for(int e = 0; e < 16; e++) eb[e] = (T.eB && n0 + c0 + e < v) ? T.eB[n0 + c0 + e] : 0;
        if(t == 0) {
#pragma unroll
          for(int e = 0; e < 16; e++) hi[e] = lo[e] = 0.f;
        } else {
          uint32_t rh[16], rl[16];
          sm100::tmem_ld16(lane_base + C::ACC_HI + c0, rh);
          sm100::tmem_ld16(lane_base + C::ACC_LO + c0, rl);
          sm100::tmem_wait_ld();
#pragma unroll
          for(int e = 0; e < 16; e++) {
            hi[e] = __uint_as_float(rh[e]);
            lo[e] = __uint_as_float(rl[e]);
          }
        }
        // S exact levels -> float-float (oz_horner), scaled by 2^(e_row + e_col - 7 (S + 1)) (e_row = e_col
        // = 0 for BF16 digits, which carry their row scales)
        uint32_t rv[S][16];
#pragma unroll
        for(int l = 0; l < S; l++) sm100::tmem_ld16(lane_base + l * NT + c0, rv[l]);
        sm100::tmem_wait_ld();
        const float sa = ldexpf(T.sign, ea - OZ_BITS * (S + 1));
#pragma unroll
        for(int e = 0; e < 16; e++) {
          const float sb = ldexpf(1.f, eb[e]);
          const ff    xx = oz_horner<S>(rv, e);
          const ff    a  = ff_add(ff{hi[e], lo[e]}, ff{(xx.hi * sa) * sb, (xx.lo * sa) * sb});
          hi[e]          = a.hi;
          lo[e]          = a.lo;
          if(P.tail) {
            const float tl = (__uint_as_float(rv[S - 1][e]) * sa) * sb;
            tsq            = fmaf(tl, tl, tsq);
          }
        }
        if(!last) {
          uint32_t rh[16], rl[16];
#pragma unroll
          for(int e = 0; e < 16; e++) {
            rh[e] = __float_as_uint(hi[e]);
            rl[e] = __float_as_uint(lo[e]);
          }
          sm100::tmem_st16(lane_base + C::ACC_HI + c0, rh);
          sm100::tmem_st16(lane_base + C::ACC_LO + c0, rl);
          sm100::tmem_wait_st();
        } else if(vrow) {
#pragma unroll
          for(int e = 0; e < 16; e++) {
            const int n = n0 + c0 + e;
            if(n >= v) continue;
            float2* cp = J.C + m * J.csm + (long long) n * J.csn;
            ff r{hi[e], lo[e]};
            if(J.accumulate) {
              const float2 o = *cp;
              r = ff_add(r, ff{o.x, o.y});
            }
            *cp = make_float2(r.hi, r.lo);
          }
        }
      }
      sm100::tc_fence_before();
      sm100::mbar_arrive(tmem_free);
    }
    if(P.tail) {
#pragma unroll
      for(int off = 16; off > 0; off >>= 1) tsq += __shfl_xor_sync(0xffffffffu, tsq, off);
      if(lane == 0 && tsq > 0.f) atomicAdd(P.tail, tsq);
    }
  }
  sm100::tc_fence_before();
  __syncthreads();
  if(warp == 1) {
    sm100::tc_fence_after();
    sm100::tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

} // namespace ccsdt
