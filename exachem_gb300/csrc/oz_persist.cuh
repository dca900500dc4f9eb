// Persistent split-precision contraction: one CTA per SM pulls tiles from a device work queue.
//
// Work item = (triplet slot, job, x, y-block, n-block) of one contraction family (phase 0: the
// l-sum / hole terms, phase 1: the d-sum / particle terms) for a batch of occupied triplets.  The
// host orders the items by estimated cost (tile rows x columns, largest first; ties keep the
// natural order, n-block fastest, so concurrently running CTAs share the A tile in L2) and the
// CTAs take them with atomicAdd on a device counter.  The triplets come from a device table, so
// the launch sequence of a batch is the same for every batch and is replayed from a CUDA graph.
//
// Roles (320 threads): warp 0 lane 0 fetches items and issues TMA loads (running ahead across
// items), warp 1 lane 0 issues the MMAs, warps 2-9 fold the digit levels into float-float.  The
// TMEM level accumulators are double buffered by term, so the fold of one term overlaps the MMAs
// of the next; the float-float accumulator of a tile lives in registers (each epilogue thread owns
// one row and half of the tile's columns).  All waits are bounded (sm100::kSpinLimit).
#pragma once

#include <cuda.h>

#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace ccsdt {

constexpr int PZ_BM = 128, PZ_KC = 64, PZ_THREADS = 320, PZ_IR = 4;
constexpr unsigned PZ_END = 0xffffffffu;

enum { PZ_OVVV_NAT = 0, PZ_OVVV_SWP = 1, PZ_T2 = 2, PZ_T2H_NAT = 3, PZ_T2H_SWP = 4, PZ_OOOVH = 5 };

struct PzParams {
  CUtensorMap     maps[6];
  const int*      tri;        // triplet table (4 ints per triplet: i, j, k, output index)
  const int*      base;       // device batch base index into tri (nullable -> 0)
  int             nslots;     // triplets per launch
  int             phase;      // 0: l-sum, 1: d-sum
  int             o, v, kp_v, kp_o;
  float2*         F;          // P arrays of slot s: F + s * 3 v^3 (P12, P34, P56 consecutive)
  const int *     ex_t2, *ex_t2h, *ex_ovvv, *ex_ooovh;
  const unsigned* order;      // cost-ordered item ids, length nitems
  unsigned        nitems;
  unsigned*       queue;      // work counter, 0 at launch
  int*            err;        // set on a bounded-wait timeout
  float*          tail;       // optional: tail[output index] = max |last kept level term|
};

struct PzTerm {
  int       mapA, mapB, az, by, bx, Kp;
  const int *eA, *eB;
  long long eA_base, eA_x, eA_y;
  float     sign;
};

// The two terms of a job, from (phase, job, i, j, k) - the same plan as the host-side batches:
// l-sum  P12[(a,c)][b]: t2h(i) nat x ooovh(k,j), t2h(k) swp x ooovh(i,j)   (P34, P56 likewise)
// d-sum  P12[a][(c,b)]: ovvv(k) nat x t2(i,j),  ovvv(j) swp x t2(i,k)     (P34, P56 likewise)
__device__ __forceinline__ PzTerm pz_term(const PzParams& P, int job, int t, int i, int j, int k) {
  const long long v = P.v, o = P.o, v2 = v * v;
  // l-sum jobs: (first, natural?, second, third) of term 0 / term 1
  //   job 0: (i,1,k,j) (k,0,i,j)   job 1: (i,0,j,k) (j,1,i,k)   job 2: (j,0,k,i) (k,1,j,i)
  // d-sum jobs:
  //   job 0: (k,1,i,j) (j,0,i,k)   job 1: (k,0,j,i) (i,1,j,k)   job 2: (j,1,k,i) (i,0,k,j)
  const int sel = job * 2 + t;
  int       e0, nat, e2, e3;
  if(P.phase == 0) {
    switch(sel) {
      case 0: e0 = i, nat = 1, e2 = k, e3 = j; break;
      case 1: e0 = k, nat = 0, e2 = i, e3 = j; break;
      case 2: e0 = i, nat = 0, e2 = j, e3 = k; break;
      case 3: e0 = j, nat = 1, e2 = i, e3 = k; break;
      case 4: e0 = j, nat = 0, e2 = k, e3 = i; break;
      default: e0 = k, nat = 1, e2 = j, e3 = i; break;
    }
  } else {
    switch(sel) {
      case 0: e0 = k, nat = 1, e2 = i, e3 = j; break;
      case 1: e0 = j, nat = 0, e2 = i, e3 = k; break;
      case 2: e0 = k, nat = 0, e2 = j, e3 = i; break;
      case 3: e0 = i, nat = 1, e2 = j, e3 = k; break;
      case 4: e0 = j, nat = 1, e2 = k, e3 = i; break;
      default: e0 = i, nat = 0, e2 = k, e3 = j; break;
    }
  }
  PzTerm T;
  if(P.phase == 0) {
    const int xx = e0, yy = e2, zz = e3;
    T.mapA = nat ? PZ_T2H_NAT : PZ_T2H_SWP;
    T.mapB = PZ_OOOVH;
    T.az = xx, T.by = zz, T.bx = yy, T.Kp = P.kp_o;
    T.eA = P.ex_t2h, T.eA_base = xx * v2, T.eA_x = nat ? v : 1, T.eA_y = nat ? 1 : v;
    T.eB   = P.ex_ooovh + (yy * o + zz) * v;
    T.sign = -1.f;
  } else {
    const int z = e0, xx = e2, yy = e3;
    T.mapA = nat ? PZ_OVVV_NAT : PZ_OVVV_SWP;
    T.mapB = PZ_T2;
    T.az = z, T.by = yy, T.bx = xx, T.Kp = P.kp_v;
    T.eA = P.ex_ovvv, T.eA_base = z * v2, T.eA_x = nat ? v : 1, T.eA_y = nat ? 1 : v;
    T.eB   = P.ex_t2 + (xx * o + yy) * v;
    T.sign = 1.f;
  }
  return T;
}

struct PzItem {
  int slot, job, x, yb, nb;
};
// item id -> fields; ids are dense in (slot, job, x, yb, nb), nb fastest
__device__ __forceinline__ PzItem pz_decode(unsigned id, int v, int yblocks, int nblocks) {
  PzItem it;
  it.nb = id % nblocks;
  id /= nblocks;
  it.yb = id % yblocks;
  id /= yblocks;
  it.x = id % v;
  id /= v;
  it.job  = id % 3;
  it.slot = id / 3;
  return it;
}

template<int S, int NT, int STAGES>
struct PzCfg {
  static constexpr int A_BYTES = S * PZ_BM * 128, B_BYTES = S * NT * 128, STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 512;
  static constexpr int HALF = NT / 2;   // columns per epilogue thread
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert(2 * S * NT <= 512, "two level buffers must fit in TMEM");
  static_assert(S * NT <= 256 && NT % 32 == 0, "MMA N limit / epilogue halves of 16");
};

template<int S, int NT, int STAGES>
__global__ void __launch_bounds__(PZ_THREADS, 1) oz_persist_kernel(const __grid_constant__ PzParams P) {
  using C = PzCfg<S, NT, STAGES>;
  const int v = P.v, yblocks = (v + PZ_BM - 1) / PZ_BM, nblocks = (v + NT - 1) / NT;
  const int base = P.base ? *P.base : 0;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full       = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint64_t* empty      = full + STAGES;
  uint64_t* item_full  = empty + STAGES;
  uint64_t* item_empty = item_full + PZ_IR;
  uint64_t* lvl_full   = item_empty + PZ_IR;   // [2] MMAs of a term done
  uint64_t* lvl_empty  = lvl_full + 2;         // [2] epilogue drained the buffer
  uint64_t* drain      = lvl_empty + 2;
  unsigned* item_id    = reinterpret_cast<unsigned*>(drain + 1);
  uint32_t* tmem_slot  = item_id + PZ_IR;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if(threadIdx.x == 0) {
    for(int s = 0; s < STAGES; s++) {
      sm100::mbar_init(&full[s], 1);
      sm100::mbar_init(&empty[s], 1);
    }
    for(int r = 0; r < PZ_IR; r++) {
      sm100::mbar_init(&item_full[r], 1);
      sm100::mbar_init(&item_empty[r], 1 + 8); // MMA thread + one arrival per epilogue warp
    }
    for(int b = 0; b < 2; b++) {
      sm100::mbar_init(&lvl_full[b], 1);
      sm100::mbar_init(&lvl_empty[b], 8);
    }
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
    // ------------------------------------------------------------ work fetch + TMA producer
    if(lane == 0) {
      for(int m = 0; m < 6; m++) sm100::prefetch_tmap(&P.maps[m]);
      int stage_it = 0;
      for(int it = 0;; it++) {
        const unsigned q  = atomicAdd(P.queue, 1u);
        const unsigned id = (q < P.nitems && !*abort_flag) ? P.order[q] : PZ_END;
        const int      r  = it % PZ_IR;
        if(it >= PZ_IR && !sm100::mbar_wait(&item_empty[r], ((it / PZ_IR) - 1) & 1)) {
          fail();
          item_id[r] = PZ_END;
          sm100::mbar_arrive(&item_full[r]);
          break;
        }
        item_id[r] = id;
        sm100::mbar_arrive(&item_full[r]); // release: the id is visible to waiters
        if(id == PZ_END) break;
        const PzItem w = pz_decode(id, v, yblocks, nblocks);
        const int*   tp = P.tri + 4 * (base + w.slot);
        const int    i = tp[0], j = tp[1], k = tp[2];
        for(int t = 0; t < 2; t++) {
          const PzTerm T = pz_term(P, w.job, t, i, j, k);
          for(int k0 = 0; k0 < T.Kp; k0 += PZ_KC, stage_it++) {
            const int s = stage_it % STAGES, use = stage_it / STAGES;
            if(use > 0 && !sm100::mbar_wait(&empty[s], (use - 1) & 1)) {
              fail();
              break;
            }
            unsigned char* a = smem + s * C::STAGE_BYTES;
            sm100::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
            sm100::tma_load_5d(a, &P.maps[T.mapA], &full[s], k0, w.yb * PZ_BM, w.x, T.az, 0);
            sm100::tma_load_5d(a + C::A_BYTES, &P.maps[T.mapB], &full[s], k0, w.nb * NT, T.by, T.bx, 0);
          }
        }
      }
      for(int u = (stage_it > STAGES ? stage_it - STAGES : 0); u < stage_it; u++)
        if(!sm100::mbar_wait(&full[u % STAGES], (u / STAGES) & 1)) fail();
    }
  } else if(warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if(lane == 0) {
      int stage_it = 0, term_it = 0;
      for(int it = 0;; it++) {
        const int r = it % PZ_IR;
        if(!sm100::mbar_wait(&item_full[r], (it / PZ_IR) & 1)) {
          fail();
          break;
        }
        const unsigned id = item_id[r];
        sm100::mbar_arrive(&item_empty[r]);
        if(id == PZ_END) break;
        const int Kp = P.phase == 0 ? P.kp_o : P.kp_v;
        for(int t = 0; t < 2; t++, term_it++) {
          const int buf = term_it & 1;
          if(term_it >= 2 && !sm100::mbar_wait(&lvl_empty[buf], ((term_it >> 1) - 1) & 1)) {
            fail();
            break;
          }
          sm100::tc_fence_after();
          const uint32_t dbase = tmem + buf * S * NT;
          for(int k0 = 0; k0 < Kp; k0 += PZ_KC, stage_it++) {
            const int s = stage_it % STAGES, use = stage_it / STAGES;
            if(!sm100::mbar_wait(&full[s], use & 1)) {
              fail();
              break;
            }
            sm100::tc_fence_after();
            const uint32_t a = sm100::smem_u32(smem + s * C::STAGE_BYTES), b = a + C::A_BYTES;
#pragma unroll
            for(int ks = 0; ks < PZ_KC / 16; ks++)
#pragma unroll
              for(int p = 1; p <= S; p++)
                sm100::mma_bf16(dbase + (p - 1) * NT, sm100::desc_kmajor_sw128(a + (p - 1) * PZ_BM * 128 + ks * 32),
                                sm100::desc_kmajor_sw128(b + ks * 32), sm100::idesc_bf16_f32(PZ_BM, (S + 1 - p) * NT),
                                (k0 == 0 && ks == 0 && p == 1) ? 0u : 1u);
            sm100::mma_commit(&empty[s]);
          }
          sm100::mma_commit(&lvl_full[buf]);
        }
        if(*abort_flag) break;
      }
      sm100::mma_commit(drain);
      if(!sm100::mbar_wait(drain, 0)) fail();
    }
  } else {
    // ------------------------------------------------------------ epilogue: 8 warps
    const int      q = warp & 3, half = (warp - 2) >> 2;   // lane quarter, column half
    const int      row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
    const int      c_lo = half * C::HALF;
    int            term_it = 0;
    float          tmax = 0.f;
    int            tail_slot = -1;
    for(int it = 0;; it++) {
      const int  r  = it % PZ_IR;
      const bool ok = __all_sync(0xffffffffu, sm100::mbar_wait(&item_full[r], (it / PZ_IR) & 1));
      if(!ok) {
        fail();
        break;
      }
      const unsigned id = item_id[r];
      __syncwarp();
      if(lane == 0) sm100::mbar_arrive(&item_empty[r]);
      if(id == PZ_END) break;
      const PzItem w = pz_decode(id, v, yblocks, nblocks);
      const int* tp = P.tri + 4 * (base + w.slot);
      if(P.tail && tp[3] != tail_slot) { // flush the per-triplet maximum when the triplet changes
        if(tail_slot >= 0) {
#pragma unroll
          for(int off = 16; off > 0; off >>= 1) tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
          if(lane == 0 && tmax > 0.f) atomicMax(reinterpret_cast<int*>(P.tail + tail_slot), __float_as_int(tmax));
        }
        tmax      = 0.f;
        tail_slot = tp[3];
      }
      const int  i = tp[0], j = tp[1], k = tp[2];
      const int  y = w.yb * PZ_BM + row, n0 = w.nb * NT + c_lo;
      const bool vrow = y < v;
      float hi[C::HALF], lo[C::HALF];
#pragma unroll
      for(int e = 0; e < C::HALF; e++) hi[e] = lo[e] = 0.f;
      bool aborted = false;
      for(int t = 0; t < 2; t++, term_it++) {
        const PzTerm T   = pz_term(P, w.job, t, i, j, k);
        const int    buf = term_it & 1;
        const bool   okw = __all_sync(0xffffffffu, sm100::mbar_wait(&lvl_full[buf], (term_it >> 1) & 1) && !*abort_flag);
        if(!okw) {
          fail();
          aborted = true;
          break;
        }
        sm100::tc_fence_after();
        const int ea = vrow ? T.eA[T.eA_base + (long long) w.x * T.eA_x + (long long) y * T.eA_y] : 0;
#pragma unroll
        for(int c0 = 0; c0 < C::HALF; c0 += 16) {
          int eb[16];
#pragma unroll
          for(int e = 0; e < 16; e++) eb[e] = (n0 + c0 + e < v) ? T.eB[n0 + c0 + e] : 0;
#pragma unroll 1
          for(int l = 0; l < S; l++) {
            uint32_t rv[16];
            sm100::tmem_ld16(lane_base + buf * S * NT + l * NT + c_lo + c0, rv);
            sm100::tmem_wait_ld();
#pragma unroll
            for(int e = 0; e < 16; e++) {
              const float term = __uint_as_float(rv[e]) * ldexpf(T.sign, ea + eb[e] - OZ_BITS * (l + 2));
              const ff    a    = ff_add_f(ff{hi[c0 + e], lo[c0 + e]}, term);
              hi[c0 + e]       = a.hi;
              lo[c0 + e]       = a.lo;
              if(l == S - 1 && vrow) tmax = fmaxf(tmax, fabsf(term));
            }
          }
        }
        sm100::tc_fence_before();
        __syncwarp();
        if(lane == 0) sm100::mbar_arrive(&lvl_empty[buf]);
      }
      if(aborted) break;
      if(vrow) {
        const long long v2 = (long long) v * v, m = (long long) w.x * v + y;
        float2*         Cb = P.F + (long long) w.slot * 3 * v2 * v + (long long) w.job * v2 * v;
        const long long csm = P.phase == 0 ? v : 1, csn = P.phase == 0 ? 1 : v2;
#pragma unroll
        for(int e = 0; e < C::HALF; e++) {
          const int n = n0 + e;
          if(n >= v) continue;
          float2* cp = Cb + m * csm + (long long) n * csn;
          ff      rr{hi[e], lo[e]};
          if(P.phase == 1) {
            const float2 old = *cp;
            rr = ff_add(rr, ff{old.x, old.y});
          }
          *cp = make_float2(rr.hi, rr.lo);
        }
      }
    }
    if(P.tail && tail_slot >= 0) {
#pragma unroll
      for(int off = 16; off > 0; off >>= 1) tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
      if(lane == 0 && tmax > 0.f) atomicMax(reinterpret_cast<int*>(P.tail + tail_slot), __float_as_int(tmax));
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
