// Persistent split-precision contraction: one CTA per SM pulls tiles from a device work queue.
//
// Work item = (triplet slot, job, x, y-block, n-block): one 128 x NT tile of one of the three
// partial arrays (job 0/1/2 = P12/P34/P56) of one occupied triplet, with all four of its terms
// (two d-sum terms, K = v, and two l-sum terms, K = o) accumulated into the same tile, so each
// element of P is written exactly once.  The host orders the items by estimated cost (largest
// first; ties keep the natural order, n-block fastest, so concurrently running CTAs share the A
// tile in L2) and the CTAs take them with atomicAdd on a device counter.  The triplets come from
// a device table, so the launch sequence of a batch is the same for every batch and can be
// replayed from a CUDA graph.
//
// Roles (608 threads): warp 0 lane 0 fetches items and issues TMA loads (running ahead across
// items), warp 1 issues the MMAs (one lane, no mbarrier waits), warp 2 is its gate (does those
// waits and hands each stage over at a named barrier), warps 3-18 fold the digit levels into
// float-float.  The TMEM level accumulators are double buffered by term, so the fold of one term
// overlaps the MMAs of the next; the float-float accumulator of a tile lives in registers (each
// epilogue thread owns one row and a quarter of the tile's columns).  All mbarrier waits are
// bounded (sm100::kSpinLimit); the named-barrier rendezvous ends when the gate's bounded waits do.
#pragma once

#include <cuda.h>

#include <type_traits>

#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace ccsdt {

// 3 role warps (TMA producer, MMA issuer, gate) + PZ_EPI epilogue warps (4 per TMEM lane quarter)
constexpr int PZ_BM = 128, PZ_EPI = 16, PZ_EPI_W0 = 3, PZ_THREADS = 32 * (PZ_EPI_W0 + PZ_EPI), PZ_IR = 4,
              PZ_TERMS = 4;

// The MMA warp and its gate warp meet at named barrier 1 (64 threads) once per pipeline stage.
// tcgen05.mma issue proceeds at the tensor pipe's pace (the issuing thread holds only a few MMAs
// ahead of the pipe), so anything else that thread does between stages idles the pipe for as
// long: an mbarrier wait there, even on a completed phase, measured 170 - 550 cycles per stage on
// GB300, against none for a named-barrier rendezvous with a warp that has already done the waits.
// So the gate warp does every wait of the MMA loop (stage full, TMEM level buffer empty, work
// items) and the MMA warp only rendezvouses.  Both walk the same stage sequence; the rendezvous
// is an OR-reduction of a stop bit (bar.red: no shared-memory flag to read back), which the gate
// sets when it must stop (a bounded wait gave up, the abort flag, the end of the work), and both
// leave at that same rendezvous, so neither is left waiting at the barrier.  Like bar.sync it
// orders the gate's observations (the TMA bytes have landed) before the MMA warp's later work.
__device__ __forceinline__ bool pz_gate_sync(bool stop) {
  uint32_t r;
  asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, 64, q;\n\tselp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(r)
               : "r"((uint32_t) stop)
               : "memory");
  return r != 0;
}
constexpr unsigned PZ_END = 0xffffffffu;

// map indices (the handle's map table): the d-sum uses 0-2, the l-sum 6-8
enum {
  PZ_OVVV_NAT = 0, PZ_OVVV_SWP = 1, PZ_T2 = 2, PZ_T2H_NAT_B = 6, PZ_T2H_SWP_B = 7, PZ_OOOVH_A = 8, PZ_NMAPS = 9
};

struct PzParams {
  CUtensorMap     maps[PZ_NMAPS];
  const int*      tri;        // triplet table (4 ints per triplet: i, j, k, output index)
  const int*      base;       // device batch base index into tri (nullable -> 0)
  int             nslots;     // triplets per launch
  int             o, v, kp_v, kp_o;
  float2*         F;          // P arrays of slot s: F + s * 3 v^3 (P12, P34, P56 consecutive)
  int             f32_out;    // store P rounded to FP32 (element e at ((float*) F)[e]) instead of
                              // float-float (F[e])
  int             f64_out;    // store P in FP64 (element e at ((double*) F)[e]): the float-float
                              // result widened (the exact fold of S <= 4 levels equals FP64's)
  const int*      ovvv_slot;  // (ia|bc) digit planes by slot: slot of occupied index z (nullable:
                              // slot = z; the Cholesky-direct mode's slab cache otherwise)
  const unsigned* order;      // cost-ordered item ids, length nitems
  unsigned        nitems;
  unsigned*       queue;      // work counter, 0 at launch
  int*            err;        // set on a bounded-wait timeout
  float*          tail;       // optional: tail[output index] += sum of squares of the last
                              // kept level's terms (a-posteriori truncation estimate)
  int             wst;        // stages (K chunks) per exact K window: a term longer than this is
                              // accumulated and folded window by window (pz_window_k)
  unsigned        spin;       // polls before a bounded mbarrier wait gives up (sm100::kSpinLimit)
  int             skip_loads; // testing: announce each stage's bytes but issue no TMA load, so
                              // the stage waits run out (the timeout path, CCSDT_E_TIMEOUT)
};

struct PzTerm {
  int mapA, mapB, a2, a3, b2, b3, Kp; // maps and their tile coordinates along dims 2, 3
};

// Longest contraction window (a multiple of kc) whose digit-level sums stay exact in an FP32
// accumulator for S digit planes.  Level l = p + q (2 <= l <= S + 1) sums sigma_p tau_q over the
// pairs p + q = l and the window's k, with |sigma_1| <= 127 and |sigma_p| <= 64 (p > 1): per k at
// most 127^2 (l = 2) or 2 127 64 + (l - 3) 64^2 (l >= 3), growing with l, so the bound of level
// S + 1 times the window length must stay <= 2^24.  S = 1..8 -> 1040, 1032, 824, 686, 587, 514,
// 456, 410 before rounding down to kc.  A term longer than its window is accumulated window by
// window, each window folded into the float-float result on its own.
__host__ __device__ constexpr int pz_window_k(int S, int kc) {
  const long per_k = S + 1 == 2 ? 127L * 127 : 2L * 127 * 64 + (long) (S + 1 - 3) * 64 * 64;
  return (int) (((1L << 24) / per_k) / kc * kc);
}
static_assert(pz_window_k(3, 64) == 768 && pz_window_k(4, 64) == 640 && pz_window_k(5, 64) == 576 &&
                pz_window_k(6, 64) == 512 && pz_window_k(7, 64) == 448 && pz_window_k(8, 64) == 384, "exact windows");
// passes of a term of nst stages with wst stages per window, and the stages of its pass w
__device__ __forceinline__ int pz_npass(int nst, int wst) { return nst <= wst ? 1 : (nst + wst - 1) / wst; }
__device__ __forceinline__ int pz_pass_st(int nst, int wst, int w) { return nst <= wst ? nst : min(wst, nst - w * wst); }

// The four terms of a job's tile, from (job, t, i, j, k) and the item's x.  The tile holds
// P[n][x][y] for 128 rows y and NT columns n (P12[a][c][b]: n = a, x = c, y = b; P34[b][a][c];
// P56[c][b][a]):
//   t = 0, 1  d-sum  P[n][x][y] += sum_d ovvv(z)[(x,y) or (y,x)][d] t2(xx,yy)[n][d]
//   t = 2, 3  l-sum  P[n][x][y] -= sum_l t2h(xx)[(n,x) or (x,n)][l] ooovh(yy,zz)[y][l]
// with, per job, (first index, natural pair order?, second, third):
//   d-sum  job 0: (k,1,i,j) (j,0,i,k)   job 1: (k,0,j,i) (i,1,j,k)   job 2: (j,1,k,i) (i,0,k,j)
//   l-sum  job 0: (i,1,k,j) (k,0,i,j)   job 1: (i,0,j,k) (j,1,i,k)   job 2: (j,0,k,i) (k,1,j,i)
// The l-sum's "natural" pair (first, second) = (n, x) is read through the swapped-stride map.
__device__ __forceinline__ PzTerm pz_term(const PzParams& P, int job, int t, int i, int j, int k, int x) {
  const int sel = job * 2 + (t & 1);
  int       e0, nat, e2, e3;
  if(t < 2) {
    switch(sel) {
      case 0: e0 = k, nat = 1, e2 = i, e3 = j; break;
      case 1: e0 = j, nat = 0, e2 = i, e3 = k; break;
      case 2: e0 = k, nat = 0, e2 = j, e3 = i; break;
      case 3: e0 = i, nat = 1, e2 = j, e3 = k; break;
      case 4: e0 = j, nat = 1, e2 = k, e3 = i; break;
      default: e0 = i, nat = 0, e2 = k, e3 = j; break;
    }
  } else {
    switch(sel) {
      case 0: e0 = i, nat = 1, e2 = k, e3 = j; break;
      case 1: e0 = k, nat = 0, e2 = i, e3 = j; break;
      case 2: e0 = i, nat = 0, e2 = j, e3 = k; break;
      case 3: e0 = j, nat = 1, e2 = i, e3 = k; break;
      case 4: e0 = j, nat = 0, e2 = k, e3 = i; break;
      default: e0 = k, nat = 1, e2 = j, e3 = i; break;
    }
  }
  PzTerm T;
  if(t < 2) {
    const int z = e0, xx = e2, yy = e3;
    T.mapA = nat ? PZ_OVVV_NAT : PZ_OVVV_SWP, T.a2 = x;              // rows (z, x, y) or (z, y, x)
    T.a3   = P.ovvv_slot ? __ldg(P.ovvv_slot + z) : z;
    T.mapB = PZ_T2, T.b2 = yy, T.b3 = xx;                            // rows (xx, yy, n)
    T.Kp = P.kp_v;
  } else {
    const int xx = e0, yy = e2, zz = e3;
    T.mapA = PZ_OOOVH_A, T.a2 = zz, T.a3 = yy;                        // rows (yy, zz, y)
    T.mapB = nat ? PZ_T2H_SWP_B : PZ_T2H_NAT_B, T.b2 = x, T.b3 = xx;   // pair rows (n, x) or (x, n)
    T.Kp = P.kp_o;
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

// Epilogue of one item: thread = one tile row (TMEM lane
// quarter q, row = 32 q + lane) x COLS = NT / 4 columns from c_lo.  Per term it waits for the MMAs
// (lvl_full of the term's buffer), folds the S exact levels with oz_horner in chunks of 8 columns
// and adds (d-sum terms) or subtracts (l-sum terms) them in float-float, releases the buffer
// (lvl_empty); finally it renormalises, scales by 2^(-7 (S + 1)) and stores the tile once (FP32
// partial arrays: the fold and the term sums in FP32, one store per element).  The
// BF16 digits carry the row scales, so the levels need no per-row or per-column factor.  Returns
// false when a bounded wait gave up.
template<int S, int NT, int NBUF, int KC>
__device__ __forceinline__ bool pz_epilogue_item(const PzParams& P, const PzItem& w, int nb, const int* tp,
                                                 uint32_t lane_base, int c_lo, int row, int lane, int& term_it,
                                                 float& tsq, uint64_t* lvl_full, uint64_t* lvl_empty,
                                                 volatile int* abort_flag) {
  constexpr int COLS = NT / 4;
  static_assert(COLS % 4 == 0 && COLS <= 32, "epilogue column chunks of 8 (and a last one of 4)");
  constexpr float kScale = 1.f / float(1ull << (OZ_BITS * (S + 1)));
  const int       v  = P.v;
  const long long v2 = (long long) v * v;
  const int       y = w.yb * PZ_BM + row, n0 = nb * NT + c_lo;
  (void) tp;
  // element (y, n) of the tile: P[n][x][y] (consecutive rows -> consecutive addresses)
  const long long e0 = (long long) w.slot * 3 * v2 * v + (long long) w.job * v2 * v + (long long) w.x * v + y;
  float hi[COLS], lo[COLS];
  const int np_d = pz_npass(P.kp_v / KC, P.wst), np_l = pz_npass(P.kp_o / KC, P.wst);
#pragma unroll 1
  for(int tw = 0; tw < 2 * (np_d + np_l); tw++, term_it++) {
    // pass tw: term t (two d-sum terms of np_d windows, then two l-sum terms of np_l windows)
    const int  t   = tw < 2 * np_d ? tw / np_d : 2 + (tw - 2 * np_d) / np_l;
    const int  buf = term_it % NBUF;
    const bool okw = __all_sync(0xffffffffu, sm100::mbar_wait(&lvl_full[buf], (term_it / NBUF) & 1, P.spin) && !*abort_flag);
    if(!okw) return false;
    sm100::tc_fence_after();
    // fold `W` columns starting at c0 whose S levels are in rv; `neg`: an l-sum term; `first`: the
    // item's first term (the accumulators start from it)
    auto fold = [&](auto& rv, int c0, auto wtag, bool neg, bool first) {
      constexpr int W = decltype(wtag)::value;
      if(P.f32_out) { // FP32 partial arrays: FP32 fold and term sums (a few roundings per element)
#pragma unroll
        for(int e = 0; e < W; e++) {
          const float x = oz_horner_f32<S, W>(rv, e);
          hi[c0 + e]    = first ? (neg ? -x : x) : (neg ? hi[c0 + e] - x : hi[c0 + e] + x);
          if(P.tail) {
            const float tl = __uint_as_float(rv[S - 1][e]) * kScale;
            tsq            = fmaf(tl, tl, tsq);
          }
        }
        return;
      }
#pragma unroll
      for(int e = 0; e < W; e++) {
        const ff    x  = oz_horner<S, W>(rv, e);
        const float xh = neg ? -x.hi : x.hi, xl = neg ? -x.lo : x.lo;
        if(first) {
          hi[c0 + e] = xh;
          lo[c0 + e] = xl;
        } else {
          // two-sum of the high words, low words added; the tile is renormalised before the store
          const float s = hi[c0 + e] + xh, z = s - hi[c0 + e];
          lo[c0 + e]    = lo[c0 + e] + (((hi[c0 + e] - (s - z)) + (xh - z)) + xl);
          hi[c0 + e]    = s;
        }
        if(P.tail) {
          const float tl = __uint_as_float(rv[S - 1][e]) * kScale;
          tsq            = fmaf(tl, tl, tsq);
        }
      }
    };
    // the buffer is released as soon as its last levels are in registers, before the fold of
    // those columns: the MMAs of the term after next need not wait for the arithmetic
    auto release = [&]() {
      sm100::tc_fence_before();
      __syncwarp();
      if(lane == 0) sm100::mbar_arrive(&lvl_empty[buf]);
    };
    auto run = [&](bool neg, bool first) {
      if constexpr(S * COLS <= 32) {
        uint32_t rv[S][COLS]; // every level of the thread's columns in one TMEM round trip
#pragma unroll
        for(int l = 0; l < S; l++) {
          if constexpr(COLS == 16) sm100::tmem_ld16(lane_base + buf * S * NT + l * NT + c_lo, rv[l]);
          else sm100::tmem_ld8(lane_base + buf * S * NT + l * NT + c_lo, rv[l]);
        }
        sm100::tmem_wait_ld();
        release();
        fold(rv, 0, std::integral_constant<int, COLS>{}, neg, first);
      } else {
        // chunks of 8 columns and, when COLS % 8 == 4, one of 4; every TMEM access starts at a
        // multiple of its own width (a thread whose first column is 4 mod 8 takes the 4 first)
        auto chunk8 = [&](int c0, bool last) {
          uint32_t rv[S][8];
#pragma unroll
          for(int l = 0; l < S; l++) sm100::tmem_ld8(lane_base + buf * S * NT + l * NT + c_lo + c0, rv[l]);
          sm100::tmem_wait_ld();
          if(last) release();
          fold(rv, c0, std::integral_constant<int, 8>{}, neg, first);
        };
        auto chunk4 = [&](int c0, bool last) {
          uint32_t rv[S][4];
#pragma unroll
          for(int l = 0; l < S; l++) sm100::tmem_ld4(lane_base + buf * S * NT + l * NT + c_lo + c0, rv[l]);
          sm100::tmem_wait_ld();
          if(last) release();
          fold(rv, c0, std::integral_constant<int, 4>{}, neg, first);
        };
        if constexpr(COLS % 8 == 0) {
#pragma unroll
          for(int c0 = 0; c0 < COLS; c0 += 8) chunk8(c0, c0 + 8 == COLS);
        } else if((c_lo & 7) == 4) {
          chunk4(0, false);
#pragma unroll
          for(int c0 = 4; c0 < COLS; c0 += 8) chunk8(c0, c0 + 8 == COLS);
        } else {
#pragma unroll
          for(int c0 = 0; c0 + 8 <= COLS; c0 += 8) chunk8(c0, false);
          chunk4(COLS - 4, true);
        }
      }
    };
    if(tw == 0) run(false, true); // d-sum terms add, l-sum terms subtract
    else if(t < 2) run(false, false);
    else run(true, false);
  }
  if(y < v) {
    if(P.f64_out) { // the float-float sums widened to FP64 (exact: 48 significant bits at most)
      double* Cd = reinterpret_cast<double*>(P.F) + e0;
#pragma unroll
      for(int e = 0; e < COLS; e++)
        if(n0 + e < v) Cd[(long long) (n0 + e) * v2] = ((double) hi[e] + (double) lo[e]) * (double) kScale;
    } else if(P.f32_out) { // the FP32 sums; the power-of-two scale is exact
      float* Cf = reinterpret_cast<float*>(P.F) + e0;
#pragma unroll
      for(int e = 0; e < COLS; e++)
        if(n0 + e < v) Cf[(long long) (n0 + e) * v2] = hi[e] * kScale;
    } else {
      float2* Cb = P.F + e0;
#pragma unroll
      for(int e = 0; e < COLS; e++) {
        const int   n = n0 + e;
        const float h = hi[e] + lo[e];
        if(n < v) Cb[(long long) n * v2] = make_float2(h * kScale, (lo[e] - (h - hi[e])) * kScale);
      }
    }
  }
  return true;
}

// Adds a warp's per-thread sums of squares to tail[slot] (one atomic per warp).
__device__ __forceinline__ void pz_flush_tail(float* tail, int slot, float tsq, int lane) {
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) tsq += __shfl_xor_sync(0xffffffffu, tsq, off);
  if(lane == 0 && tsq > 0.f) atomicAdd(tail + slot, tsq);
}

// The MMAs of one pipeline stage (KC = 64 or 32 along K, KC / 16 k-steps of 16): for every
// k-step, S MMAs A_p x [B_1 .. B_{S+1-p}] into the level columns (p - 1) NT ...  Rows are KC x 2
// bytes (128 B under the 128-byte swizzle, 64 B under the 64-byte one).  The descriptors are built
// once per stage: the start-address field (bits 0-13, address >> 4) is linear, so the plane and
// k-step offsets (multiples of 16 B, all inside the 228 KB window) are added to it directly.
// `first`: the stage opens the term (its first MMA overwrites the accumulators).  The whole warp
// calls it; the lanes with `issue` set (one) issue.
template<int KC>
__device__ __forceinline__ uint64_t pz_desc(uint32_t smem_addr) {
  static_assert(KC == 64 || KC == 32, "K chunks of 64 (128-byte rows) or 32 (64-byte rows)");
  return KC == 64 ? sm100::desc_kmajor_sw128(smem_addr) : sm100::desc_kmajor_sw64(smem_addr);
}
template<int S, int NT, int KC>
__device__ __forceinline__ void pz_issue_stage(uint32_t dbase, uint32_t a_smem, uint32_t b_smem, bool first,
                                               uint32_t issue) {
  const uint64_t da = pz_desc<KC>(a_smem), db = pz_desc<KC>(b_smem);
#pragma unroll
  for(int ks = 0; ks < KC / 16; ks++)
#pragma unroll
    for(int p = 1; p <= S; p++)
      sm100::mma_bf16_if(dbase + (p - 1) * NT, da + (uint64_t) (((p - 1) * PZ_BM * KC * 2 + ks * 32) >> 4),
                         db + (uint64_t) ((ks * 32) >> 4), sm100::idesc_bf16_f32(PZ_BM, (S + 1 - p) * NT),
                         (first && ks == 0 && p == 1) ? 0u : 1u, issue);
}

template<int S, int NT, int STAGES, int KC>
struct PzCfg {
  static constexpr int A_BYTES = S * PZ_BM * KC * 2, B_BYTES = S * NT * KC * 2, STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 512;
  static constexpr int COLS = NT / 4;   // columns per epilogue thread
  static constexpr uint32_t TMEM_COLS = 512;
  // level buffers in TMEM (S x NT columns each): three where they fit, so the MMA issuer can run
  // two terms ahead of the epilogue (a short l-sum term then never leaves the tensor pipe idle)
  static constexpr int NBUF = 3 * S * NT <= 512 ? 3 : 2;
  static_assert(2 * S * NT <= 512, "two level buffers must fit in TMEM");
  static_assert(S * NT <= 256 && NT % 16 == 0, "MMA N limit / epilogue quarters of 4k columns");
};

template<int S, int NT, int STAGES, int KC>
__global__ void __launch_bounds__(PZ_THREADS, 1) oz_persist_kernel(const __grid_constant__ PzParams P) {
  using C = PzCfg<S, NT, STAGES, KC>;
  const int v = P.v, yblocks = (v + PZ_BM - 1) / PZ_BM, nblocks = (v + NT - 1) / NT;
  const int base = P.base ? *P.base : 0;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full       = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint64_t* empty      = full + STAGES;
  uint64_t* item_full  = empty + STAGES;
  uint64_t* item_empty = item_full + PZ_IR;
  uint64_t* lvl_full   = item_empty + PZ_IR;   // [NBUF] MMAs of a term done
  uint64_t* lvl_empty  = lvl_full + 3;         // [NBUF] epilogue drained the buffer
  uint64_t* drain      = lvl_empty + 3;
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
      sm100::mbar_init(&item_empty[r], 1 + PZ_EPI); // gate + one arrival per epilogue warp
    }
    for(int b = 0; b < C::NBUF; b++) {
      sm100::mbar_init(&lvl_full[b], 1);
      sm100::mbar_init(&lvl_empty[b], PZ_EPI);
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
      for(int m: {PZ_OVVV_NAT, PZ_OVVV_SWP, PZ_T2, PZ_T2H_NAT_B, PZ_T2H_SWP_B, PZ_OOOVH_A}) sm100::prefetch_tmap(&P.maps[m]);
      int stage_it = 0;
      for(int it = 0;; it++) {
        const unsigned q  = atomicAdd(P.queue, 1u);
        const unsigned id = (q < P.nitems && !*abort_flag) ? P.order[q] : PZ_END;
        const int      r  = it % PZ_IR;
        if(it >= PZ_IR && !sm100::mbar_wait(&item_empty[r], ((it / PZ_IR) - 1) & 1, P.spin)) {
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
        for(int t = 0; t < PZ_TERMS; t++) {
          const PzTerm T = pz_term(P, w.job, t, i, j, k, w.x);
          for(int k0 = 0; k0 < T.Kp; k0 += KC, stage_it++) {
            const int s = stage_it % STAGES, use = stage_it / STAGES;
            if(use > 0 && !sm100::mbar_wait(&empty[s], (use - 1) & 1, P.spin)) {
              fail();
              break;
            }
            unsigned char* a = smem + s * C::STAGE_BYTES;
            sm100::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
            if(!P.skip_loads) {
              sm100::tma_load_5d(a, &P.maps[T.mapA], &full[s], k0, w.yb * PZ_BM, T.a2, T.a3, 0);
              sm100::tma_load_5d(a + C::A_BYTES, &P.maps[T.mapB], &full[s], k0, w.nb * NT, T.b2, T.b3, 0);
            }
          }
        }
      }
      for(int u = (stage_it > STAGES ? stage_it - STAGES : 0); u < stage_it; u++)
        if(!sm100::mbar_wait(&full[u % STAGES], (u / STAGES) & 1, P.spin)) fail();
    }
  } else if(warp == 1) {
    // ------------------------------------------------------------ MMA issuer (the warp runs the
    // loop, lane 0 issues).  The MMAs need no item data: every item is the same sequence of terms and stages, and the
    // gate says when the work ends.  Between stages the loop does as little as it can (no
    // modulo, no shared-memory reads): the tensor pipe idles for as long as it runs.
    const uint32_t a0 = sm100::smem_u32(smem);
    uint32_t       a = a0;
    int            s = 0, term_it = 0;
    bool           stop = false;
    while(!stop) {
      for(int t = 0; t < PZ_TERMS && !stop; t++) {
        const int nst = (t < 2 ? P.kp_v : P.kp_o) / KC, np = pz_npass(nst, P.wst);
        for(int w = 0; w < np && !stop; w++, term_it++) { // one TMEM level buffer per window
          const int      ns    = pz_pass_st(nst, P.wst, w);
          const uint32_t dbase = tmem + (term_it % C::NBUF) * S * NT;
          for(int u = 0; u < ns; u++) {
            if((stop = pz_gate_sync(false))) break;
            sm100::tc_fence_after();
            pz_issue_stage<S, NT, KC>(dbase, a, a + C::A_BYTES, u == 0, lane == 0);
            sm100::mma_commit_if(&empty[s], lane == 0);
            a += C::STAGE_BYTES;
            if(++s == STAGES) s = 0, a = a0;
          }
          if(!stop) sm100::mma_commit_if(&lvl_full[term_it % C::NBUF], lane == 0);
        }
      }
    }
    if(lane == 0) {
      sm100::mma_commit(drain);
      if(!sm100::mbar_wait(drain, 0, P.spin)) fail();
    }
  } else if(warp == 2) {
    // ------------------------------------------------------------ gate: the MMA issuer's waits
    int  stage_it = 0, term_it = 0;
    bool stop     = false;
    for(int it = 0; !stop; it++) {
      const int r  = it % PZ_IR;
      int       ok = 1;
      unsigned  id = PZ_END;
      if(lane == 0) {
        ok = sm100::mbar_wait(&item_full[r], (it / PZ_IR) & 1, P.spin);
        if(ok) {
          id = item_id[r];
          sm100::mbar_arrive(&item_empty[r]);
        } else
          fail();
      }
      if(__shfl_sync(0xffffffffu, ok && id != PZ_END, 0) == 0) { // the issuer's next rendezvous ends it
        pz_gate_sync(true);
        break;
      }
      for(int t = 0; t < PZ_TERMS && !stop; t++) {
        const int nst = (t < 2 ? P.kp_v : P.kp_o) / KC, np = pz_npass(nst, P.wst);
        for(int w = 0; w < np && !stop; w++, term_it++) {
          const int ns  = pz_pass_st(nst, P.wst, w);
          const int buf = term_it % C::NBUF;
          if(lane == 0 && term_it >= C::NBUF) ok = sm100::mbar_wait(&lvl_empty[buf], ((term_it / C::NBUF) - 1) & 1, P.spin);
          for(int u = 0; u < ns; u++, stage_it++) {
            bool mine = false;
            if(lane == 0) {
              if(ok) ok = sm100::mbar_wait(&full[stage_it % STAGES], (stage_it / STAGES) & 1, P.spin);
              if(!ok) fail();
              mine = !ok || *abort_flag;
            }
            __syncwarp();
            if((stop = pz_gate_sync(mine))) break;
          }
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue: PZ_EPI warps
    // Thread = one tile row (TMEM lane) x a quarter of the tile's columns (pz_epilogue_item).
    const int      q = warp & 3, cq = (warp - PZ_EPI_W0) >> 2; // TMEM lane quarter, column quarter
    const int      row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
    const int      c_lo = cq * C::COLS;
    int            term_it = 0;
    float          tsq = 0.f;                                // sum of squares of last-level terms
    int            tail_slot = -1;
    for(int it = 0;; it++) {
      const int  r  = it % PZ_IR;
      const bool ok = __all_sync(0xffffffffu, sm100::mbar_wait(&item_full[r], (it / PZ_IR) & 1, P.spin));
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
      if(P.tail && tp[3] != tail_slot) { // flush the per-triplet sum when the triplet changes
        if(tail_slot >= 0) pz_flush_tail(P.tail, tail_slot, tsq, lane);
        tsq       = 0.f;
        tail_slot = tp[3];
      }
      if(!pz_epilogue_item<S, NT, C::NBUF, KC>(P, w, w.nb, tp, lane_base, c_lo, row, lane, term_it, tsq, lvl_full,
                                               lvl_empty, abort_flag)) {
        fail();
        break;
      }
    }
    if(P.tail && tail_slot >= 0) pz_flush_tail(P.tail, tail_slot, tsq, lane);
  }
  sm100::tc_fence_before();
  __syncthreads();
  if(warp == 1) {
    sm100::tc_fence_after();
    sm100::tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

} // namespace ccsdt
