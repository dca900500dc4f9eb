// Tiled energy of a batch of triplets with the partial arrays staged by TMA (split-precision path).
//
// The same work units and orbit arithmetic as energy_tiled.cuh (one sorted 8-wide virtual block
// triple X <= Y <= Z per unit, W_xyz = P12[x][z][y] + P34[y][x][z] + P56[z][y][x], every orbit
// {a, b, c} with its six orderings), but the eighteen 8 x 8 x 8 boxes a unit needs - for each of
// its six ordered cubes, the matching box of P12, P34 and P56 - are copied into shared memory by
// eighteen TMA tensor loads issued by eighteen lanes of one warp, so no thread computes an address
// into the partial arrays and out-of-range rows (v not a multiple of 8) arrive as zeros.  The orbits then
// read their W values from the boxes directly: cube q of the unit at its local (x, y, z) is
// box12_q[x][z][y] + box34_q[y][x][z] + box56_q[z][y][x], summed in the order of the
// pass-by-pass kernel, so both kernels give the same W bit for bit.
//
// Pipeline: unit n + 1's singles data are read into registers while unit n is evaluated and, with
// two box stages (the FP32 default), its boxes load too; float-float boxes (twice the bytes) use one
// stage, which lets two CTAs share an SM instead of one - the faster of the two on GB300.
//
// Lane -> orbit: warp g (16 per unit, two per thread block warp), lane (u = lane % 8, w = lane / 8)
// takes la = w + 4 (g % 2), lb = u, lc = (u + w + g / 2) % 8.  For every one of the eighteen reads
// (each position of each box layout takes each of the three coordinates) the 32 lanes then touch
// at most two addresses per bank.
//
// Needs the partial arrays' row pitch to be a multiple of 16 bytes (v % 4 == 0 for FP32 elements,
// v even for float-float); the host falls back to the pass-by-pass kernel otherwise.
#pragma once

#include "energy_tiled.cuh"
#include "sm100_ptx.cuh"

namespace ccsdt {

constexpr int EM_THREADS = 256, EM_BOXES = 18;

struct TmaEnergyArgs {
  CUtensorMap   pmap;      // partial arrays of the batch: dims (v, v, v, 3 slots), box 8 x 8 x 8 x 1
  const float * oovv, *t1; // FP32 copies
  const double *oovv_d, *t1_d; // FP64 originals (FP64 partial arrays)
  const double *eo, *ev;
  const int3*   tiles;     // sorted block triples
  int           ntiles;
  int           o, v;
  const int*    tri;       // 4 ints per triplet: i, j, k, output index
  const int*    base;      // device batch base index into tri (nullable -> 0)
  double*       part;      // [slot][gridDim.x][6]
  int           want_sens;
  int*          err;       // set when a bounded wait gave up
  unsigned      spin;
  int           skip_loads; // testing: announce each unit's bytes but issue no box load, so the
                            // waits run out (the timeout path, CCSDT_E_TIMEOUT)
};

// bytes of dynamic shared memory: the eighteen boxes of each of the NST box stages
template<typename TP>
constexpr size_t em_stage_bytes() {
  return (size_t) EM_BOXES * ET_B * ET_B * ET_B * sizeof(TP);
}
template<typename TP, int NST>
constexpr size_t em_smem_bytes() {
  return NST * em_stage_bytes<TP>();
}
// resident CTAs per SM the shared memory allows (the launch bounds follow it)
template<typename TP, int NST>
constexpr int em_min_blocks() {
  return std::is_same<TP, float>::value ? (NST == 2 ? 2 : 4) : (NST == 2 ? 1 : 2);
}

// Per-stage shared data of a unit besides the boxes: the singles' integrals and amplitudes of its
// three blocks, its virtual orbital energies, the orbit-wide part of D and the distinct-cube flags.
// SS: the singles' scalar (float; double for FP64 partial arrays), ES: the orbital energies'
// (float-float pair; double).
template<typename SS, typename ES>
struct EmSingles {
  SS  Ojk[3][3][ET_B * ET_B], Oik[3][3][ET_B * ET_B], Oij[3][3][ET_B * ET_B];
  SS  ti[3][ET_B], tj[3][ET_B], tk[3][ET_B];
  ES  evs[3][ET_B];
  ES  dab[ET_B * ET_B];
  int slot_on[6];
};

// A thread's share of one unit's singles data, loaded from global memory into registers while the
// previous unit is being evaluated and stored to that unit's stage afterwards.
template<typename SS, typename ES>
struct EmPrefetch {
  SS  o[2][3]; // (jk), (ik), (ij) integrals at the thread's two singles positions
  SS  t[3];    // t_i, t_j, t_k at (block, index) = (tid / 8, tid % 8), threads 0..23
  ES  ev;      // e_v there
  ES  dab;     // e_i + e_j + e_k - e_a - e_b, threads 64..127
  int on;      // distinct-cube flag, threads 96..101
};

// FP64 partial arrays: the singles parts of V and the orbit's energy terms in FP64, compensated
// (Kahan) FP64 sums - the precision of the plain FP64 path's energy.
__device__ __forceinline__ void et_singles_f64(const double (*Ojk)[3][ET_B * ET_B],
                                               const double (*Oik)[3][ET_B * ET_B],
                                               const double (*Oij)[3][ET_B * ET_B], const double (*ti)[ET_B],
                                               const double (*tj)[ET_B], const double (*tk)[ET_B], int la, int lb,
                                               int lc, double (&sg)[6]) {
  constexpr int B = ET_B;
  const int loc[3] = {la, lb, lc};
#pragma unroll
  for(int q = 0; q < 6; q++) {
    const int p0 = kPerm(q, 0), p1 = kPerm(q, 1), p2 = kPerm(q, 2);
    const int x = loc[p0], y = loc[p1], z = loc[p2];
    sg[q] = Ojk[p1][p2][y * B + z] * ti[p0][x] + Oik[p0][p2][x * B + z] * tj[p1][y] + Oij[p0][p1][x * B + y] * tk[p2][z];
  }
}
__device__ __forceinline__ void et_orbit_values_f64(const double (&w)[6], const double (&sg)[6],
                                                    const double (*evs)[ET_B], const double* dab, bool all_on,
                                                    const int* slot_on, int la, int lb, int lc, int want_sens,
                                                    CSum& s4, CSum& s5, float& sens) {
  constexpr int B = ET_B;
  const double ca = w[0] + w[3] + w[4], cb = w[1] + w[2] + w[5]; // the two cyclic classes
  const double sga = sg[0] + sg[3] + sg[4], sgb = sg[1] + sg[2] + sg[5];
  double       zy4 = 0.0, zys = 0.0;
  float        sn  = 0.f;
#pragma unroll
  for(int q = 0; q < 6; q++) {
    if(!all_on && !slot_on[q]) continue;
    const bool   in_a = q == 0 || q == 3 || q == 4;
    const double z    = 3.0 * w[q] + (in_a ? ca : cb);   // 4 W_q + the other two of its class
    const double y4   = 3.0 * w[q] - (in_a ? cb : ca);   // 3 W_q - the other class
    const double ys   = 3.0 * sg[q] - (in_a ? sgb : sga);
    zy4 += z * y4;
    zys += z * ys;
    if(want_sens) {
      const float y5 = (float) (y4 + ys), zf = (float) z;
      sn             = fmaf(18.f * y5, y5, fmaf(12.f * zf, zf, sn));
    }
  }
  const double d = dab[la * B + lb] - evs[2][lc];
  s4.add(zy4 / d);
  s5.add((zy4 + zys) / d);
  const float id = (float) (1.0 / d);
  sens           = fmaf(sn * id, id, sens);
}

// NST = 2: unit n + 1's boxes load into the other stage while unit n is evaluated; NST = 1: one
// stage (the load waits for the previous unit's orbits), twice the resident CTAs hiding it.
template<typename TP, int NST>
static __global__ void __launch_bounds__(EM_THREADS, (em_min_blocks<TP, NST>()))
  energy_tma_batch_kernel(const __grid_constant__ TmaEnergyArgs A) {
  static_assert(NST == 1 || NST == 2, "one or two box stages");
  constexpr int  B = ET_B, B3 = B * B * B;
  constexpr bool kF32 = std::is_same<TP, float>::value, kF64 = std::is_same<TP, double>::value;
  using SS = typename std::conditional<kF64, double, float>::type;
  using ES = typename std::conditional<kF64, double, float2>::type;
  extern __shared__ __align__(128) unsigned char em_dyn[];
  // stage st: boxes [pass][slot q][512] at em_dyn + st * em_stage_bytes (pass 0 = P12, 1 = P34, 2 = P56)
  __shared__ EmSingles<SS, ES> sgl[2];
  __shared__ uint64_t          full[2];

  const int       slot = blockIdx.y, b0 = A.base ? *A.base : 0;
  const int*      tp   = A.tri + 4 * (b0 + slot);
  const int       i = tp[0], j = tp[1], k = tp[2];
  const int       v = A.v, o = A.o, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long v2 = (long long) v * v;
  const ff        eijk = ff_add(ff_add(ff_from_double(A.eo[i]), ff_from_double(A.eo[j])), ff_from_double(A.eo[k]));
  const double    eijk_d = A.eo[i] + A.eo[j] + A.eo[k];
  const SS*       goovv  = kF64 ? reinterpret_cast<const SS*>(A.oovv_d) : reinterpret_cast<const SS*>(A.oovv);
  const SS*       gt1    = kF64 ? reinterpret_cast<const SS*>(A.t1_d) : reinterpret_cast<const SS*>(A.t1);
  const SS *      gOjk = goovv + ((long long) j * o + k) * v2, *gOik = goovv + ((long long) i * o + k) * v2,
           *gOij = goovv + ((long long) i * o + j) * v2;
  if(tid == 0) {
    sm100::mbar_init(&full[0], 1);
    sm100::mbar_init(&full[1], 1);
    sm100::mbar_fence_init();
    sm100::prefetch_tmap(&A.pmap);
  }
  __syncthreads();

  // the last warp issues a unit's eighteen box loads into stage st, one per lane (lane 0 first
  // announces the stage's bytes), so the issue is short and off the warps with prefetch extras
  auto issue = [&](int tile, int st) {
    const int3 tt     = A.tiles[tile];
    const int  rb0[3] = {tt.x * B, tt.y * B, tt.z * B};
    auto       b0f    = [&](int p) { return p == 0 ? rb0[0] : p == 1 ? rb0[1] : rb0[2]; };
    TP*        box    = reinterpret_cast<TP*>(em_dyn + st * em_stage_bytes<TP>());
    if(lane == 0) sm100::mbar_arrive_expect_tx(&full[st], (uint32_t) em_stage_bytes<TP>());
    __syncwarp();
    if(lane < EM_BOXES && !A.skip_loads) {
      const int  b = lane, pass = b / 6, q = b % 6;
      const int* P = c_perm[q];
      // (slowest, middle, fastest) block positions of the pass's array: P12[a][c][b],
      // P34[b][a][c], P56[c][b][a] with a, b, c in the blocks at positions P[0], P[1], P[2]
      const int q0 = pass == 0 ? P[0] : pass == 1 ? P[1] : P[2];
      const int q1 = pass == 0 ? P[2] : pass == 1 ? P[0] : P[1];
      const int q2 = pass == 0 ? P[1] : pass == 1 ? P[2] : P[0];
      // the stage was last read through the generic proxy; the TMA writes it through the async one
      sm100::fence_proxy_async_smem();
      sm100::tma_load_4d(box + (size_t) b * B3, &A.pmap, &full[st], b0f(q2), b0f(q1), b0f(q0), 3 * slot + pass);
    }
  };
  constexpr int kIssueWarp = EM_THREADS / 32 - 1;
  // every thread loads its share of a unit's singles data into registers
  auto prefetch = [&](int tile, EmPrefetch<SS, ES>& r) {
    const int3 tt     = A.tiles[tile];
    const int  rb0[3] = {tt.x * B, tt.y * B, tt.z * B};
    const int  rbn[3] = {min(B, v - rb0[0]), min(B, v - rb0[1]), min(B, v - rb0[2])};
    auto       b0f    = [&](int p) { return p == 0 ? rb0[0] : p == 1 ? rb0[1] : rb0[2]; };
    auto       bnf    = [&](int p) { return p == 0 ? rbn[0] : p == 1 ? rbn[1] : rbn[2]; };
#pragma unroll
    for(int h = 0; h < 2; h++) { // the six ordered pairs of distinct blocks, 64 entries each
      const int e = tid + h * EM_THREADS;
      r.o[h][0] = r.o[h][1] = r.o[h][2] = SS(0);
      if(e < 6 * B * B) {
        const int       pi = e / (B * B), uu = pi >> 1, ww = (pi & 1) ? (uu == 2 ? 1 : 2) : (uu == 0 ? 1 : 0);
        const int       x = (e / B) % B, y = e % B;
        const long long off = (long long) (b0f(uu) + x) * v + b0f(ww) + y;
        if(x < bnf(uu) && y < bnf(ww)) r.o[h][0] = gOjk[off], r.o[h][1] = gOik[off], r.o[h][2] = gOij[off];
      }
    }
    if(tid < 3 * B) {
      const int  uu = tid / B, x = tid % B;
      const bool ok = x < bnf(uu);
      const int  a  = b0f(uu) + x;
      r.t[0] = ok ? gt1[(long long) i * v + a] : SS(0);
      r.t[1] = ok ? gt1[(long long) j * v + a] : SS(0);
      r.t[2] = ok ? gt1[(long long) k * v + a] : SS(0);
      if constexpr(kF64) {
        r.ev = ok ? A.ev[a] : 0.0;
      } else {
        const ff e = ok ? ff_from_double(A.ev[a]) : ff{0.f, 0.f};
        r.ev       = make_float2(e.hi, e.lo);
      }
    } else if(tid >= 64 && tid < 64 + B * B) { // a in block 0, b in block 1
      const int x = (tid - 64) / B, y = (tid - 64) % B;
      if constexpr(kF64) {
        r.dab = eijk_d - (x < rbn[0] ? A.ev[rb0[0] + x] : 0.0) - (y < rbn[1] ? A.ev[rb0[1] + y] : 0.0);
      } else {
        const ff ea = x < rbn[0] ? ff_from_double(A.ev[rb0[0] + x]) : ff{0.f, 0.f};
        const ff eb = y < rbn[1] ? ff_from_double(A.ev[rb0[1] + y]) : ff{0.f, 0.f};
        const ff d  = ff_add(ff_add(eijk, ff_neg(ea)), ff_neg(eb));
        r.dab       = make_float2(d.hi, d.lo);
      }
      if(tid >= 96 && tid < 102) { // a cube counts once per distinct ordered block triple
        const int  t6 = tid - 96;
        const int* P  = c_perm[t6];
        r.on          = 1;
        for(int q = 0; q < t6; q++) {
          const int* Q = c_perm[q];
          if(b0f(P[0]) == b0f(Q[0]) && b0f(P[1]) == b0f(Q[1]) && b0f(P[2]) == b0f(Q[2])) r.on = 0;
        }
      }
    }
  };
  auto store = [&](const EmPrefetch<SS, ES>& r, EmSingles<SS, ES>& S_) {
#pragma unroll
    for(int h = 0; h < 2; h++) {
      const int e = tid + h * EM_THREADS;
      if(e < 6 * B * B) {
        const int pi = e / (B * B), uu = pi >> 1, ww = (pi & 1) ? (uu == 2 ? 1 : 2) : (uu == 0 ? 1 : 0);
        const int x = (e / B) % B, y = e % B;
        S_.Ojk[uu][ww][x * B + y] = r.o[h][0];
        S_.Oik[uu][ww][x * B + y] = r.o[h][1];
        S_.Oij[uu][ww][x * B + y] = r.o[h][2];
      }
    }
    if(tid < 3 * B) {
      const int uu = tid / B, x = tid % B;
      S_.ti[uu][x] = r.t[0], S_.tj[uu][x] = r.t[1], S_.tk[uu][x] = r.t[2];
      S_.evs[uu][x] = r.ev;
    } else if(tid >= 64 && tid < 64 + B * B) {
      S_.dab[tid - 64] = r.dab;
      if(tid >= 96 && tid < 102) S_.slot_on[tid - 96] = r.on;
    }
  };

  ff    s4{0.f, 0.f}, s5{0.f, 0.f};
  CSum  d4, d5; // the FP64 partial arrays' sums
  float sens = 0.f;
  // this thread's two orbits of every unit (warps g = warp and warp + 8)
  const int u = lane & 7, w = lane >> 3;
  int       la_[2], lb_[2], lc_[2];
#pragma unroll
  for(int h = 0; h < 2; h++) {
    const int g = warp + 8 * h;
    la_[h] = w + 4 * (g & 1), lb_[h] = u, lc_[h] = (u + w + (g >> 1)) & 7;
  }
  bool               failed = false;
  EmPrefetch<SS, ES> pre{};
  if((int) blockIdx.x < A.ntiles) {
    if(NST == 2 && warp == kIssueWarp) issue(blockIdx.x, 0);
    prefetch(blockIdx.x, pre);
  }
  // Pipeline: while unit n is evaluated, unit n + 1's singles data are in registers and (two
  // stages) its boxes in flight into the other stage.  The singles always have two stages.
  int n = 0;
  for(int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x, n++) {
    const int ss = n & 1, st = NST == 2 ? ss : 0;
    store(pre, sgl[ss]);
    __syncthreads(); // the unit's singles are visible; unit n - 1's orbits are done with its box stage
    const int next = tile + gridDim.x;
    // after a wait gave up the stages are not re-armed (their phases never completed); the issuing
    // warp decides as one
    const bool may_issue = warp == kIssueWarp && !__any_sync(0xffffffffu, failed);
    if(NST == 1 && may_issue) issue(tile, 0);
    if(next < A.ntiles) {
      if(NST == 2 && may_issue) issue(next, st ^ 1);
      prefetch(next, pre);
    }
    // Each thread waits for the boxes itself (the wait makes the TMA's writes visible to it).  A
    // thread whose wait gave up evaluates nothing more and waits no more, but keeps to the loop's
    // barriers, so no consensus is needed; the call then reports the timeout.
    const uint32_t parity = NST == 2 ? (n >> 1) & 1 : n & 1;
    if(!failed && !sm100::mbar_wait(&full[st], parity, A.spin)) failed = true;
    if(failed) continue;
    const EmSingles<SS, ES>& S_ = sgl[ss];
    const TP*                box = reinterpret_cast<const TP*>(em_dyn + st * em_stage_bytes<TP>());
    const int3               tt  = A.tiles[tile];
    const int                rbn[3] = {min(B, v - tt.x * B), min(B, v - tt.y * B), min(B, v - tt.z * B)};
    const bool all_on = S_.slot_on[0] & S_.slot_on[1] & S_.slot_on[2] & S_.slot_on[3] & S_.slot_on[4] & S_.slot_on[5];
#pragma unroll
    for(int h = 0; h < 2; h++) {
      const int la = la_[h], lb = lb_[h], lc = lc_[h];
      if(la >= rbn[0] || lb >= rbn[1] || lc >= rbn[2]) continue;
      const int loc[3] = {la, lb, lc};
      if constexpr(kF64) {
        double sg[6], wv[6];
        et_singles_f64(S_.Ojk, S_.Oik, S_.Oij, S_.ti, S_.tj, S_.tk, la, lb, lc, sg);
#pragma unroll
        for(int q = 0; q < 6; q++) {
          const int x = loc[kPerm(q, 0)], y = loc[kPerm(q, 1)], z = loc[kPerm(q, 2)];
          wv[q] = box[(0 * 6 + q) * B3 + (x * B + z) * B + y] + box[(1 * 6 + q) * B3 + (y * B + x) * B + z] +
                  box[(2 * 6 + q) * B3 + (z * B + y) * B + x];
        }
        et_orbit_values_f64(wv, sg, S_.evs, S_.dab, all_on, S_.slot_on, la, lb, lc, A.want_sens, d4, d5, sens);
        continue;
      } else {
      float sg[6];
      et_singles(S_.Ojk, S_.Oik, S_.Oij, S_.ti, S_.tj, S_.tk, la, lb, lc, sg);
      if constexpr(kF32) {
        float wv[6];
#pragma unroll
        for(int q = 0; q < 6; q++) {
          const int x = loc[kPerm(q, 0)], y = loc[kPerm(q, 1)], z = loc[kPerm(q, 2)];
          wv[q] = box[(0 * 6 + q) * B3 + (x * B + z) * B + y];
          wv[q] += box[(1 * 6 + q) * B3 + (y * B + x) * B + z];
          wv[q] += box[(2 * 6 + q) * B3 + (z * B + y) * B + x];
        }
        et_orbit_values_f32(wv, sg, S_.evs, S_.dab, all_on, S_.slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
      } else {
        ff wv[6];
#pragma unroll
        for(int q = 0; q < 6; q++) {
          const int    x = loc[kPerm(q, 0)], y = loc[kPerm(q, 1)], z = loc[kPerm(q, 2)];
          const float2 p12 = box[(0 * 6 + q) * B3 + (x * B + z) * B + y];
          const float2 p34 = box[(1 * 6 + q) * B3 + (y * B + x) * B + z];
          const float2 p56 = box[(2 * 6 + q) * B3 + (z * B + y) * B + x];
          // the pass-by-pass kernel's order: two-sum of the high words with the low words added,
          // then a float-float add of the third array
          const ff hs = ff_two_sum(p12.x, p34.x);
          wv[q]       = ff_add(ff{hs.hi, hs.lo + (p12.y + p34.y)}, ff{p56.x, p56.y});
        }
        et_orbit_values(wv, sg, S_.evs, S_.dab, all_on, S_.slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
      }
      }
    }
  }
  if(failed) atomicExch(A.err, 1);
  double* part = A.part + 6 * ((long long) slot * gridDim.x + blockIdx.x);
  CSum    c4, c5;
  if constexpr(kF64) {
    c4 = d4, c5 = d5;
  } else {
    c4.add((double) s4.hi);
    c4.add((double) s4.lo);
    c5.add((double) s5.hi);
    c5.add((double) s5.lo);
  }
  block_reduce_csum(c4, c5, part);
  __shared__ float ssum[EM_THREADS / 32];
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) sens += __shfl_down_sync(0xffffffffu, sens, off);
  if(lane == 0) ssum[warp] = sens;
  __syncthreads();
  if(tid == 0) {
    double t = 0.0;
    for(int q = 0; q < EM_THREADS / 32; q++) t += ssum[q];
    part[4] = t;
    part[5] = 0.0;
  }
}

} // namespace ccsdt
