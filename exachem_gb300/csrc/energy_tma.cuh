// Tiled energy of a batch of triplets with the partial arrays staged by TMA (split-precision path).
//
// The same work units and orbit arithmetic as energy_tiled.cuh (one sorted 8-wide virtual block
// triple X <= Y <= Z per unit, W_xyz = P12[x][z][y] + P34[y][x][z] + P56[z][y][x], every orbit
// {a, b, c} with its six orderings), but the eighteen 8 x 8 x 8 boxes a unit needs - for each of
// its six ordered cubes, the matching box of P12, P34 and P56 - are copied into shared memory by
// eighteen TMA tensor loads issued by one thread, so no thread computes an address into the
// partial arrays and out-of-range rows (v not a multiple of 8) arrive as zeros.  The orbits then
// read their W values from the boxes directly: cube q of the unit at its local (x, y, z) is
// box12_q[x][z][y] + box34_q[y][x][z] + box56_q[z][y][x], summed in the order of the
// pass-by-pass kernel, so both kernels give the same W bit for bit.
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
};

// bytes of dynamic shared memory: the eighteen boxes
template<typename TP>
constexpr size_t em_smem_bytes() {
  return (size_t) EM_BOXES * ET_B * ET_B * ET_B * sizeof(TP);
}

template<typename TP>
static __global__ void __launch_bounds__(EM_THREADS, std::is_same<TP, float>::value ? 4 : 2)
  energy_tma_batch_kernel(const __grid_constant__ TmaEnergyArgs A) {
  constexpr int  B = ET_B, B3 = B * B * B;
  constexpr bool kF32 = std::is_same<TP, float>::value;
  extern __shared__ __align__(128) unsigned char em_dyn[];
  TP* box = reinterpret_cast<TP*>(em_dyn); // [pass][slot q][512]: pass 0 = P12, 1 = P34, 2 = P56
  __shared__ float    Ojk[3][3][B * B], Oik[3][3][B * B], Oij[3][3][B * B];
  __shared__ float    ti[3][B], tj[3][B], tk[3][B];
  __shared__ float2   evs[3][B];
  __shared__ float2   dab[B * B];
  __shared__ int      slot_on[6];
  __shared__ uint64_t full;
  __shared__ int      failed;

  const int       slot = blockIdx.y, b0 = A.base ? *A.base : 0;
  const int*      tp   = A.tri + 4 * (b0 + slot);
  const int       i = tp[0], j = tp[1], k = tp[2];
  const int       v = A.v, o = A.o, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long v2 = (long long) v * v;
  const ff        eijk = ff_add(ff_add(ff_from_double(A.eo[i]), ff_from_double(A.eo[j])), ff_from_double(A.eo[k]));
  const float *   gOjk = A.oovv + ((long long) j * o + k) * v2, *gOik = A.oovv + ((long long) i * o + k) * v2,
              *gOij = A.oovv + ((long long) i * o + j) * v2;
  if(tid == 0) {
    sm100::mbar_init(&full, 1);
    sm100::mbar_fence_init();
    sm100::prefetch_tmap(&A.pmap);
    failed = 0;
  }
  __syncthreads();
  ff       s4{0.f, 0.f}, s5{0.f, 0.f};
  float    sens  = 0.f;
  uint32_t phase = 0;
  // this thread's two orbits of every unit (warps g = warp and warp + 8)
  const int u = lane & 7, w = lane >> 3;
  int       la_[2], lb_[2], lc_[2];
#pragma unroll
  for(int h = 0; h < 2; h++) {
    const int g = warp + 8 * h;
    la_[h] = w + 4 * (g & 1), lb_[h] = u, lc_[h] = (u + w + (g >> 1)) & 7;
  }

  for(int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    const int3 tt     = A.tiles[tile];
    const int  rb0[3] = {tt.x * B, tt.y * B, tt.z * B};
    const int  rbn[3] = {min(B, v - rb0[0]), min(B, v - rb0[1]), min(B, v - rb0[2])};
    auto       b0f    = [&](int p) { return p == 0 ? rb0[0] : p == 1 ? rb0[1] : rb0[2]; };
    auto       bnf    = [&](int p) { return p == 0 ? rbn[0] : p == 1 ? rbn[1] : rbn[2]; };
    __syncthreads(); // the previous unit's orbits are done with the boxes and the singles
    if(tid == 0) {
      // the boxes were last read through the generic proxy; the TMA writes them through the async one
      sm100::fence_proxy_async_smem();
      sm100::mbar_arrive_expect_tx(&full, (uint32_t) em_smem_bytes<TP>());
#pragma unroll 1
      for(int b = 0; b < EM_BOXES; b++) {
        const int  pass = b / 6, q = b % 6;
        const int* P    = c_perm[q];
        // (slowest, middle, fastest) block positions of the pass's array: P12[a][c][b],
        // P34[b][a][c], P56[c][b][a] with a, b, c in the blocks at positions P[0], P[1], P[2]
        const int q0 = pass == 0 ? P[0] : pass == 1 ? P[1] : P[2];
        const int q1 = pass == 0 ? P[2] : pass == 1 ? P[0] : P[1];
        const int q2 = pass == 0 ? P[1] : pass == 1 ? P[2] : P[0];
        sm100::tma_load_4d(box + (size_t) b * B3, &A.pmap, &full, b0f(q2), b0f(q1), b0f(q0), 3 * slot + pass);
      }
    } else if(tid >= 96 && tid < 102) { // a slot counts once per distinct ordered block triple
      const int  t6 = tid - 96;
      const int* P  = c_perm[t6];
      int        on = 1;
      for(int q = 0; q < t6; q++) {
        const int* Q = c_perm[q];
        if(b0f(P[0]) == b0f(Q[0]) && b0f(P[1]) == b0f(Q[1]) && b0f(P[2]) == b0f(Q[2])) on = 0;
      }
      slot_on[t6] = on;
    }
    // singles data of the three blocks (the orbits read the six ordered pairs of distinct blocks)
    for(int e = tid; e < 6 * B * B; e += EM_THREADS) {
      const int       pi = e / (B * B), uu = pi >> 1, ww = (pi & 1) ? (uu == 2 ? 1 : 2) : (uu == 0 ? 1 : 0);
      const int       x = (e / B) % B, y = e % B;
      const bool      ok  = x < bnf(uu) && y < bnf(ww);
      const long long off = (long long) (b0f(uu) + x) * v + b0f(ww) + y;
      Ojk[uu][ww][x * B + y] = ok ? gOjk[off] : 0.f;
      Oik[uu][ww][x * B + y] = ok ? gOik[off] : 0.f;
      Oij[uu][ww][x * B + y] = ok ? gOij[off] : 0.f;
    }
    if(tid < 3 * B) {
      const int  uu = tid / B, x = tid % B;
      const bool ok = x < bnf(uu);
      const int  a  = b0f(uu) + x;
      ti[uu][x] = ok ? A.t1[(long long) i * v + a] : 0.f;
      tj[uu][x] = ok ? A.t1[(long long) j * v + a] : 0.f;
      tk[uu][x] = ok ? A.t1[(long long) k * v + a] : 0.f;
      const ff e = ok ? ff_from_double(A.ev[a]) : ff{0.f, 0.f};
      evs[uu][x] = make_float2(e.hi, e.lo);
    } else if(tid >= 64 && tid < 64 + B * B) { // the orbit-wide part of D: a in block 0, b in block 1
      const int x = (tid - 64) / B, y = (tid - 64) % B;
      const ff  ea = x < rbn[0] ? ff_from_double(A.ev[rb0[0] + x]) : ff{0.f, 0.f};
      const ff  eb = y < rbn[1] ? ff_from_double(A.ev[rb0[1] + y]) : ff{0.f, 0.f};
      const ff  d  = ff_add(ff_add(eijk, ff_neg(ea)), ff_neg(eb));
      dab[tid - 64] = make_float2(d.hi, d.lo);
    }
    // the boxes: every thread waits (bounded) for the unit's TMA bytes
    const bool ok = sm100::mbar_wait(&full, phase, A.spin);
    phase ^= 1;
    if(!ok) failed = 1;
    __syncthreads(); // singles staged; every thread's wait has finished
    if(failed) break;
    const bool all_on = slot_on[0] & slot_on[1] & slot_on[2] & slot_on[3] & slot_on[4] & slot_on[5];
#pragma unroll
    for(int h = 0; h < 2; h++) {
      const int la = la_[h], lb = lb_[h], lc = lc_[h];
      if(la >= rbn[0] || lb >= rbn[1] || lc >= rbn[2]) continue;
      const int loc[3] = {la, lb, lc};
      float     sg[6];
      et_singles(Ojk, Oik, Oij, ti, tj, tk, la, lb, lc, sg);
      if constexpr(kF32) {
        float wv[6];
#pragma unroll
        for(int q = 0; q < 6; q++) {
          const int x = loc[kPerm(q, 0)], y = loc[kPerm(q, 1)], z = loc[kPerm(q, 2)];
          wv[q] = box[(0 * 6 + q) * B3 + (x * B + z) * B + y];
          wv[q] += box[(1 * 6 + q) * B3 + (y * B + x) * B + z];
          wv[q] += box[(2 * 6 + q) * B3 + (z * B + y) * B + x];
        }
        et_orbit_values_f32(wv, sg, evs, dab, all_on, slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
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
          const ff h = ff_two_sum(p12.x, p34.x);
          wv[q]      = ff_add(ff{h.hi, h.lo + (p12.y + p34.y)}, ff{p56.x, p56.y});
        }
        et_orbit_values(wv, sg, evs, dab, all_on, slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
      }
    }
  }
  if(failed && tid == 0) atomicExch(A.err, 1);
  double* part = A.part + 6 * ((long long) slot * gridDim.x + blockIdx.x);
  CSum    c4, c5;
  c4.add((double) s4.hi);
  c4.add((double) s4.lo);
  c5.add((double) s5.hi);
  c5.add((double) s5.lo);
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
