// Tiled float-float energy of one occupied triplet (split-precision path).
//
// Restates the energy of ccsd_t_all_fused_cpu.hpp:597-619 in the closed-shell form
//   e = Z Y / D,  Z = 4 W_abc + W_bca + W_cab,  Y = 3 V_abc - V_acb - V_bac - V_cba,
//   W_xyz = P12[x][z][y] + P34[y][x][z] + P56[z][y][x]
// for every (a, b, c).  The virtual range is cut into blocks of 8; one work item is a sorted
// block triple X <= Y <= Z.  Its six ordered block cubes (the permutations of (X, Y, Z)) are
// summed from P12 / P34 / P56 into shared memory - each array read once, in runs of 8
// contiguous elements - so every permuted W an element needs is on chip.  The singles'
// integrals and amplitudes of the three blocks are staged too.  Work items are walked by a
// persistent grid in a fixed order; per-CTA float-float sums are written for a fixed-order
// reduction, so the result is deterministic.
#pragma once

#include <type_traits>

#include "fp64_kernels.cuh"
#include "ozaki.cuh"

namespace ccsdt {

constexpr int ET_B = 8, ET_THREADS = 256;

struct TiledEnergyArgs {
  const void *  P12, *P34, *P56; // float2 elements, or float for the FP32 form of the kernel
  const float * oovv, *t1; // FP32 copies
  const double *eo, *ev;
  const int3*   tiles;     // sorted block triples
  int           ntiles;
  int           o, v, i, j, k;
  double*       part;      // 6 doubles per CTA: E[T] (s, c), E(T) (s, c), sum (18 Y^2 + 12 Z^2) / D^2, 0
  int           want_sens; // accumulate the sensitivity sum (only for a-posteriori estimates)
};

// slot s <-> permutation (p0, p1, p2) of the block positions; for the ordering xyz of slot s,
// the slots of the orderings yzx, zxy (cyclic) and xzy, yxz, zyx (one transposition)
// (constexpr functions, folded at compile time inside the unrolled loops)
__host__ __device__ constexpr int kPerm(int s, int pos) {
  return pos == 0 ? s >> 1 : pos == 1 ? (s == 0 || s == 5 ? 1 : s == 1 || s == 3 ? 2 : 0) : (s == 1 || s == 4 ? 1 : s == 0 || s == 2 ? 2 : 0);
}
__host__ __device__ constexpr int kSlot(int p0, int p1, int p2) { return p0 * 2 + (p1 > p2 ? 1 : 0); }
// Shared-memory position of orbit coordinates (la, lb, lc) in a W cube: an XOR swizzle (linear over
// GF(2), a bijection on 0..511) under which every half-warp access the kernel makes - any two of
// the three coordinates varying, one over 0..7 and one over an aligned pair - touches 16 distinct
// bank pairs: bank bits = (lc ^ la ^ (lb & 6), (lb ^ la) & 1).
__host__ __device__ constexpr int kSwz(int la, int lb, int lc) {
  return (la << 6) | ((lb & 6) << 3) | (((lb ^ la) & 1) << 3) | ((lc ^ la ^ (lb & 6)) & 7);
}
__host__ __device__ constexpr int kCyc1(int s) { return kSlot(kPerm(s, 1), kPerm(s, 2), kPerm(s, 0)); }
__host__ __device__ constexpr int kCyc2(int s) { return kSlot(kPerm(s, 2), kPerm(s, 0), kPerm(s, 1)); }
__host__ __device__ constexpr int kXzy(int s) { return kSlot(kPerm(s, 0), kPerm(s, 2), kPerm(s, 1)); }
__host__ __device__ constexpr int kYxz(int s) { return kSlot(kPerm(s, 1), kPerm(s, 0), kPerm(s, 2)); }
__host__ __device__ constexpr int kZyx(int s) { return kSlot(kPerm(s, 2), kPerm(s, 1), kPerm(s, 0)); }
static_assert(kCyc1(0) == 3 && kCyc1(1) == 5 && kCyc1(2) == 1 && kCyc1(3) == 4 && kCyc1(4) == 0 && kCyc1(5) == 2, "");
static_assert(kCyc2(0) == 4 && kCyc2(1) == 2 && kCyc2(2) == 5 && kCyc2(3) == 0 && kCyc2(4) == 3 && kCyc2(5) == 1, "");
static_assert(kXzy(0) == 1 && kXzy(1) == 0 && kXzy(2) == 3 && kXzy(3) == 2 && kXzy(4) == 5 && kXzy(5) == 4, "");
static_assert(kYxz(0) == 2 && kYxz(1) == 4 && kYxz(2) == 0 && kYxz(3) == 5 && kYxz(4) == 1 && kYxz(5) == 3, "");
static_assert(kZyx(0) == 5 && kZyx(1) == 3 && kZyx(2) == 4 && kZyx(3) == 1 && kZyx(4) == 2 && kZyx(5) == 0, "");
static __device__ __constant__ int c_perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

__device__ __forceinline__ int perm_slot(int p0, int p1, int p2) {
  // (0,1,2)=0 (0,2,1)=1 (1,0,2)=2 (1,2,0)=3 (2,0,1)=4 (2,1,0)=5
  return p0 * 2 + (p1 > p2 ? 1 : 0);
}

// Singles part of V at the six orderings of an orbit: (jy|kz) t_i^x + (ix|kz) t_j^y + (ix|jy) t_k^z
// with (x, y, z) the ordering's local indices.
__device__ __forceinline__ void et_singles(const float (*Ojk)[3][ET_B * ET_B], const float (*Oik)[3][ET_B * ET_B],
                                           const float (*Oij)[3][ET_B * ET_B], const float (*ti)[ET_B],
                                           const float (*tj)[ET_B], const float (*tk)[ET_B], int la, int lb, int lc,
                                           float (&sg)[6]) {
  constexpr int B = ET_B;
  const int loc[3] = {la, lb, lc};
#pragma unroll
  for(int q = 0; q < 6; q++) {
    const int p0 = kPerm(q, 0), p1 = kPerm(q, 1), p2 = kPerm(q, 2);
    const int x = loc[p0], y = loc[p1], z = loc[p2];
    sg[q] = __fmaf_rn(Ojk[p1][p2][y * B + z], ti[p0][x],
                      __fmaf_rn(Oik[p0][p2][x * B + z], tj[p1][y], __fmul_rn(Oij[p0][p1][x * B + y], tk[p2][z])));
  }
}

// One orbit {a, b, c} of a work item: the index triple (la, lb, lc) local to the sorted block
// triple (a' in block 0, b' in block 1, c' in block 2) and all six of its orderings (the six
// slots q; w[q] = W at the ordering's indices).  D is common to the orbit, and an ordering counts
// only if its slot is a distinct ordered block triple (so every ordered (a, b, c) counts once).
// Adds the orbit's E[T] and E(T) terms to s4 / s5 and, with want_sens, its first-order
// sensitivity to sens.  Float-float W.
__device__ __forceinline__ void et_orbit_values(const ff (&w)[6], const float (&sg)[6], const float2 (*evs)[ET_B],
                                                const float2* dab, bool all_on, const int* slot_on, int la, int lb,
                                                int lc, int want_sens, ff& s4, ff& s5, float& sens) {
  constexpr int B = ET_B;
  // The six orderings form two cyclic classes, {q, yzx(q), zxy(q)} and the three orderings
  // one transposition away (xzy, yxz, zyx of q), which are the other class.  With the class
  // sums C: Z_q = 4 W_q + W_yzx + W_zxy = 3 W_q + C_own, Y_q = 3 V_q - C_other(V).
  const ff    ca  = ff_add(ff_add(w[0], w[3]), w[4]); // class of ordering 0: slots 0, 3, 4
  const ff    cb  = ff_add(ff_add(w[1], w[2]), w[5]); // slots 1, 2, 5
  const float sga = sg[0] + sg[3] + sg[4], sgb = sg[1] + sg[2] + sg[5];
  ff    zy4{0.f, 0.f}, zys{0.f, 0.f};
  float sn = 0.f;
  if(all_on) {
    // All six orderings count: the orbit sums follow from the class sums.
    //   sum_q Z_q Y4_q = 9 sum_q W_q^2 + 3 (C_a^2 + C_b^2) - 12 C_a C_b
    //   sum_q Z_q ys_q = 3 sum_q W_q ys_q + 3 (C_a - C_b)(S_a - S_b)
    // (class a: Z = 3 W + C_a, Y4 = 3 W - C_b, ys = 3 sg - S_b; class b with a and b swapped)
    ffacc sqa, wya;
#pragma unroll
    for(int q = 0; q < 6; q++) {
      const bool  in_a = q == 0 || q == 3 || q == 4;
      const float ys   = __fmaf_rn(3.f, sg[q], -(in_a ? sgb : sga));
      sqa.add_sq(w[q]);
      wya.add_mul_f(w[q], ys);
      if(want_sens) { // the estimate needs Z and Y only to float precision
        const float z  = __fmaf_rn(3.f, w[q].hi, in_a ? ca.hi : cb.hi);
        const float y5 = __fadd_rn(__fmaf_rn(3.f, w[q].hi, -(in_a ? cb.hi : ca.hi)), ys);
        sn = __fmaf_rn(__fmul_rn(18.f, y5), y5, __fmaf_rn(__fmul_rn(12.f, z), z, sn));
      }
    }
    const ff sq = sqa.get(), wy = wya.get();
    zy4 = ff_add(ff_add(ff_mul_f(sq, 9.f), ff_mul_f(ff_add(ff_mul(ca, ca), ff_mul(cb, cb)), 3.f)),
                 ff_neg(ff_mul_f(ff_mul(ca, cb), 12.f)));
    zys = ff_add(ff_mul_f(wy, 3.f), ff_mul_f(ff_add(ca, ff_neg(cb)), 3.f * (sga - sgb)));
  } else
#pragma unroll
  for(int q = 0; q < 6; q++) {
    if(!slot_on[q]) continue;
    const bool  in_a = q == 0 || q == 3 || q == 4;
    const ff    t3 = ff_mul_f(w[q], 3.f);
    const ff    z  = ff_add(t3, in_a ? ca : cb);
    const ff    y4 = ff_add(t3, ff_neg(in_a ? cb : ca));
    const float ys = __fmaf_rn(3.f, sg[q], -(in_a ? sgb : sga)); // singles part of Y
    zy4 = ff_add(zy4, ff_mul(z, y4));
    zys = ff_add(zys, ff_mul_f(z, ys));
    // first-order sensitivity to errors in W: W_abc enters Z_abc (x4), Z_bca, Z_cab and,
    // through V, Y_abc (x3), Y_acb, Y_bac, Y_cba; with uncorrelated signs
    //   |dE/dW|^2 ~ (16 + 1 + 1) Y^2 / D^2 + (9 + 1 + 1 + 1) Z^2 / D^2
    if(want_sens) {
      const float y5 = __fadd_rn(y4.hi, ys);
      sn = __fmaf_rn(__fmul_rn(18.f, y5), y5, __fmaf_rn(__fmul_rn(12.f, z.hi), z.hi, sn));
    }
  }
  const ff zy5 = ff_add(zy4, zys);
  const float2 dd = dab[la * B + lb], ec = evs[2][lc];
  const ff     id = ff_div_fast(ff{1.f, 0.f}, ff_add(ff{dd.x, dd.y}, ff{-ec.x, -ec.y})); // 1 / D (orbit-wide)
  s4   = ff_add(s4, ff_mul(zy4, id));
  s5   = ff_add(s5, ff_mul(zy5, id));
  sens = __fmaf_rn(__fmul_rn(sn, id.hi), id.hi, sens);
}

__device__ __forceinline__ void et_orbit(const float2 (*W)[ET_B * ET_B * ET_B], const float (*Ojk)[3][ET_B * ET_B],
                                         const float (*Oik)[3][ET_B * ET_B], const float (*Oij)[3][ET_B * ET_B],
                                         const float (*ti)[ET_B], const float (*tj)[ET_B], const float (*tk)[ET_B],
                                         const float2 (*evs)[ET_B], const float2* dab, bool all_on, const int* slot_on,
                                         int la, int lb, int lc, int want_sens, ff& s4, ff& s5, float& sens) {
  ff    w[6];
  float sg[6];
#pragma unroll
  for(int q = 0; q < 6; q++) {
    const float2 t = W[q][kSwz(la, lb, lc)]; // = W at the ordering's local (x, y, z) of slot q
    w[q]           = ff{t.x, t.y};
  }
  et_singles(Ojk, Oik, Oij, ti, tj, tk, la, lb, lc, sg);
  et_orbit_values(w, sg, evs, dab, all_on, slot_on, la, lb, lc, want_sens, s4, s5, sens);
}

// The same orbit from FP32 partial arrays (P stored rounded to FP32: the split path at few digit
// planes, whose own contraction error is far above FP32's rounding).  Z and Y per ordering in FP32
// (Z = 3 W + C_own, Y4 = 3 W - C_other directly: no class-sum identity, whose terms cancel), the
// orbit's six products summed in FP32, one correctly rounded reciprocal of D, and the orbit's
// share added to the thread's float-float sums.  The rounding errors are unbiased and average out
// over the v^3 / 6 orbits of a triplet.
__device__ __forceinline__ void et_orbit_values_f32(const float (&w)[6], const float (&sg)[6],
                                                    const float2 (*evs)[ET_B], const float2* dab, bool all_on,
                                                    const int* slot_on, int la, int lb, int lc, int want_sens, ff& s4,
                                                    ff& s5, float& sens) {
  constexpr int B = ET_B;
  const float ca = w[0] + w[3] + w[4], cb = w[1] + w[2] + w[5]; // the two cyclic classes
  const float sga = sg[0] + sg[3] + sg[4], sgb = sg[1] + sg[2] + sg[5];
  float       zy4 = 0.f, zys = 0.f, sn = 0.f;
#pragma unroll
  for(int q = 0; q < 6; q++) {
    if(!all_on && !slot_on[q]) continue;
    const bool  in_a = q == 0 || q == 3 || q == 4;
    const float z    = __fmaf_rn(3.f, w[q], in_a ? ca : cb);
    const float y4   = __fmaf_rn(3.f, w[q], -(in_a ? cb : ca));
    const float ys   = __fmaf_rn(3.f, sg[q], -(in_a ? sgb : sga));
    zy4              = __fmaf_rn(z, y4, zy4);
    zys              = __fmaf_rn(z, ys, zys);
    if(want_sens) {
      const float y5 = __fadd_rn(y4, ys);
      sn             = __fmaf_rn(__fmul_rn(18.f, y5), y5, __fmaf_rn(__fmul_rn(12.f, z), z, sn));
    }
  }
  const float2 dd = dab[la * B + lb], ec = evs[2][lc];
  const float  id = __frcp_rn(ff_add(ff{dd.x, dd.y}, ff{-ec.x, -ec.y}).hi); // 1 / D
  s4   = ff_add_f(s4, __fmul_rn(zy4, id));
  s5   = ff_add_f(s5, __fmul_rn(__fadd_rn(zy4, zys), id));
  sens = __fmaf_rn(__fmul_rn(sn, id), id, sens);
}

__device__ __forceinline__ void et_orbit_f32(const float (*W)[ET_B * ET_B * ET_B], const float (*Ojk)[3][ET_B * ET_B],
                                             const float (*Oik)[3][ET_B * ET_B], const float (*Oij)[3][ET_B * ET_B],
                                             const float (*ti)[ET_B], const float (*tj)[ET_B], const float (*tk)[ET_B],
                                             const float2 (*evs)[ET_B], const float2* dab, bool all_on,
                                             const int* slot_on, int la, int lb, int lc, int want_sens, ff& s4, ff& s5,
                                             float& sens) {
  float w[6], sg[6];
#pragma unroll
  for(int q = 0; q < 6; q++) w[q] = W[q][kSwz(la, lb, lc)];
  et_singles(Ojk, Oik, Oij, ti, tj, tk, la, lb, lc, sg);
  et_orbit_values_f32(w, sg, evs, dab, all_on, slot_on, la, lb, lc, want_sens, s4, s5, sens);
}

// TP = float2: float-float partial arrays; TP = float: FP32 partial arrays
template<typename TP>
__device__ __forceinline__ void energy_tiled_body(const TiledEnergyArgs& A, const TP* P12, const TP* P34, const TP* P56,
                                                  int i, int j, int k, double* part, int gblock, int gsize) {
  constexpr int  B = ET_B, B3 = B * B * B;
  constexpr bool kF32 = std::is_same<TP, float>::value;
  __shared__ TP  W[6][B3];               // [slot][a'][b'][c'] (a', b', c' local to the slot's blocks)
  __shared__ float  Ojk[3][3][B * B], Oik[3][3][B * B], Oij[3][3][B * B];
  __shared__ float  ti[3][B], tj[3][B], tk[3][B];
  __shared__ float2 evs[3][B];
  __shared__ float2 dab[B * B];          // e_i + e_j + e_k - e_a - e_b (float-float), a in block 0, b in block 1
  __shared__ int    slot_on[6];
  __shared__ long long cube0[3][6];      // offset of the slot's local (0, 0, 0) in pass p's array

  const int       v = A.v, o = A.o, tid = threadIdx.x;
  const long long v2 = (long long) v * v;
  const ff        eijk = ff_add(ff_add(ff_from_double(A.eo[i]), ff_from_double(A.eo[j])), ff_from_double(A.eo[k]));
  const float *   gOjk = A.oovv + ((long long) j * o + k) * v2, *gOik = A.oovv + ((long long) i * o + k) * v2,
              *gOij = A.oovv + ((long long) i * o + j) * v2;
  ff    s4{0.f, 0.f}, s5{0.f, 0.f};
  float sens = 0.f; // first-order sensitivity of the energy to errors in W (a-posteriori estimate)
  // this thread's cube positions r = tid and tid + 256: local (slowest, middle, fastest) index
  // (r / 64, r / 8 % 8, r % 8) of every pass's array, as an element offset
  const long long rel0 = ((long long) (tid >> 6) * v + ((tid >> 3) & 7)) * v + (tid & 7), rel1 = rel0 + 4 * v2;

  for(int tile = gblock; tile < A.ntiles; tile += gsize) {
    // every thread reads the block triple (one broadcast load) and keeps its bounds in registers
    const int3 tt    = A.tiles[tile];
    const int  rb0[3] = {tt.x * B, tt.y * B, tt.z * B};
    const int  rbn[3] = {min(B, v - rb0[0]), min(B, v - rb0[1]), min(B, v - rb0[2])};
    auto       b0    = [&](int u) { return u == 0 ? rb0[0] : u == 1 ? rb0[1] : rb0[2]; };
    auto       bn    = [&](int u) { return u == 0 ? rbn[0] : u == 1 ? rbn[1] : rbn[2]; };
    __syncthreads(); // the previous item's orbits are done with the shared arrays
    if(tid >= 96 && tid < 102) { // a slot counts once per distinct ordered block triple
      const int  t6 = tid - 96;
      const int* P  = c_perm[t6];
      int        on = 1;
      for(int q = 0; q < t6; q++) {
        const int* Q = c_perm[q];
        if(b0(P[0]) == b0(Q[0]) && b0(P[1]) == b0(Q[1]) && b0(P[2]) == b0(Q[2])) on = 0;
      }
      slot_on[t6] = on;
    } else if(tid >= 32 && tid < 50) { // pass p reads its array with (slowest, middle, fastest)
      const int  pp = (tid - 32) / 6, sl = (tid - 32) % 6; // = blocks (P0, P2, P1) / (P1, P0, P2) / (P2, P1, P0)
      const int* P  = c_perm[sl];
      const int  q0 = pp == 0 ? P[0] : pp == 1 ? P[1] : P[2], q1 = pp == 0 ? P[2] : pp == 1 ? P[0] : P[1],
                 q2 = pp == 0 ? P[1] : pp == 1 ? P[2] : P[0];
      cube0[pp][sl] = ((long long) b0(q0) * v + b0(q1)) * v + b0(q2);
    }
    // singles data of the three blocks: the orbits read the six ordered pairs of distinct blocks
    for(int e = tid; e < 6 * B * B; e += ET_THREADS) {
      const int pi = e / (B * B), u = pi >> 1, w = (pi & 1) ? (u == 2 ? 1 : 2) : (u == 0 ? 1 : 0);
      const int x = (e / B) % B, y = e % B;
      const bool ok = x < bn(u) && y < bn(w);
      const long long off = (long long) (b0(u) + x) * v + b0(w) + y;
      Ojk[u][w][x * B + y] = ok ? gOjk[off] : 0.f;
      Oik[u][w][x * B + y] = ok ? gOik[off] : 0.f;
      Oij[u][w][x * B + y] = ok ? gOij[off] : 0.f;
    }
    if(tid < 3 * B) {
      const int u = tid / B, x = tid % B;
      const bool ok = x < bn(u);
      const int  a = b0(u) + x;
      ti[u][x] = ok ? A.t1[(long long) i * v + a] : 0.f;
      tj[u][x] = ok ? A.t1[(long long) j * v + a] : 0.f;
      tk[u][x] = ok ? A.t1[(long long) k * v + a] : 0.f;
      const ff e = ok ? ff_from_double(A.ev[a]) : ff{0.f, 0.f};
      evs[u][x] = make_float2(e.hi, e.lo);
    }
    __syncthreads();
    if(tid < B * B) { // the orbit-wide part of D: a in block 0, b in block 1
      const int    x = tid / B, y = tid % B;
      const float2 ea = evs[0][x], eb = evs[1][y];
      const ff     d  = ff_add(ff_add(eijk, ff{-ea.x, -ea.y}), ff{-eb.x, -eb.y});
      dab[tid]        = make_float2(d.hi, d.lo);
    }
    // W of the six slots, stored by orbit coordinates (loc[P[0]], loc[P[1]], loc[P[2]]) = the
    // slot's local (a', b', c'): three passes, each reading one array along its contiguous index
    // (a thread's 12 loads of a pass are issued before its shared-memory updates).  Thread tid
    // handles local positions r = tid and tid + 256 of every slot: (slowest, middle, fastest)
    // local index of the pass's array = (r / 64, r / 8 % 8, r % 8).
    static_assert(6 * B3 == 12 * ET_THREADS, "two positions of each of the six cubes per thread");
    TP*        Wf   = &W[0][0];
    const bool full = rbn[0] == B && rbn[1] == B && rbn[2] == B;
    // pass p's loads (a thread's 12, all issued before any of them is used)
    auto load_pass = [&](auto pass_tag, TP (&x)[12], int (&widx)[12]) {
      constexpr int pass = decltype(pass_tag)::value;
#pragma unroll
      for(int it = 0; it < 12; it++) {
        const int s = it >> 1, r = tid + (it & 1) * ET_THREADS;
        const int P0 = kPerm(s, 0), P1 = kPerm(s, 1), P2 = kPerm(s, 2);
        const int f = r & 7, m = (r >> 3) & 7, sl = r >> 6;
        int       la, lb, lc; // slot-local (a', b', c'): a in block P0, b in P1, c in P2
        const TP* src;
        if(pass == 0) { // P12[a][c][b]: b fastest
          la = sl, lc = m, lb = f;
          src = P12;
        } else if(pass == 1) { // P34[b][a][c]: c fastest
          lb = sl, la = m, lc = f;
          src = P34;
        } else { // P56[c][b][a]: a fastest
          lc = sl, lb = m, la = f;
          src = P56;
        }
        // (sl, m, f) of this thread do not depend on the tile: local offset rel0 (+ 4 v^2 for r >= 256)
        const long long off = cube0[pass][s] + (it & 1 ? rel1 : rel0);
        const bool      ok  = full || (la < rbn[P0] && lb < rbn[P1] && lc < rbn[P2]);
        x[it]               = ok ? src[off] : TP{};
        if(it & 1) {
          // r + 256 sets bit 2 of the pass's slowest coordinate (sl < 4 for r < 256); kSwz is
          // linear over GF(2) with disjoint fields, so the index changes by a constant XOR
          const int q = pass == 0 ? P0 : pass == 1 ? P1 : P2; // argument of kSwz holding sl
          widx[it]    = widx[it - 1] ^ (q == 0 ? 260 : q == 1 ? 36 : 4);
        } else {
          int loc[3] = {0, 0, 0};
          loc[P0] = la, loc[P1] = lb, loc[P2] = lc;
          widx[it] = s * B3 + kSwz(loc[0], loc[1], loc[2]);
        }
      }
    };
    // pass p's shared-memory updates
    auto apply_pass = [&](auto pass_tag, const TP (&x)[12], const int (&widx)[12]) {
      constexpr int pass = decltype(pass_tag)::value;
#pragma unroll
      for(int it = 0; it < 12; it++) {
        if constexpr(kF32) {
          if(pass == 0) Wf[widx[it]] = x[it];
          else Wf[widx[it]] += x[it];
        } else if(pass == 0) Wf[widx[it]] = x[it];
        else if(pass == 1) { // two-sum of the high words, low words added; renormalised in pass 2
          const float2 o = Wf[widx[it]];
          const ff     h = ff_two_sum(o.x, x[it].x);
          Wf[widx[it]]   = make_float2(h.hi, h.lo + (o.y + x[it].y));
        } else {
          const float2 o = Wf[widx[it]];
          const ff     r = ff_add(ff{o.x, o.y}, ff{x[it].x, x[it].y});
          Wf[widx[it]]   = make_float2(r.hi, r.lo);
        }
      }
    };
    // The next pass's loads are issued before the barrier that separates the passes' updates, so
    // their latency overlaps the wait.  Pass 0 needs no barrier before it: the one after the
    // staging made cube0 visible, and the previous item's orbits finished with W before the
    // barrier at the top of the item.
    {
      TP  x[12];
      int widx[12];
      load_pass(std::integral_constant<int, 0>{}, x, widx);
      apply_pass(std::integral_constant<int, 0>{}, x, widx);
      load_pass(std::integral_constant<int, 1>{}, x, widx);
      __syncthreads();
      apply_pass(std::integral_constant<int, 1>{}, x, widx);
      load_pass(std::integral_constant<int, 2>{}, x, widx);
      __syncthreads();
      apply_pass(std::integral_constant<int, 2>{}, x, widx);
    }
    __syncthreads();
    // energies by orbit: a thread takes one index triple (a' in block 0, b' in block 1, c' in
    // block 2 of the sorted triple) and all six of its orderings, which live in the six slots.
    // The six W values are read once, D is common to the orbit, and an ordering counts only if
    // its slot is a distinct ordered block triple (so every ordered (a, b, c) counts once).
    const bool all_on = slot_on[0] & slot_on[1] & slot_on[2] & slot_on[3] & slot_on[4] & slot_on[5];
    for(int r = tid; r < B3; r += ET_THREADS) {
      const int la = r / (B * B), lb = (r / B) % B, lc = r % B;
      if(la >= rbn[0] || lb >= rbn[1] || lc >= rbn[2]) continue;
      if constexpr(kF32)
        et_orbit_f32(W, Ojk, Oik, Oij, ti, tj, tk, evs, dab, all_on, slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
      else
        et_orbit(W, Ojk, Oik, Oij, ti, tj, tk, evs, dab, all_on, slot_on, la, lb, lc, A.want_sens, s4, s5, sens);
    }
  }
  CSum c4, c5;
  c4.add((double) s4.hi);
  c4.add((double) s4.lo);
  c5.add((double) s5.hi);
  c5.add((double) s5.lo);
  block_reduce_csum(c4, c5, part);
  // fixed-order block sum of the sensitivity
  __shared__ float ssum[ET_THREADS / 32];
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) sens += __shfl_down_sync(0xffffffffu, sens, off);
  if((threadIdx.x & 31) == 0) ssum[threadIdx.x >> 5] = sens;
  __syncthreads();
  if(threadIdx.x == 0) {
    double t = 0.0;
    for(int q = 0; q < ET_THREADS / 32; q++) t += ssum[q];
    part[4] = t;
    part[5] = 0.0;
  }
}

template<typename TP>
static __global__ void __launch_bounds__(ET_THREADS, 4) energy_tiled_kernel(const __grid_constant__ TiledEnergyArgs A) {
  energy_tiled_body<TP>(A, static_cast<const TP*>(A.P12), static_cast<const TP*>(A.P34), static_cast<const TP*>(A.P56),
                        A.i, A.j, A.k, A.part + 6 * (long long) blockIdx.x, blockIdx.x, gridDim.x);
}

// Batched form: blockIdx.y = triplet slot; the triplet and its P arrays come from the batch
// tables (4 ints per triplet: i, j, k, output index; P arrays of slot s at F + s * 3 v^3 elements
// of TP: float2 for float-float, float for FP32 partial arrays).
struct BatchEnergyArgs {
  TiledEnergyArgs base_args; // P12/P34/P56/i/j/k/part unused
  const int*      tri;
  const int*      base;
  const void*     F;
  double*         part;      // [slot][gridDim.x][6]
};

template<typename TP>
static __global__ void __launch_bounds__(ET_THREADS, 4) energy_tiled_batch_kernel(const __grid_constant__ BatchEnergyArgs A) {
  const int       slot = blockIdx.y, b0 = A.base ? *A.base : 0;
  const int*      tp   = A.tri + 4 * (b0 + slot);
  const long long v3   = (long long) A.base_args.v * A.base_args.v * A.base_args.v;
  const TP*       F    = static_cast<const TP*>(A.F) + (long long) slot * 3 * v3;
  energy_tiled_body<TP>(A.base_args, F, F + v3, F + 2 * v3, tp[0], tp[1], tp[2],
                        A.part + 6 * ((long long) slot * gridDim.x + blockIdx.x), blockIdx.x, gridDim.x);
}

// Fixed-order parallel sum of per-CTA partials (6 doubles each) for one triplet -> out[2]
// (energies); sens_out[0] (optional) receives scale * the summed sensitivity.
static __global__ void __launch_bounds__(256) reduce_parts_parallel_kernel(const double* part, int nparts, double scale,
                                                                     double* out, double* sens_out) {
  CSum a, b;
  const int per = (nparts + blockDim.x - 1) / blockDim.x;
  const int q0 = threadIdx.x * per, q1 = min(nparts, q0 + per);
  for(int q = q0; q < q1; q++) {
    a.add(part[6 * q + 0]);
    a.c += part[6 * q + 1];
    b.add(part[6 * q + 2]);
    b.c += part[6 * q + 3];
  }
  if(sens_out && threadIdx.x == 0) { // sensitivity of the scaled energy: scale^2 * sum of squares
    double t = 0.0;
    for(int q = 0; q < nparts; q++) t += part[6 * q + 4];
    sens_out[0] = scale * scale * t;
  }
  __shared__ double tmp[4];
  // reuse the fixed-shape block reduction (its shared scratch is sized for 256 threads)
  block_reduce_csum(a, b, tmp);
  __syncthreads();
  if(threadIdx.x == 0) {
    out[0] = scale * (tmp[0] + tmp[1]);
    out[1] = scale * (tmp[2] + tmp[3]);
  }
}

// One block per slot: fixed-order sum of that slot's partials; writes etrip[2 out] (scaled by
// m / 9) and, if given, sens[out].
static __global__ void __launch_bounds__(256) reduce_parts_batch_kernel(const double* part, int nparts, const int* tri,
                                                                 const int* base, double* etrip, double* sens) {
  const int  slot = blockIdx.x, b0 = base ? *base : 0;
  const int* tp   = tri + 4 * (b0 + slot);
  const int  i = tp[0], j = tp[1], k = tp[2], out = tp[3];
  const int  m = (i == j && j == k) ? 1 : ((i == j || j == k || i == k) ? 3 : 6);
  const double* pp = part + 6 * (long long) slot * nparts;
  CSum a, b;
  const int per = (nparts + blockDim.x - 1) / blockDim.x;
  const int q0 = threadIdx.x * per, q1 = min(nparts, q0 + per);
  for(int q = q0; q < q1; q++) {
    a.add(pp[6 * q + 0]);
    a.c += pp[6 * q + 1];
    b.add(pp[6 * q + 2]);
    b.c += pp[6 * q + 3];
  }
  __shared__ double tmp[4];
  block_reduce_csum(a, b, tmp);
  __syncthreads();
  if(threadIdx.x == 0) {
    const double sc = m / 9.0;
    etrip[2 * out]     = sc * (tmp[0] + tmp[1]);
    etrip[2 * out + 1] = sc * (tmp[2] + tmp[3]);
    if(sens) {
      double t = 0.0;
      for(int q = 0; q < nparts; q++) t += pp[6 * q + 4];
      sens[out] = sc * sc * t;
    }
  }
}

static __global__ void advance_base_kernel(int* base, int by) {
  if(threadIdx.x == 0 && blockIdx.x == 0) *base += by;
}

} // namespace ccsdt
