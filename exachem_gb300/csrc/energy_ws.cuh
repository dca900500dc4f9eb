// Warp-specialised form of the batched float-float energy (the arithmetic of energy_tiled_body,
// same work items, same orbits): 4 producer warps stage the next work item - the six W cubes
// summed from P12 / P34 / P56, the singles' integrals and amplitudes, the orbit-wide part of D -
// into one of two shared-memory buffers while 8 consumer warps evaluate the orbits of the current
// item from the other.  In the block-synchronous kernel every thread stages and then evaluates,
// with five CTA barriers per item; here the consumers meet the producers only at the hand-over of
// a buffer, so the producers' global-load latency and their pass barriers overlap the consumers'
// arithmetic.
//
// Hand-over by named barriers: the side that fills (producers) or frees (consumers) a buffer
// arrives (bar.arrive), the side that needs it waits (bar.sync), 384 threads each time.  Both
// sides walk the same item sequence and the consumers free a buffer only when the producers will
// fill it again (items n + 2 < count), so every barrier phase that is started also completes.
#pragma once

#include "energy_tiled.cuh"

namespace ccsdt {

constexpr int EW_PROD = 128, EW_CONS = 256, EW_THREADS = EW_PROD + EW_CONS;
// named barrier ids (0 is __syncthreads): producers among themselves, buffer b full (2 + b),
// buffer b free (4 + b), consumers among themselves
constexpr int EW_BAR_PROD = 1, EW_BAR_FULL = 2, EW_BAR_FREE = 4, EW_BAR_CONS = 6;

// one staged work item
struct EwStage {
  float2    W[6][ET_B * ET_B * ET_B];       // [slot][swizzled orbit coordinates], float-float
  float     Ojk[3][3][ET_B * ET_B], Oik[3][3][ET_B * ET_B], Oij[3][3][ET_B * ET_B];
  float     ti[3][ET_B], tj[3][ET_B], tk[3][ET_B];
  float2    evs[3][ET_B];
  float2    dab[ET_B * ET_B];               // e_i + e_j + e_k - e_a - e_b, a in block 0, b in block 1
  long long cube0[3][6];                    // offset of slot s's local (0, 0, 0) in pass p's array
  int       slot_on[6];
  int       rbn[3];
};
constexpr int EW_SMEM = 2 * (int) sizeof(EwStage);

__device__ __forceinline__ void ew_bar_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void ew_bar_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Producer side: stage item `tile` of the triplet into S (128 threads, p = 0..127).
__device__ __forceinline__ void ew_stage(const TiledEnergyArgs& E, const float2* P12, const float2* P34,
                                         const float2* P56, int i, int j, int k, const ff& eijk, int tile, EwStage& S,
                                         int p, long long rel0) {
  constexpr int B = ET_B, B3 = B * B * B;
  const int       v = E.v, o = E.o;
  const long long v2 = (long long) v * v;
  const int3      tt     = E.tiles[tile];
  const int       rb0[3] = {tt.x * B, tt.y * B, tt.z * B};
  const int       rbn[3] = {min(B, v - rb0[0]), min(B, v - rb0[1]), min(B, v - rb0[2])};
  auto            b0     = [&](int u) { return u == 0 ? rb0[0] : u == 1 ? rb0[1] : rb0[2]; };
  auto            bn     = [&](int u) { return u == 0 ? rbn[0] : u == 1 ? rbn[1] : rbn[2]; };
  if(p < 3) S.rbn[p] = rbn[p];
  if(p >= 96 && p < 102) { // a slot counts once per distinct ordered block triple
    const int  t6 = p - 96;
    const int* P  = c_perm[t6];
    int        on = 1;
    for(int q = 0; q < t6; q++) {
      const int* Q = c_perm[q];
      if(b0(P[0]) == b0(Q[0]) && b0(P[1]) == b0(Q[1]) && b0(P[2]) == b0(Q[2])) on = 0;
    }
    S.slot_on[t6] = on;
  } else if(p >= 32 && p < 50) { // pass pp reads its array with (slowest, middle, fastest)
    const int  pp = (p - 32) / 6, sl = (p - 32) % 6; // = blocks (P0, P2, P1) / (P1, P0, P2) / (P2, P1, P0)
    const int* P  = c_perm[sl];
    const int  q0 = pp == 0 ? P[0] : pp == 1 ? P[1] : P[2], q1 = pp == 0 ? P[2] : pp == 1 ? P[0] : P[1],
               q2 = pp == 0 ? P[1] : pp == 1 ? P[2] : P[0];
    S.cube0[pp][sl] = ((long long) b0(q0) * v + b0(q1)) * v + b0(q2);
  }
  // singles data of the three blocks (the six ordered pairs of distinct blocks)
  const float *gOjk = E.oovv + ((long long) j * o + k) * v2, *gOik = E.oovv + ((long long) i * o + k) * v2,
              *gOij = E.oovv + ((long long) i * o + j) * v2;
  for(int e = p; e < 6 * B * B; e += EW_PROD) {
    const int pi = e / (B * B), u = pi >> 1, w = (pi & 1) ? (u == 2 ? 1 : 2) : (u == 0 ? 1 : 0);
    const int x = (e / B) % B, y = e % B;
    const bool      ok  = x < bn(u) && y < bn(w);
    const long long off = (long long) (b0(u) + x) * v + b0(w) + y;
    S.Ojk[u][w][x * B + y] = ok ? gOjk[off] : 0.f;
    S.Oik[u][w][x * B + y] = ok ? gOik[off] : 0.f;
    S.Oij[u][w][x * B + y] = ok ? gOij[off] : 0.f;
  }
  if(p < 3 * B) {
    const int  u = p / B, x = p % B;
    const bool ok = x < bn(u);
    const int  a  = b0(u) + x;
    S.ti[u][x] = ok ? E.t1[(long long) i * v + a] : 0.f;
    S.tj[u][x] = ok ? E.t1[(long long) j * v + a] : 0.f;
    S.tk[u][x] = ok ? E.t1[(long long) k * v + a] : 0.f;
    const ff e = ok ? ff_from_double(E.ev[a]) : ff{0.f, 0.f};
    S.evs[u][x] = make_float2(e.hi, e.lo);
  } else if(p >= 64) { // the orbit-wide part of D (the same float-float steps as the staged form)
    const int x = (p - 64) / B, y = (p - 64) % B;
    const ff  ea = x < bn(0) ? ff_from_double(E.ev[b0(0) + x]) : ff{0.f, 0.f};
    const ff  eb = y < bn(1) ? ff_from_double(E.ev[b0(1) + y]) : ff{0.f, 0.f};
    const ff  d  = ff_add(ff_add(eijk, ff{-ea.hi, -ea.lo}), ff{-eb.hi, -eb.lo});
    S.dab[p - 64] = make_float2(d.hi, d.lo);
  }
  ew_bar_sync(EW_BAR_PROD, EW_PROD); // cube0 visible to every producer
  // W of the six slots by orbit coordinates, three passes (one array each, read along its
  // contiguous index); a producer takes local positions r = p + 128 m (m = 0..3) of every slot:
  // (slowest, middle, fastest) local index (r / 64, r / 8 % 8, r % 8) = rel0 + 2 m v^2.
  const bool full = rbn[0] == B && rbn[1] == B && rbn[2] == B;
  float2*    Wf   = &S.W[0][0];
#pragma unroll
  for(int pass = 0; pass < 3; pass++) {
    if(pass > 0) ew_bar_sync(EW_BAR_PROD, EW_PROD);
    const float2* src = pass == 0 ? P12 : pass == 1 ? P34 : P56;
#pragma unroll
    for(int m = 0; m < 4; m++) { // position r = p + 128 m of the six slots: 6 loads in flight
      float2 x[6];
      int    widx[6];
#pragma unroll
      for(int it = 0; it < 6; it++) {
        const int s = it;
        const int P0 = kPerm(s, 0), P1 = kPerm(s, 1), P2 = kPerm(s, 2);
        const int f = p & 7, md = (p >> 3) & 7, sl = (p >> 6) + 2 * m;
        int       la, lb, lc; // slot-local (a', b', c'): a in block P0, b in P1, c in P2
        if(pass == 0) { // P12[a][c][b]: b fastest
          la = sl, lc = md, lb = f;
        } else if(pass == 1) { // P34[b][a][c]: c fastest
          lb = sl, la = md, lc = f;
        } else { // P56[c][b][a]: a fastest
          lc = sl, lb = md, la = f;
        }
        const long long off = S.cube0[pass][s] + rel0 + 2LL * m * v2;
        const bool      ok  = full || (la < rbn[P0] && lb < rbn[P1] && lc < rbn[P2]);
        x[it]               = ok ? src[off] : make_float2(0.f, 0.f);
        int loc[3]          = {0, 0, 0};
        loc[P0] = la, loc[P1] = lb, loc[P2] = lc;
        widx[it] = s * B3 + kSwz(loc[0], loc[1], loc[2]);
      }
#pragma unroll
      for(int it = 0; it < 6; it++) {
        if(pass == 0) Wf[widx[it]] = x[it];
        else if(pass == 1) { // two-sum of the high words, low words added; renormalised in pass 2
          const float2 q = Wf[widx[it]];
          const ff     h = ff_two_sum(q.x, x[it].x);
          Wf[widx[it]]   = make_float2(h.hi, h.lo + (q.y + x[it].y));
        } else {
          const float2 q = Wf[widx[it]];
          const ff     r = ff_add(ff{q.x, q.y}, ff{x[it].x, x[it].y});
          Wf[widx[it]]   = make_float2(r.hi, r.lo);
        }
      }
    }
  }
}

static __global__ void __launch_bounds__(EW_THREADS, 2) energy_ws_batch_kernel(const __grid_constant__ BatchEnergyArgs A) {
  constexpr int B = ET_B, B3 = B * B * B;
  extern __shared__ __align__(16) unsigned char ew_smem[];
  EwStage*               stage = reinterpret_cast<EwStage*>(ew_smem); // [2]
  const TiledEnergyArgs& E     = A.base_args;
  const int              slot = blockIdx.y, bb = A.base ? *A.base : 0;
  const int*             tp   = A.tri + 4 * (bb + slot);
  const int              i = tp[0], j = tp[1], k = tp[2];
  const long long        v3 = (long long) E.v * E.v * E.v;
  const float2*          F  = A.F + (long long) slot * 3 * v3;
  const int              gblock = blockIdx.x, gsize = gridDim.x;
  const int              nitems = gblock < E.ntiles ? (E.ntiles - gblock + gsize - 1) / gsize : 0;
  double*                part   = A.part + 6 * ((long long) slot * gridDim.x + blockIdx.x);
  __shared__ double      red[5][EW_CONS / 32];

  if(threadIdx.x < EW_PROD) {
    // ---------------------------------------------------------------- producers
    const int       p    = threadIdx.x;
    const ff        eijk = ff_add(ff_add(ff_from_double(E.eo[i]), ff_from_double(E.eo[j])), ff_from_double(E.eo[k]));
    const long long rel0 = ((long long) (p >> 6) * E.v + ((p >> 3) & 7)) * E.v + (p & 7);
    for(int n = 0; n < nitems; n++) {
      const int b = n & 1;
      if(n >= 2) ew_bar_sync(EW_BAR_FREE + b, EW_THREADS); // the consumers are done with item n - 2
      ew_stage(E, F, F + v3, F + 2 * v3, i, j, k, eijk, gblock + n * gsize, stage[b], p, rel0);
      ew_bar_arrive(EW_BAR_FULL + b, EW_THREADS);
    }
  } else {
    // ---------------------------------------------------------------- consumers
    const int c = threadIdx.x - EW_PROD;
    ff        s4{0.f, 0.f}, s5{0.f, 0.f};
    float     sens = 0.f;
    for(int n = 0; n < nitems; n++) {
      const int b = n & 1;
      ew_bar_sync(EW_BAR_FULL + b, EW_THREADS);
      const EwStage& S      = stage[b];
      const bool     all_on = S.slot_on[0] & S.slot_on[1] & S.slot_on[2] & S.slot_on[3] & S.slot_on[4] & S.slot_on[5];
      const int      n0 = S.rbn[0], n1 = S.rbn[1], n2 = S.rbn[2];
      for(int r = c; r < B3; r += EW_CONS) {
        const int la = r / (B * B), lb = (r / B) % B, lc = r % B;
        if(la >= n0 || lb >= n1 || lc >= n2) continue;
        et_orbit(S.W, S.Ojk, S.Oik, S.Oij, S.ti, S.tj, S.tk, S.evs, S.dab, all_on, S.slot_on, la, lb, lc, E.want_sens,
                 s4, s5, sens);
      }
      if(n + 2 < nitems) ew_bar_arrive(EW_BAR_FREE + b, EW_THREADS); // the producers refill it
    }
    // fixed-order reduction over the consumer warps: E[T] (s, c), E(T) (s, c), sensitivity
    CSum c4, c5;
    c4.add((double) s4.hi);
    c4.add((double) s4.lo);
    c5.add((double) s5.hi);
    c5.add((double) s5.lo);
    double sd = sens;
    const int lane = c & 31, w = c >> 5;
#pragma unroll
    for(int off = 16; off > 0; off >>= 1) {
      CSum oa, ob;
      oa.s = __shfl_down_sync(0xffffffffu, c4.s, off);
      oa.c = __shfl_down_sync(0xffffffffu, c4.c, off);
      ob.s = __shfl_down_sync(0xffffffffu, c5.s, off);
      ob.c = __shfl_down_sync(0xffffffffu, c5.c, off);
      c4.merge(oa);
      c5.merge(ob);
      sd += __shfl_down_sync(0xffffffffu, sd, off);
    }
    if(lane == 0) {
      red[0][w] = c4.s, red[1][w] = c4.c, red[2][w] = c5.s, red[3][w] = c5.c, red[4][w] = sd;
    }
    ew_bar_sync(EW_BAR_CONS, EW_CONS);
    if(c == 0) {
      CSum ta, tb;
      double ts = 0.0;
      for(int q = 0; q < EW_CONS / 32; q++) {
        ta.add(red[0][q]);
        ta.c += red[1][q];
        tb.add(red[2][q]);
        tb.c += red[3][q];
        ts += red[4][q];
      }
      part[0] = ta.s, part[1] = ta.c, part[2] = tb.s, part[3] = tb.c, part[4] = ts, part[5] = 0.0;
    }
  }
  __syncthreads();
}

} // namespace ccsdt
