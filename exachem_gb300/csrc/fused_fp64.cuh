// Plain FP64 path, fused: the triples block stays on chip and the energy follows the contractions
// in the same kernel.
//
// Work unit = (occupied triplet i < k, sorted triple X <= Y <= Z of 8-wide virtual blocks).  Its six
// ordered cubes (a in block P0, b in P1, c in P2 for the six permutations P of the positions) hold
// the connected triples W_abc of every ordering of the unit's index triples; they live in shared
// memory (6 x 512 doubles) and never go to HBM.  W is the sum of twelve contractions (the d2 family
// of the reference, ccsd_t_all_fused_cpu.hpp:330-428, over the virtual d; the d1 family, :172-270,
// over the occupied l), in the closed-shell spatial form:
//   d-sum  +t_ij^ad (kc|bd) +t_ik^ad (jb|cd) +t_ji^bd (kc|ad) +t_jk^bd (ia|cd) +t_ki^cd (jb|ad) +t_kj^cd (ia|bd)
//   l-sum  -t_il^ac (kl|jb) -t_kl^ca (il|jb) -t_il^ab (jl|kc) -t_jl^ba (il|kc) -t_jl^bc (kl|ia) -t_kl^cb (jl|ia)
// One warp owns one cube: for each term it runs the cube's 8 x 64 contraction on FP64 DMMA tiles
// (mma.sync.m16n8k4.f64; the pair index of the term - 64 rows - is M, the single index - 8 - is N),
// accumulates in registers and adds the tile into its cube.  After a CTA barrier the six warps
// evaluate the energy of every ordered (a, b, c) of the unit (cpu.hpp:597-619: E[T] += Z Y4 / D,
// E(T) += Z Y5 / D with Z = 4 W_abc + W_bca + W_cab, Y = 3 V_abc - V_acb - V_bac - V_cba) from the
// cubes in shared memory, in FP64 with compensated sums, and reduce per CTA with warp shuffles.
//
// Operands are read from L2 straight into the DMMA fragments (four consecutive kappa per row: one
// 32-byte sector per fragment row): GB300's FP64 pipe retires ~3.5 flop per clock per SM, so each
// SM needs only ~2 bytes per clock of operands and a staging copy through shared memory would buy
// nothing.  Every distinct cube costs 512 x (6 v + 6 o) multiply-adds; a unit with a repeated
// block (X = Y or Y = Z) has equal cubes, computed once and read through `canon`.
#pragma once

#include "energy_tiled.cuh"
#include "fp64_kernels.cuh"

namespace ccsdt {

constexpr int FX_WARPS = 6, FX_THREADS = 32 * FX_WARPS;

// the twelve terms: sum (d-sum, K = v) or not (l-sum, K = o); the role of the single index (0 = a,
// 1 = b, 2 = c) and of the pair's first and second index; the occupied positions (0 = i, 1 = j,
// 2 = k) of the single operand (s0, s1) and of the pair operand (pz).
//   d-sum: single t2[s0][s1][m][kappa], pair ovvv[pz][r1][r2][kappa]
//   l-sum: single ooovh[s0][s1][m][kappa] = (s0 kappa|s1 m), pair t2h[pz][r1][r2][kappa] = t_{pz kappa}^{r1 r2}
struct FxTerm {
  int dsum, rm, r1, r2, s0, s1, pz;
};
__device__ __constant__ FxTerm c_fx_terms[12] = {
  {1, 0, 2, 1, 0, 1, 2}, {1, 0, 1, 2, 0, 2, 1}, {1, 1, 2, 0, 1, 0, 2}, // t_ij^ad (kc|bd), t_ik^ad (jb|cd), t_ji^bd (kc|ad)
  {1, 1, 0, 2, 1, 2, 0}, {1, 2, 1, 0, 2, 0, 1}, {1, 2, 0, 1, 2, 1, 0}, // t_jk^bd (ia|cd), t_ki^cd (jb|ad), t_kj^cd (ia|bd)
  {0, 1, 0, 2, 2, 1, 0}, {0, 1, 2, 0, 0, 1, 2}, {0, 2, 0, 1, 1, 2, 0}, // t_il^ac (kl|jb), t_kl^ca (il|jb), t_il^ab (jl|kc)
  {0, 2, 1, 0, 0, 2, 1}, {0, 0, 1, 2, 2, 0, 1}, {0, 0, 2, 1, 1, 0, 2}, // t_jl^ba (il|kc), t_jl^bc (kl|ia), t_kl^cb (jl|ia)
};

struct FusedArgs {
  const double *t2, *t2h;
  const double *ov_i, *ov_j, *ov_k; // (ia|bc) slabs (v^3 each) of the triplet's occupied indices
  const double *ooovh, *oovv, *t1, *eo, *ev;
  const int3*   tiles; // sorted block triples
  int           ntiles;
  int           o, v, i, j, k;
  double*       part;  // 4 doubles per CTA: E[T] (s, c), E(T) (s, c)
};

static __global__ void __launch_bounds__(FX_THREADS, 3) t3_fused_fp64_kernel(const __grid_constant__ FusedArgs A) {
  constexpr int B = ET_B, B3 = B * B * B;
  __shared__ double W[6][B3];  // cube q: [a'][b'][c'] local to its blocks (blk(P0), blk(P1), blk(P2))
  __shared__ int    canon[6]; // first cube with the same ordered block triple (itself if distinct)
  __shared__ double red[4][FX_WARPS];
  const int        v = A.v, o = A.o, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int        g = lane >> 2, tq = lane & 3;
  const long long  v2 = (long long) v * v;
  const double     eijk = A.eo[A.i] + A.eo[A.j] + A.eo[A.k];
  CSum             s4, s5;

  for(int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    const int3 tt  = A.tiles[tile];
    auto       blk = [&](int p) { return p == 0 ? tt.x : p == 1 ? tt.y : tt.z; }; // block at position p
    if(tid < 6) { // a unit with a repeated block has equal cubes: each is computed and counted once
      const int* P = c_perm[tid];
      int        c = tid;
      for(int p = tid - 1; p >= 0; p--) {
        const int* Q = c_perm[p];
        if(blk(P[0]) == blk(Q[0]) && blk(P[1]) == blk(Q[1]) && blk(P[2]) == blk(Q[2])) c = p;
      }
      canon[tid] = c;
    }
    __syncthreads();
    // ---------------------------------------------------------------- contractions: warp = cube q
    if(canon[warp] == warp) {
      const int q = warp, P0 = c_perm[q][0], P1 = c_perm[q][1], P2 = c_perm[q][2];
      // first global index of role r (0 = a, 1 = b, 2 = c) and occupied index at position p, by
      // selects (a runtime index into a local array would live in local memory)
      const int rba = blk(P0) * B, rbb = blk(P1) * B, rbc = blk(P2) * B;
      auto      rb  = [&](int r) { return r == 0 ? rba : r == 1 ? rbb : rbc; };
      auto      oc  = [&](int p) { return p == 0 ? A.i : p == 1 ? A.j : A.k; };
      double*   Wq    = W[q];
      for(int e = lane; e < B3; e += 32) Wq[e] = 0.0;
      __syncwarp();
#pragma unroll 1
      for(int term = 0; term < 12; term++) {
        const FxTerm T = c_fx_terms[term];
        const int    K = T.dsum ? v : o;
        // single operand row (N index = the single role, local g)
        const int     gs = rb(T.rm) + g;
        const double* sp = T.dsum ? A.t2 + ((long long) oc(T.s0) * o + oc(T.s1)) * v2 + (long long) gs * v
                                  : A.ooovh + ((long long) oc(T.s0) * o + oc(T.s1)) * v * o + (long long) gs * o;
        const bool    sv = gs < v;
        // pair operand rows (M index = (r1, r2), 16 rows per tile t: r1 local 2 t + h, r2 local g)
        const double* pbase = T.dsum ? (T.pz == 0 ? A.ov_i : T.pz == 1 ? A.ov_j : A.ov_k)
                                     : A.t2h + (long long) oc(T.pz) * v2 * o;
        // row (r1 local n1, r2 local g) at p0 + n1 v K; rows with a global index >= v read as zero
        const int       g2   = rb(T.r2) + g;
        const int       nlim = g2 < v ? v - rb(T.r1) : 0; // local r1 rows < nlim exist
        const long long vK   = (long long) v * K;
        const double*   p0   = pbase + ((long long) rb(T.r1) * v + (g2 < v ? g2 : 0)) * K;
        double acc[4][4];
#pragma unroll
        for(int t = 0; t < 4; t++)
#pragma unroll
          for(int z = 0; z < 4; z++) acc[t][z] = 0.0;
        for(int k0 = 0; k0 < K; k0 += 4) {
          const int  kk = k0 + tq;
          const bool kin = kk < K;
          const double b = (sv && kin) ? sp[kk] : 0.0;
#pragma unroll
          for(int t = 0; t < 4; t++) {
            const double a0 = (2 * t < nlim && kin) ? p0[(2 * t) * vK + kk] : 0.0;
            const double a1 = (2 * t + 1 < nlim && kin) ? p0[(2 * t + 1) * vK + kk] : 0.0;
            dmma_m16n8k4(acc[t], a0, a1, b);
          }
        }
        // tile element (row g + 8 h, column 2 tq + e) of tile t: r1 local 2 t + h, r2 local g, single 2 tq + e
        // cube element [a'][b'][c'] at a' 64 + b' 8 + c': role r has stride 64 >> 3 r
        const double sgn = T.dsum ? 1.0 : -1.0;
        const int    st1 = 64 >> (3 * T.r1), st2 = 64 >> (3 * T.r2), stm = 64 >> (3 * T.rm);
#pragma unroll
        for(int t = 0; t < 4; t++)
#pragma unroll
          for(int h = 0; h < 2; h++)
#pragma unroll
            for(int e = 0; e < 2; e++) Wq[(2 * t + h) * st1 + g * st2 + (2 * tq + e) * stm] += sgn * acc[t][h * 2 + e];
        __syncwarp(); // the next term maps the cube's elements to other lanes
      }
    }
    __syncthreads(); // all distinct cubes are complete
    // ---------------------------------------------------------------- energy of the unit
    for(int e = tid; e < 6 * B3; e += FX_THREADS) {
      const int q = e / B3, r = e % B3;
      if(canon[q] != q) continue;
      const int* P  = c_perm[q];
      const int  la = r / (B * B), lb = (r / B) % B, lc = r % B;
      const int  a = blk(P[0]) * B + la, b = blk(P[1]) * B + lb, c = blk(P[2]) * B + lc;
      if(a >= v || b >= v || c >= v) continue;
      // W at the orderings of (a, b, c): the cube of the permuted positions, at the permuted local
      auto w_at = [&](int p0, int p1, int p2, int x, int y, int z) {
        return W[canon[kSlot(p0, p1, p2)]][(x * B + y) * B + z];
      };
      const double wabc = W[q][r];
      const double wbca = w_at(P[1], P[2], P[0], lb, lc, la), wcab = w_at(P[2], P[0], P[1], lc, la, lb);
      const double wacb = w_at(P[0], P[2], P[1], la, lc, lb), wbac = w_at(P[1], P[0], P[2], lb, la, lc);
      const double wcba = w_at(P[2], P[1], P[0], lc, lb, la);
      const double z  = 4.0 * wabc + wbca + wcab;
      const double y4 = 3.0 * wabc - wacb - wbac - wcba;
      // singles part of V_xyz: (jy|kz) t_i^x + (ix|kz) t_j^y + (ix|jy) t_k^z
      auto sg = [&](int x, int y, int zz) {
        return A.oovv[((long long) A.j * o + A.k) * v2 + (long long) y * v + zz] * A.t1[(long long) A.i * v + x] +
               A.oovv[((long long) A.i * o + A.k) * v2 + (long long) x * v + zz] * A.t1[(long long) A.j * v + y] +
               A.oovv[((long long) A.i * o + A.j) * v2 + (long long) x * v + y] * A.t1[(long long) A.k * v + zz];
      };
      const double y5 = y4 + 3.0 * sg(a, b, c) - sg(a, c, b) - sg(b, a, c) - sg(c, b, a);
      const double d  = eijk - A.ev[a] - A.ev[b] - A.ev[c];
      s4.add(z * y4 / d);
      s5.add(z * y5 / d);
    }
    __syncthreads(); // the cubes and canon are free for the next unit
  }
  // ---------------------------------------------------------------- fixed-order CTA reduction
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) {
    CSum o4, o5;
    o4.s = __shfl_down_sync(0xffffffffu, s4.s, off);
    o4.c = __shfl_down_sync(0xffffffffu, s4.c, off);
    o5.s = __shfl_down_sync(0xffffffffu, s5.s, off);
    o5.c = __shfl_down_sync(0xffffffffu, s5.c, off);
    s4.merge(o4);
    s5.merge(o5);
  }
  if(lane == 0) red[0][warp] = s4.s, red[1][warp] = s4.c, red[2][warp] = s5.s, red[3][warp] = s5.c;
  __syncthreads();
  if(tid == 0) {
    CSum a4, a5;
    for(int w = 0; w < FX_WARPS; w++) {
      a4.add(red[0][w]);
      a4.c += red[1][w];
      a5.add(red[2][w]);
      a5.c += red[3][w];
    }
    double* out = A.part + 4 * (long long) blockIdx.x;
    out[0] = a4.s, out[1] = a4.c, out[2] = a5.s, out[3] = a5.c;
  }
}

} // namespace ccsdt
