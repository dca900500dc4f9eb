// Plain FP64 path: DMMA (mma.sync.m16n8k4.f64) contractions and the fused energy.
//
// Per occupied triplet (i <= j <= k) the connected triples W_abc is kept as three
// partial arrays, one per row index of the contractions:
//   P12[a][c][b]  terms whose amplitude carries a (d-sum) / whose pair is (a,c) (l-sum)
//   P34[b][a][c]  ... b / (b,a)
//   P56[c][b][a]  ... c / (c,b)
// so W_abc = P12[a][c][b] + P34[b][a][c] + P56[c][b][a].  Each array is written by
// exactly one GEMM per contraction family: the l-sum (the reference's d1 family,
// ccsd_t_all_fused_cpu.hpp:172-270) initialises it, the d-sum (d2 family,
// cpu.hpp:330-428) accumulates on top.
#pragma once

#include "common.cuh"

namespace ccsdt {

// One GEMM term: sum_kappa A(m, kappa) * B(n, kappa), kappa contiguous in memory.
struct GemmTerm {
  const double* A;
  RowMap        ma;
  const double* B;
  RowMap        mb;
  int           K;
  double        alpha;
};

// C[M x N] (row-major, ldc = N) = beta * C + sum over terms.  Up to 2 terms.
struct GemmJob {
  GemmTerm  t[2];
  int       nterms;
  double*   C;
  long long M, N;
  double    beta;
};

struct GemmBatch {
  GemmJob job[3];
};

constexpr int D_BM = 64, D_BN = 64, D_BK = 16, D_THREADS = 128;

__device__ __forceinline__ void dmma_m16n8k4(double (&c)[4], double a0, double a1, double b0) {
  asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
               "{%0,%1,%2,%3};\n"
               : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
               : "d"(a0), "d"(a1), "d"(b0));
}

// Grid: x = linear tile id (M-major over ceil(N/64) column tiles), z = job.  Block: 128 threads = 4 warps (2 x 2), each
// warp owns a 32 x 32 sub-tile = 2 (m16) x 4 (n8) DMMA tiles.
static __global__ void __launch_bounds__(D_THREADS) dmma_gemm_kernel(const __grid_constant__ GemmBatch batch) {
  const GemmJob&   J       = batch.job[blockIdx.z];
  const long long tiles_n = (J.N + D_BN - 1) / D_BN;
  const long long m0 = (long long) (blockIdx.x / tiles_n) * D_BM, n0 = (long long) (blockIdx.x % tiles_n) * D_BN;
  if(m0 >= J.M || n0 >= J.N) return;

  __shared__ double As[D_BK][D_BM + 2];
  __shared__ double Bs[D_BK][D_BN + 2];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, tq = lane & 3;

  double acc[2][4][4];
#pragma unroll
  for(int x = 0; x < 2; x++)
#pragma unroll
    for(int y = 0; y < 4; y++)
#pragma unroll
      for(int z = 0; z < 4; z++) acc[x][y][z] = 0.0;

  // loader mapping: thread -> (row = tid / 2, 8 consecutive kappa)
  const int lr = tid >> 1, lk = (tid & 1) * 8;

  for(int term = 0; term < J.nterms; term++) {
    const GemmTerm& T  = J.t[term];
    const long long ma = m0 + lr, nb = n0 + lr;
    const bool      va = ma < J.M, vb = nb < J.N;
    const double*   pa = va ? T.A + row_addr(T.ma, ma) : nullptr;
    const double*   pb = vb ? T.B + row_addr(T.mb, nb) : nullptr;
    const double    al = T.alpha;
    for(int k0 = 0; k0 < T.K; k0 += D_BK) {
      __syncthreads();
#pragma unroll
      for(int u = 0; u < 8; u++) {
        const int kk = k0 + lk + u;
        As[lk + u][lr] = (va && kk < T.K) ? al * pa[kk] : 0.0;
        Bs[lk + u][lr] = (vb && kk < T.K) ? pb[kk] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for(int ks = 0; ks < D_BK; ks += 4) {
        double a[2][2], b[4];
#pragma unroll
        for(int x = 0; x < 2; x++) {
          a[x][0] = As[ks + tq][wm + x * 16 + g];
          a[x][1] = As[ks + tq][wm + x * 16 + g + 8];
        }
#pragma unroll
        for(int y = 0; y < 4; y++) b[y] = Bs[ks + tq][wn + y * 8 + g];
#pragma unroll
        for(int x = 0; x < 2; x++)
#pragma unroll
          for(int y = 0; y < 4; y++) dmma_m16n8k4(acc[x][y], a[x][0], a[x][1], b[y]);
      }
    }
  }

  // epilogue: C = beta * C + acc
#pragma unroll
  for(int x = 0; x < 2; x++)
#pragma unroll
    for(int y = 0; y < 4; y++)
#pragma unroll
      for(int h = 0; h < 2; h++) {
        const long long m = m0 + wm + x * 16 + g + h * 8;
        if(m >= J.M) continue;
#pragma unroll
        for(int e = 0; e < 2; e++) {
          const long long n = n0 + wn + y * 8 + tq * 2 + e;
          if(n >= J.N) continue;
          double* cp = J.C + m * J.N + n;
          double  v  = acc[x][y][h * 2 + e];
          *cp        = (J.beta != 0.0) ? J.beta * *cp + v : v;
        }
      }
}

// ---------------------------------------------------------------------------------------
// Energy of one triplet from its partial arrays (restates ccsd_t_all_fused_cpu.hpp:597-619
// in the closed-shell form):
//   W_xyz = P12[x][z][y] + P34[y][x][z] + P56[z][y][x]
//   Z     = 4 W_abc + W_bca + W_cab
//   Y4    = 3 W_abc - W_acb - W_bac - W_cba,   Y5 = Y4 + (same combination of singles)
//   singles_xyz = (jy|kz) t_i^x + (ix|kz) t_j^y + (ix|jy) t_k^z
//   e4 += Z Y4 / D,  e5 += Z Y5 / D,  D = e_i + e_j + e_k - e_a - e_b - e_c
// Per-block compensated partials go to part[blockIdx.x] (4 doubles: s4, c4, s5, c5).
struct EnergyArgs {
  const double *P12, *P34, *P56;
  const double *oovv, *t1, *eo, *ev;
  int           o, v, i, j, k;
  double*       part;
};

constexpr int E_THREADS = 256;

__device__ inline void block_reduce_csum(CSum& a, CSum& b, double* out) {
  __shared__ double sh[4][E_THREADS / 32];
  const int         lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // fixed-shape tree: deterministic
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) {
    CSum oa, ob;
    oa.s = __shfl_down_sync(0xffffffffu, a.s, off);
    oa.c = __shfl_down_sync(0xffffffffu, a.c, off);
    ob.s = __shfl_down_sync(0xffffffffu, b.s, off);
    ob.c = __shfl_down_sync(0xffffffffu, b.c, off);
    a.merge(oa);
    b.merge(ob);
  }
  if(lane == 0) {
    sh[0][w] = a.s;
    sh[1][w] = a.c;
    sh[2][w] = b.s;
    sh[3][w] = b.c;
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    CSum ta, tb;
    for(int q = 0; q < E_THREADS / 32; q++) {
      ta.add(sh[0][q]);
      ta.c += sh[1][q];
      tb.add(sh[2][q]);
      tb.c += sh[3][q];
    }
    out[0] = ta.s;
    out[1] = ta.c;
    out[2] = tb.s;
    out[3] = tb.c;
  }
}

static __global__ void __launch_bounds__(E_THREADS) energy_fp64_kernel(const __grid_constant__ EnergyArgs A) {
  const int       v = A.v, o = A.o;
  const long long v2 = (long long) v * v, n = v2 * v;
  const int       i = A.i, j = A.j, k = A.k;
  const double    eijk = A.eo[i] + A.eo[j] + A.eo[k];
  const double *  Ojk = A.oovv + ((long long) j * o + k) * v2, *Oik = A.oovv + ((long long) i * o + k) * v2,
               *Oij = A.oovv + ((long long) i * o + j) * v2;
  const double *ti = A.t1 + (long long) i * v, *tj = A.t1 + (long long) j * v, *tk = A.t1 + (long long) k * v;
  CSum s4, s5;
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n;
      e += (long long) gridDim.x * blockDim.x) {
    const int a = (int) (e / v2), b = (int) ((e / v) % v), c = (int) (e % v);
#define WP(x, y, z) (A.P12[((long long) (x) * v + (z)) * v + (y)] + A.P34[((long long) (y) * v + (x)) * v + (z)] + \
                     A.P56[((long long) (z) * v + (y)) * v + (x)])
#define SG(x, y, z) (Ojk[(long long) (y) * v + (z)] * ti[x] + Oik[(long long) (x) * v + (z)] * tj[y] + \
                     Oij[(long long) (x) * v + (y)] * tk[z])
    const double wabc = WP(a, b, c), wbca = WP(b, c, a), wcab = WP(c, a, b);
    const double wacb = WP(a, c, b), wbac = WP(b, a, c), wcba = WP(c, b, a);
    const double z  = 4.0 * wabc + wbca + wcab;
    const double y4 = 3.0 * wabc - wacb - wbac - wcba;
    const double y5 = y4 + 3.0 * SG(a, b, c) - SG(a, c, b) - SG(b, a, c) - SG(c, b, a);
#undef WP
#undef SG
    const double d = eijk - A.ev[a] - A.ev[b] - A.ev[c];
    s4.add(z * y4 / d);
    s5.add(z * y5 / d);
  }
  block_reduce_csum(s4, s5, A.part + 4 * (long long) blockIdx.x);
}

// Sums nparts block partials for one triplet and scales by m/9: E_THREADS threads each take a
// contiguous run of partials, then the fixed-shape block tree (deterministic for a given nparts).
// Launch with one block of E_THREADS threads.
static __global__ void __launch_bounds__(E_THREADS) reduce_parts_kernel(const double* part, int nparts, double scale,
                                                                      double* out) {
  CSum a, b;
  const int per = (nparts + E_THREADS - 1) / E_THREADS;
  const int q0 = threadIdx.x * per, q1 = min(nparts, q0 + per);
  for(int q = q0; q < q1; q++) {
    a.add(part[4 * q + 0]);
    a.c += part[4 * q + 1];
    b.add(part[4 * q + 2]);
    b.c += part[4 * q + 3];
  }
  __shared__ double tmp[4];
  block_reduce_csum(a, b, tmp);
  __syncthreads();
  if(threadIdx.x == 0) {
    out[0] = scale * (tmp[0] + tmp[1]);
    out[1] = scale * (tmp[2] + tmp[3]);
  }
}

// x -> float-float (hi = x rounded to FP32, lo = the remainder rounded), element by element.
static __global__ void to_ff_kernel(const double* x, float2* y, long long n) {
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long) gridDim.x * blockDim.x) {
    const float hi = (float) x[e];
    y[e]           = make_float2(hi, (float) (x[e] - (double) hi));
  }
}

static __global__ void to_f32_kernel(const double* x, float* y, long long n) {
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long) gridDim.x * blockDim.x)
    y[e] = (float) x[e];
}

// Compensated fixed-order sum of per-triplet energies e[2 n] -> out[2].
static __global__ void reduce_triplets_kernel(const double* e, long long n, double* out) {
  if(threadIdx.x != 0 || blockIdx.x != 0) return;
  CSum a, b;
  for(long long q = 0; q < n; q++) {
    a.add(e[2 * q]);
    b.add(e[2 * q + 1]);
  }
  out[0] = a.value();
  out[1] = b.value();
}

// dst[x][p][l] = src[x][l][p] for p < P (P = v*v or o*v): the kappa-contiguous copies the
// l-sum contractions read (t2 -> t2h[x][(a,b)][l], ooov -> ooovh[y][(z,c)][l]).
static __global__ void transpose_mid_kernel(const double* src, double* dst, int X, int L, long long P) {
  const long long total = (long long) X * L * P;
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < total;
      e += (long long) gridDim.x * blockDim.x) {
    const long long x = e / (L * P), r = e % (L * P), l = r / P, p = r % P;
    dst[(x * P + p) * L + l] = src[e];
  }
}

static __global__ void nonfinite_count_kernel(const double* p, long long n, unsigned long long* cnt) {
  unsigned long long local = 0;
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < n;
      e += (long long) gridDim.x * blockDim.x)
    local += !isfinite(p[e]);
  if(local) atomicAdd(cnt, local);
}

} // namespace ccsdt
