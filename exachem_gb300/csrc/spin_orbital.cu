// Open-shell (UHF) (T) over spin orbitals, FP64 DMMA contractions over the spin-allowed blocks.
//
// The quantity ExaChem's fused driver sums with is_restricted = false
// (exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:383-392 spin filter and factor; the 27 contraction
// families of ccsd_t_all_fused_cpu.hpp:172-577 and its energy loop :597-619):
//
//   X_ijk(a; bc) = - sum_e t2(a,e,j,k) <ie||bc> - sum_m t2(b,c,i,m) <jk||ma>
//   W_ijk^abc    = P(i/jk) P(a/bc) X,   V_ijk^abc = P(i/jk) P(a/bc) t1(a,i) <jk||bc>
//   E[T] = sum_{i<j<k} sum_{a<b<c} W W / D,   E(T) = sum (W + V) W / D
//
// with P(p/qr) f(pqr) = f(pqr) - f(qpr) - f(rqp).  Spin orbitals follow ExaChem's MO order
// (occupied alpha | beta, virtual alpha | beta), so for i < j < k the spins are sorted, and the
// only virtual triples a < b < c with W != 0 carry the same spin pattern.  For a triplet and
// each of the three permutations p of (i, j, k) the energy reads X_p at (a; b c), (b; a c) and
// (c; b a): three spin blocks X_p[x][y z] with fixed spins of x, y and z.  Each block is one
// two-term GEMM whose contraction ranges the spins fix as well:
//   d-term: e runs over the one spin with {s_x, s_e} = {s_j, s_k}; zero unless also
//           {s_i, s_e} = {s_y, s_z}
//   s-term: m runs over the one spin with {s_y, s_z} = {s_i, s_m}; zero unless also
//           {s_j, s_k} = {s_m, s_x}
// Blocks with equal (p, s_x, s_y, s_z) are computed once (aaa: one block per permutation).
// Against dense spin-orbital GEMMs this is about five times less work, and no element of a
// spin-forbidden block of the inputs is read.  The plan of a triplet (so_plan) is host logic,
// exposed for tests as ccsdt_debug_spin_orbital_plan.
//
// GEMM operands need the contraction index contiguous; three one-time permuted copies give that:
//   tt[j][k][a][e] = t2(a,e,j,k),  vv[i][b][c][e] = <ie||bc>,  uu[j][k][a][m] = <jk||ma>
// while t2(b,c,i,m) is m-contiguous already.  Triplets rotate over a few streams, each with its
// own block slots and energy accumulators, so small blocks of neighbouring triplets overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"
#include "fp64_kernels.cuh"
#include "ozaki.cuh"

using namespace ccsdt;

namespace {

constexpr int kSoStreams = 4;   // triplets in flight
constexpr int kSoGrid    = 304; // energy kernel blocks (2 per SM)
constexpr int kSoThreads = 256;

// dst (row-major over n1 x n2 x n3 inner dims) = src at sum_d idx_d * s_d
__global__ void __launch_bounds__(256) permute4_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                                       long long n1, long long n2, long long n3, long long total,
                                                       long long s0, long long s1, long long s2, long long s3) {
  for(long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x; e < total;
      e += (long long) gridDim.x * blockDim.x) {
    long long r = e;
    const long long d3 = r % n3;
    r /= n3;
    const long long d2 = r % n2;
    r /= n2;
    const long long d1 = r % n1, d0 = r / n1;
    dst[e] = src[d0 * s0 + d1 * s1 + d2 * s2 + d3 * s3];
  }
}

// One spin block X[x - x0][(y - y0) nz + (z - z0)], FP64 (X) or float-float (Xf, the split path);
// both null: the block is zero.
struct SoBlock {
  const double* X;
  int           x0, y0, z0, ny, nz;
  const float2* Xf;
};

struct SoEnergyArgs {
  SoBlock       blk[3][3]; // [permutation ijk, jik, kji][position (a; b c), (b; a c), (c; b a)]
  const double *eps_o, *eps_v, *t1, *v2ijab;
  int           O, V, oa, va;
  int           i, j, k;
  int           a0, na, b0, nb, c0, nc;
  int           lt_ab, lt_bc; // a < b (b < c) required: same spin
  double*       part;         // [gridDim.x][4] compensated accumulators, kept across triplets
};

struct SoSpins {
  int oa, va, O, V;
  int occ(int p) const { return p >= oa; }
  int vlo(int s) const { return s ? va : 0; }
  int vn(int s) const { return s ? V - va : va; }
};

// multiset {p, q} == {r, s} over spins 0 / 1 (the sum fixes the multiset)
__host__ __device__ inline bool same_pair(int p, int q, int r, int s) { return p + q == r + s; }

__device__ __forceinline__ double so_x(const SoBlock& b, int x, int y, int z) {
  const long long e = ((long long) (x - b.x0) * b.ny + (y - b.y0)) * b.nz + (z - b.z0);
  if(b.Xf) {
    const float2 f = b.Xf[e];
    return (double) f.x + (double) f.y;
  }
  return b.X ? b.X[e] : 0.0;
}

// Energy of one triplet: W and V at every a < b < c of the triplet's spin pattern, restating
// ccsd_t_all_fused_cpu.hpp:597-619 (e4 += W W / D, e5 += (W + V) W / D) over spin orbitals.
// The singles term V reads t1(x, i') and <j'k'||yz> only where their spins allow a nonzero.
__global__ void __launch_bounds__(kSoThreads) so_energy_kernel(const __grid_constant__ SoEnergyArgs A) {
  const int    perm[3][3] = {{A.i, A.j, A.k}, {A.j, A.i, A.k}, {A.k, A.j, A.i}};
  const double eo         = A.eps_o[A.i] + A.eps_o[A.j] + A.eps_o[A.k];
  CSum         e4, e5;
  const long long total = (long long) A.na * A.nb * A.nc;
  for(long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x; t < total;
      t += (long long) gridDim.x * blockDim.x) {
    const int       c = A.c0 + (int) (t % A.nc);
    const long long r = t / A.nc;
    const int       b = A.b0 + (int) (r % A.nb), a = A.a0 + (int) (r / A.nb);
    if((A.lt_ab && a >= b) || (A.lt_bc && b >= c)) continue;
    double w = 0.0, vt = 0.0;
#pragma unroll
    for(int p = 0; p < 3; p++) {
      const double x = so_x(A.blk[p][0], a, b, c) - so_x(A.blk[p][1], b, a, c) - so_x(A.blk[p][2], c, b, a);
      w += p ? -x : x;
    }
    const int xyz[3][3] = {{a, b, c}, {b, a, c}, {c, b, a}};
#pragma unroll
    for(int p = 0; p < 3; p++) {
      const int ip = perm[p][0], jp = perm[p][1], kp = perm[p][2];
      const int si = ip >= A.oa, sjk = (jp >= A.oa) + (kp >= A.oa);
#pragma unroll
      for(int q = 0; q < 3; q++) {
        const int x = xyz[q][0], y = xyz[q][1], z = xyz[q][2];
        if((x >= A.va) != si || (y >= A.va) + (z >= A.va) != sjk) continue;
        const double g = A.t1[(long long) x * A.O + ip] * A.v2ijab[(((long long) jp * A.O + kp) * A.V + y) * A.V + z];
        vt += ((p == 0) == (q == 0)) ? g : -g;
      }
    }
    const double d  = eo - A.eps_v[a] - A.eps_v[b] - A.eps_v[c];
    const double wd = w / d;
    e4.add(w * wd);
    e5.add((w + vt) * wd);
  }
  // block reduction of the compensated pairs, merged into this block's accumulator
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) {
    CSum o4, o5;
    o4.s = __shfl_down_sync(0xffffffffu, e4.s, off);
    o4.c = __shfl_down_sync(0xffffffffu, e4.c, off);
    o5.s = __shfl_down_sync(0xffffffffu, e5.s, off);
    o5.c = __shfl_down_sync(0xffffffffu, e5.c, off);
    e4.merge(o4);
    e5.merge(o5);
  }
  __shared__ double red[kSoThreads / 32][4];
  const int         lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(lane == 0) {
    red[warp][0] = e4.s;
    red[warp][1] = e4.c;
    red[warp][2] = e5.s;
    red[warp][3] = e5.c;
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    double* acc = A.part + 4 * blockIdx.x;
    CSum    s4, s5;
    s4.s = acc[0];
    s4.c = acc[1];
    s5.s = acc[2];
    s5.c = acc[3];
    for(int w = 0; w < kSoThreads / 32; w++) {
      CSum o4, o5;
      o4.s = red[w][0];
      o4.c = red[w][1];
      o5.s = red[w][2];
      o5.c = red[w][3];
      s4.merge(o4);
      s5.merge(o5);
    }
    acc[0] = s4.s;
    acc[1] = s4.c;
    acc[2] = s5.s;
    acc[3] = s5.c;
  }
}

} // namespace

namespace {

// The contraction blocks of one triplet, as offsets into the operand arrays (host logic only).
// Block b is X[x - x0][(y - y0) nz + (z - z0)] over nx x (ny nz) elements:
//   d-term  - sum_e tt[d_a + x' V + e'] vv[d_b + y' V^2 + z' V + e']          e' < d_k
//   s-term  - sum_m uu[s_a + x' O + m'] t2[s_b + y' V O^2 + z' O^2 + m']       m' < s_k
// with x', y', z' the indices within the block.  of[p][q] = the block the energy reads for
// permutation p (ijk, jik, kji) at position q ((a; b c), (b; a c), (c; b a)), -1 where it is zero.
struct SoPlanBlock {
  int       x0, y0, z0, nx, ny, nz;
  int       has_d, has_s, d_k, s_k;
  long long d_a, d_b, s_a, s_b;
};
struct SoPlan {
  int         nblk;
  SoPlanBlock blk[9];
  int         of[3][3];
};

SoPlan so_plan(const SoSpins& S, int i, int j, int k) {
  const long long O = S.O, V = S.V;
  const int       perm[3][3] = {{i, j, k}, {j, i, k}, {k, j, i}};
  const int       si = S.occ(i), sj = S.occ(j), sk = S.occ(k);
  // spins of (x, y, z) at the three positions; the virtual triple carries the pattern (s_i, s_j, s_k)
  const int pos[3][3] = {{si, sj, sk}, {sj, si, sk}, {sk, sj, si}};
  SoPlan    P{};
  for(int p = 0; p < 3; p++) {
    const int ip = perm[p][0], jp = perm[p][1], kp = perm[p][2];
    const int s_i = S.occ(ip), s_j = S.occ(jp), s_k = S.occ(kp);
    for(int q = 0; q < 3; q++) {
      const int sx = pos[q][0], sy = pos[q][1], sz = pos[q][2];
      int       same = -1; // an earlier position of this permutation with the same spins
      for(int r = 0; r < q; r++)
        if(pos[r][0] == sx && pos[r][1] == sy && pos[r][2] == sz) same = r;
      if(same >= 0) {
        P.of[p][q] = P.of[p][same];
        continue;
      }
      SoPlanBlock B{S.vlo(sx), S.vlo(sy), S.vlo(sz), S.vn(sx), S.vn(sy), S.vn(sz), 0, 0, 0, 0, 0, 0, 0, 0};
      if(sx == s_j || sx == s_k) { // d-term: - sum_e tt[j'][k'][x][e] vv[i'][y][z][e]
        const int se = s_j + s_k - sx;
        if(same_pair(s_i, se, sy, sz)) {
          B.has_d = 1;
          B.d_k   = S.vn(se);
          B.d_a   = (((long long) jp * O + kp) * V + S.vlo(sx)) * V + S.vlo(se);
          B.d_b   = (((long long) ip * V + S.vlo(sy)) * V + S.vlo(sz)) * V + S.vlo(se);
        }
      }
      if(s_i == sy || s_i == sz) { // s-term: - sum_m uu[j'][k'][x][m] t2[y][z][i'][m]
        const int sm = sy + sz - s_i, m0 = sm ? S.oa : 0;
        if(same_pair(s_j, s_k, sm, sx)) {
          B.has_s = 1;
          B.s_k   = sm ? S.O - S.oa : S.oa;
          B.s_a   = (((long long) jp * O + kp) * V + S.vlo(sx)) * O + m0;
          B.s_b   = ((long long) S.vlo(sy) * V + S.vlo(sz)) * O * O + (long long) ip * O + m0;
        }
      }
      if(!(B.has_d || B.has_s) || B.nx == 0 || B.ny == 0 || B.nz == 0) { // zero, or no point reads it
        P.of[p][q] = -1;
        continue;
      }
      P.of[p][q]      = P.nblk;
      P.blk[P.nblk++] = B;
    }
  }
  return P;
}

// Digit planes (BF16, S planes) of the four contraction operands for the split path, one set per
// spin of the contraction index: tt / vv over e of spin s (columns [vlo(s), vlo(s) + vn(s)) of
// their rows), uu / t2 over m of spin s.  Row r of set (X, s) at X[s] + r Kp, plane stride R Kp.
struct SoPlanes {
  int                   S = 0;
  const __nv_bfloat16 * tt[2] = {}, *vv[2] = {}, *uu[2] = {}, *t2[2] = {};
  long long             Kv[2] = {}, Ko[2] = {};               // padded contraction lengths
  long long             R_tt = 0, R_vv = 0, R_uu = 0, R_t2 = 0; // rows
};

// Launches a triplet's plan on `st` (block b into slots[b], up to three GEMM jobs per launch) and
// fills the energy kernel's block table.  With planes (pl.S > 0): BF16-digit Ozaki GEMMs with
// float-float blocks, from the spin's digit planes.
cudaError_t so_contract(const SoSpins& S, const SoPlan& P, const double* tt, const double* vv, const double* uu,
                        const double* t2, double* const* slots, SoBlock (&blk)[3][3], cudaStream_t st,
                        const SoPlanes& pl) {
  const long long O = S.O, V = S.V;
  if(pl.S > 0) {
    OzBatch   batch{};
    int       nj = 0;
    long long max_tiles = 0;
    batch.S = pl.S;
    for(int b = 0; b < P.nblk; b++) {
      const SoPlanBlock& B = P.blk[b];
      OzJob              J{};
      int                nt = 0;
      if(B.has_d) { // rows of tt (j, k, a) and vv (i, b, c); e of the spin the block's offset starts at
        const long long e0 = B.d_a % V;
        const int       se = (e0 == S.va && B.d_k == S.V - S.va) ? 1 : 0;
        const long long Kp = pl.Kv[se];
        J.t[nt++] = OzTerm{pl.tt[se] + (B.d_a / V) * Kp, nullptr, oz_plain(), pl.R_tt * Kp,
                           pl.vv[se] + (B.d_b / V) * Kp, nullptr, OzRows{V, 1, B.nz}, pl.R_vv * Kp, (int) Kp, -1.f};
      }
      if(B.has_s) { // rows of uu (j, k, a) and t2 (b, c, i); m of the block's spin
        const long long m0 = B.s_a % O;
        const int       sm = (m0 == S.oa && B.s_k == S.O - S.oa) ? 1 : 0;
        const long long Kp = pl.Ko[sm];
        J.t[nt++] = OzTerm{pl.uu[sm] + (B.s_a / O) * Kp, nullptr, oz_plain(), pl.R_uu * Kp,
                           pl.t2[sm] + (B.s_b / O) * Kp, nullptr, OzRows{V * O, O, B.nz}, pl.R_t2 * Kp, (int) Kp, -1.f};
      }
      J.nterms        = nt;
      J.C             = reinterpret_cast<float2*>(slots[b]);
      J.M             = B.nx;
      J.N             = (long long) B.ny * B.nz;
      J.accumulate    = 0;
      batch.job[nj++] = J;
      max_tiles       = std::max(max_tiles, oz_gemm_tiles(J.M, J.N));
      if(nj == 3 || b == P.nblk - 1) {
        const cudaError_t e = oz_gemm_bf16(batch, nj, max_tiles, st);
        if(e != cudaSuccess) return e;
        batch     = OzBatch{};
        batch.S   = pl.S;
        nj        = 0;
        max_tiles = 0;
      }
    }
    for(int p = 0; p < 3; p++)
      for(int q = 0; q < 3; q++) {
        const int b = P.of[p][q];
        blk[p][q]   = b < 0 ? SoBlock{nullptr, 0, 0, 0, 0, 0, nullptr}
                            : SoBlock{nullptr,         P.blk[b].x0, P.blk[b].y0, P.blk[b].z0, P.blk[b].ny, P.blk[b].nz,
                                      reinterpret_cast<const float2*>(slots[b])};
      }
    return cudaSuccess;
  }
  GemmBatch       batch{};
  int             nj        = 0;
  long long       max_tiles = 0;
  for(int b = 0; b < P.nblk; b++) {
    const SoPlanBlock& B = P.blk[b];
    GemmJob            J{};
    int                nt = 0;
    if(B.has_d)
      J.t[nt++] = GemmTerm{tt + B.d_a, plain_rows(V), vv + B.d_b, RowMap{V * V, V, B.nz}, B.d_k, -1.0};
    if(B.has_s)
      J.t[nt++] = GemmTerm{uu + B.s_a, plain_rows(O), t2 + B.s_b, RowMap{V * O * O, O * O, B.nz}, B.s_k, -1.0};
    J.nterms = nt;
    J.C      = slots[b];
    J.M      = B.nx;
    J.N      = (long long) B.ny * B.nz;
    J.beta   = 0.0;
    const long long tiles = ((J.M + D_BM - 1) / D_BM) * ((J.N + D_BN - 1) / D_BN);
    if(tiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
    batch.job[nj++] = J;
    max_tiles       = std::max(max_tiles, tiles);
    if(nj == 3 || b == P.nblk - 1) {
      dmma_gemm_kernel<<<dim3((unsigned) max_tiles, 1, (unsigned) nj), D_THREADS, 0, st>>>(batch);
      const cudaError_t e = cudaGetLastError();
      if(e != cudaSuccess) return e;
      batch     = GemmBatch{};
      nj        = 0;
      max_tiles = 0;
    }
  }
  for(int p = 0; p < 3; p++)
    for(int q = 0; q < 3; q++) {
      const int b = P.of[p][q];
      blk[p][q]   = b < 0 ? SoBlock{nullptr, 0, 0, 0, 0, 0, nullptr}
                          : SoBlock{slots[b], P.blk[b].x0, P.blk[b].y0, P.blk[b].z0, P.blk[b].ny, P.blk[b].nz, nullptr};
    }
  return cudaSuccess;
}

// Device allocations of one call, released on every exit path.
struct SoArena {
  std::vector<void*> ptrs;
  cudaStream_t       streams[kSoStreams] = {};
  cudaEvent_t        ev[2 + kSoStreams]  = {};
  double*            alloc(size_t n, cudaError_t& e) {
    void* p = nullptr;
    if(e == cudaSuccess && n) e = ccsdt::dev_malloc(&p, n * sizeof(double));
    if(p) ptrs.push_back(p);
    return static_cast<double*>(p);
  }
  ~SoArena() {
    for(auto& s : streams)
      if(s) cudaStreamSynchronize(s);
    for(void* p : ptrs)
      if(p) cudaFree(p);
    for(auto& s : streams)
      if(s) cudaStreamDestroy(s);
    for(auto& x : ev)
      if(x) cudaEventDestroy(x);
  }
};

void launch_permute(const double* src, double* dst, long long n0, long long n1, long long n2, long long n3,
                    long long s0, long long s1, long long s2, long long s3, cudaStream_t st) {
  const long long total = n0 * n1 * n2 * n3;
  if(total == 0) return;
  const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 16);
  permute4_kernel<<<(unsigned) blocks, 256, 0, st>>>(src, dst, n1, n2, n3, total, s0, s1, s2, s3);
}

} // namespace

// slices = 0: FP64 DMMA contractions; 1..6: BF16 digit planes of the operands (Ozaki GEMMs on
// mma.sync, float-float blocks), the FP64 energy unchanged.
static ccsdt_status so_energy(int oa, int ob, int va, int vb, const double* eps_occ, const double* eps_vir,
                              const double* t1, const double* t2, const double* v2ijab, const double* v2ijka,
                              const double* v2iabc, int on_device, int shard_index, int shard_count, int slices,
                              double* energies, double* seconds) {
  if(oa < 0 || ob < 0 || va < 0 || vb < 0 || !energies || slices < 0 || slices > 6) return CCSDT_E_INVALID;
  if(shard_count <= 1) shard_count = 1, shard_index = 0;
  if(shard_index < 0 || shard_index >= shard_count) return CCSDT_E_INVALID;
  if(oa > 4096 || ob > 4096 || va > 4096 || vb > 4096) return CCSDT_E_INVALID;
  energies[0] = energies[1] = 0.0;
  if(seconds) *seconds = 0.0;
  const long long O = (long long) oa + ob, V = (long long) va + vb;
  if(O < 3 || V < 3) return CCSDT_OK; // no i < j < k or no a < b < c
  if(!eps_occ || !eps_vir || !t1 || !t2 || !v2ijab || !v2ijka || !v2iabc) return CCSDT_E_INVALID;
  const SoSpins   S{oa, va, (int) O, (int) V};
  const long long nmax = std::max(va, vb), slot = nmax * nmax * nmax;

  SoArena     M;
  cudaError_t e = cudaSuccess;
  for(auto& s : M.streams)
    if(e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  for(auto& x : M.ev)
    if(e == cudaSuccess) e = cudaEventCreate(&x);
  if(e != cudaSuccess) return CCSDT_E_CUDA;
  cudaStream_t st = M.streams[0];

  const double *d_eo = eps_occ, *d_ev = eps_vir, *d_t1 = t1, *d_t2 = t2, *d_ijab = v2ijab, *d_ijka = v2ijka,
               *d_iabc = v2iabc;
  double* tt = M.alloc(O * O * V * V, e);
  double* vv = M.alloc(O * V * V * V, e);
  double* uu = M.alloc(O * O * O * V, e);
  double* part = M.alloc((size_t) kSoStreams * kSoGrid * 4, e);
  double* slots[kSoStreams][9];
  for(int s = 0; s < kSoStreams; s++)
    for(int b = 0; b < 9; b++) slots[s][b] = M.alloc(slot, e);
  double* stage = nullptr;
  if(!on_device) {
    double* h[5] = {M.alloc(O, e), M.alloc(V, e), M.alloc(V * O, e), M.alloc(V * V * O * O, e),
                    M.alloc(O * O * V * V, e)};
    stage        = M.alloc(std::max(O * V * V * V, O * O * O * V), e);
    if(e != cudaSuccess) return e == cudaErrorMemoryAllocation ? CCSDT_E_OOM : CCSDT_E_CUDA;
    cudaEventRecord(M.ev[0], st);
    const double*   src[5] = {eps_occ, eps_vir, t1, t2, v2ijab};
    const long long n[5]   = {O, V, V * O, V * V * O * O, O * O * V * V};
    for(int x = 0; x < 5 && e == cudaSuccess; x++)
      e = cudaMemcpyAsync(h[x], src[x], n[x] * sizeof(double), cudaMemcpyHostToDevice, st);
    d_eo = h[0], d_ev = h[1], d_t1 = h[2], d_t2 = h[3], d_ijab = h[4];
  } else {
    if(e != cudaSuccess) return e == cudaErrorMemoryAllocation ? CCSDT_E_OOM : CCSDT_E_CUDA;
    // the call's own streams are non-blocking, so nothing orders them after the caller's work that
    // produced the inputs (on any stream, the legacy default one included): wait for all of it
    if(cudaDeviceSynchronize() != cudaSuccess) {
      cudaGetLastError();
      return CCSDT_E_CUDA;
    }
    cudaEventRecord(M.ev[0], st);
  }
  // contraction-index-contiguous copies (tt[j][k][a][e], vv[i][b][c][e], uu[j][k][a][m])
  launch_permute(d_t2, tt, O, O, V, V, O, 1, V * O * O, O * O, st);
  if(!on_device && e == cudaSuccess) {
    e      = cudaMemcpyAsync(stage, v2iabc, O * V * V * V * sizeof(double), cudaMemcpyHostToDevice, st);
    d_iabc = stage;
  }
  launch_permute(d_iabc, vv, O, V, V, V, V * V * V, V, 1, V * V, st);
  if(!on_device && e == cudaSuccess) {
    e      = cudaMemcpyAsync(stage, v2ijka, O * O * O * V * sizeof(double), cudaMemcpyHostToDevice, st);
    d_ijka = stage;
  }
  launch_permute(d_ijka, uu, O, O, V, O, O * O * V, O * V, 1, V, st);
  // split path: digit planes of tt, vv (over e) and uu, t2 (over m), per spin of the contraction index
  SoPlanes pl;
  if(slices > 0 && e == cudaSuccess) {
    pl.S    = slices;
    pl.R_tt = O * O * V, pl.R_vv = O * V * V, pl.R_uu = O * O * V, pl.R_t2 = V * V * O;
    for(int sp = 0; sp < 2 && e == cudaSuccess; sp++) {
      const long long nv = S.vn(sp), no = sp ? O - oa : oa, v0 = S.vlo(sp), o0 = sp ? oa : 0;
      pl.Kv[sp] = (nv + 31) / 32 * 32, pl.Ko[sp] = (no + 31) / 32 * 32;
      struct {
        const double*          x;
        long long              R, K, Kp, ld;
        const __nv_bfloat16**  out;
      } q[4] = {{tt + v0, pl.R_tt, nv, pl.Kv[sp], V, &pl.tt[sp]}, {vv + v0, pl.R_vv, nv, pl.Kv[sp], V, &pl.vv[sp]},
                {uu + o0, pl.R_uu, no, pl.Ko[sp], O, &pl.uu[sp]}, {d_t2 + o0, pl.R_t2, no, pl.Ko[sp], O, &pl.t2[sp]}};
      for(auto& c: q) {
        if(c.K == 0 || e != cudaSuccess) continue;
        // BF16 planes and the (unused) row exponents in one allocation of doubles
        const long long bytes = (long long) slices * c.R * c.Kp * 2 + c.R * 4;
        double*         buf   = M.alloc((size_t) ((bytes + 7) / 8), e);
        if(e != cudaSuccess) break;
        auto* planes = reinterpret_cast<__nv_bfloat16*>(buf);
        auto* exps   = reinterpret_cast<int*>(reinterpret_cast<char*>(buf) + (long long) slices * c.R * c.Kp * 2);
        oz_slice_rows_kernel<__nv_bfloat16><<<4096, 256, 0, st>>>(c.x, c.R, (int) c.K, (int) c.Kp, slices, planes,
                                                                   c.R * c.Kp, exps, c.ld);
        e      = cudaGetLastError();
        *c.out = planes;
      }
    }
    if(e != cudaSuccess) return e == cudaErrorMemoryAllocation ? CCSDT_E_OOM : CCSDT_E_CUDA;
  }
  if(e == cudaSuccess) e = cudaMemsetAsync(part, 0, (size_t) kSoStreams * kSoGrid * 4 * sizeof(double), st);
  if(e == cudaSuccess) e = cudaGetLastError();
  if(e == cudaSuccess) e = cudaEventRecord(M.ev[1], st);
  for(int s = 1; s < kSoStreams && e == cudaSuccess; s++) e = cudaStreamWaitEvent(M.streams[s], M.ev[1], 0);

  long t = 0, n = 0; // triplets seen, triplets of this shard
  for(int i = 0; i < O && e == cudaSuccess; i++)
    for(int j = i + 1; j < O && e == cudaSuccess; j++)
      for(int k = j + 1; k < O && e == cudaSuccess; k++) {
        if(t++ % shard_count != shard_index) continue;
        const int si = S.occ(i), sj = S.occ(j), sk = S.occ(k);
        const int na = S.vn(si), nb = S.vn(sj), nc = S.vn(sk);
        if((long long) na * nb * nc == 0) continue;
        const int    s  = (int) (n++ % kSoStreams);
        SoEnergyArgs A{};
        e = so_contract(S, so_plan(S, i, j, k), tt, vv, uu, d_t2, slots[s], A.blk, M.streams[s], pl);
        if(e != cudaSuccess) break;
        A.eps_o = d_eo, A.eps_v = d_ev, A.t1 = d_t1, A.v2ijab = d_ijab;
        A.O = (int) O, A.V = (int) V, A.oa = oa, A.va = va;
        A.i = i, A.j = j, A.k = k;
        A.a0 = S.vlo(si), A.na = na, A.b0 = S.vlo(sj), A.nb = nb, A.c0 = S.vlo(sk), A.nc = nc;
        A.lt_ab = si == sj, A.lt_bc = sj == sk;
        A.part  = part + (size_t) s * kSoGrid * 4;
        const long long pts  = (long long) na * nb * nc;
        const int       grid = (int) std::min<long long>(kSoGrid, (pts + kSoThreads - 1) / kSoThreads);
        so_energy_kernel<<<grid, kSoThreads, 0, M.streams[s]>>>(A);
        e = cudaGetLastError();
      }
  for(int s = 1; s < kSoStreams && e == cudaSuccess; s++) {
    e = cudaEventRecord(M.ev[1 + s], M.streams[s]);
    if(e == cudaSuccess) e = cudaStreamWaitEvent(st, M.ev[1 + s], 0);
  }
  std::vector<double> hp((size_t) kSoStreams * kSoGrid * 4);
  if(e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if(e == cudaSuccess) e = cudaEventRecord(M.ev[1], st);
  if(e == cudaSuccess) e = cudaStreamSynchronize(st);
  if(e != cudaSuccess) {
    cudaGetLastError();
    return CCSDT_E_CUDA;
  }
  CSum s4, s5;
  for(size_t b = 0; b < hp.size(); b += 4) {
    CSum o4, o5;
    o4.s = hp[b], o4.c = hp[b + 1], o5.s = hp[b + 2], o5.c = hp[b + 3];
    s4.merge(o4);
    s5.merge(o5);
  }
  energies[0] = s4.value();
  energies[1] = s5.value();
  if(seconds) {
    float ms = 0.f;
    if(cudaEventElapsedTime(&ms, M.ev[0], M.ev[1]) == cudaSuccess) *seconds = ms * 1e-3;
  }
  if(!std::isfinite(energies[0]) || !std::isfinite(energies[1])) return CCSDT_E_NONFINITE;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_energy_spin_orbital(int oa, int ob, int va, int vb, const double* eps_occ,
                                                  const double* eps_vir, const double* t1, const double* t2,
                                                  const double* v2ijab, const double* v2ijka,
                                                  const double* v2iabc, int on_device, int shard_index,
                                                  int shard_count, double* energies, double* seconds) {
  return so_energy(oa, ob, va, vb, eps_occ, eps_vir, t1, t2, v2ijab, v2ijka, v2iabc, on_device, shard_index,
                   shard_count, 0, energies, seconds);
}

extern "C" ccsdt_status ccsdt_energy_spin_orbital_split(int oa, int ob, int va, int vb, const double* eps_occ,
                                                        const double* eps_vir, const double* t1, const double* t2,
                                                        const double* v2ijab, const double* v2ijka,
                                                        const double* v2iabc, int on_device, int shard_index,
                                                        int shard_count, int slices, double* energies,
                                                        double* seconds) {
  if(slices < 1) return CCSDT_E_INVALID;
  return so_energy(oa, ob, va, vb, eps_occ, eps_vir, t1, t2, v2ijab, v2ijka, v2iabc, on_device, shard_index,
                   shard_count, slices, energies, seconds);
}

extern "C" ccsdt_status ccsdt_debug_spin_orbital_plan(int oa, int ob, int va, int vb, int i, int j, int k, int* of,
                                                      long long* blocks, int* nblk) {
  if(oa < 0 || ob < 0 || va < 0 || vb < 0 || !of || !blocks || !nblk) return CCSDT_E_INVALID;
  const int O = oa + ob, V = va + vb;
  if(!(0 <= i && i < j && j < k && k < O)) return CCSDT_E_INVALID;
  const SoPlan P = so_plan(SoSpins{oa, va, O, V}, i, j, k);
  *nblk          = P.nblk;
  for(int p = 0; p < 3; p++)
    for(int q = 0; q < 3; q++) of[3 * p + q] = P.of[p][q];
  for(int b = 0; b < P.nblk; b++) {
    const SoPlanBlock& B = P.blk[b];
    const long long    r[14] = {B.x0,  B.y0,  B.z0,  B.nx,  B.ny,  B.nz,  B.has_d,
                                B.d_k, B.d_a, B.d_b, B.has_s, B.s_k, B.s_a, B.s_b};
    for(int x = 0; x < 14; x++) blocks[14 * b + x] = r[x];
  }
  return CCSDT_OK;
}
