// Split-precision (Ozaki) contractions: slicing, slice GEMMs, float-float recombination.
//
// Every operand row r (length K along the contraction) is scaled by 2^-e_r, with e_r the
// smallest exponent such that max_k |x[r,k]| (1 + 2^-7) < 2^e_r, and written as
//   x[r,k] = 2^e_r  sum_{p=1..S} 2^{-7p} sigma_p[r,k],   sigma_p integer,
//   |sigma_1| <= 127, |sigma_p| <= 64 (p > 1)   (round-to-nearest digit extraction).
// Each digit is exact in BF16 and in INT8.  The product of two rows is then
//   sum_k x y = 2^{e_x + e_y} sum_{l=2..S+1} 2^{-7l} L_l,   L_l = sum_{p+q=l} sum_k sigma_p tau_q.
// For K <= 512 every L_l (l <= 7) is an integer below 2^24, so it is EXACT in an FP32
// tensor-core accumulator (and in INT32 for the INT8 variant); the levels are combined in
// float-float (pairs of FP32, ~48 bits), not FP64, because FP64 issue on GB300 is 1/64 of FP32.
// Products with p + q > S + 1 are dropped; that truncation is the method's only error.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace ccsdt {

constexpr int OZ_BITS = 7;
constexpr int OZ_MAX_SLICES = 8;

// ---------------------------------------------------------------------------------- float-float
// Products and sums that feed error terms are written with the _rn intrinsics, which the compiler
// never contracts into fused multiply-adds, so every kernel that inlines these helpers rounds the
// same way.
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  float s = a + b, z = s - a;
  return ff{s, (a - (s - z)) + (b - z)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = ff_two_sum(a.hi, b.hi);
  float lo = s.lo + a.lo + b.lo;
  float hi = s.hi + lo;
  return ff{hi, lo - (hi - s.hi)};
}
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  ff s = ff_two_sum(a.hi, b);
  float lo = s.lo + a.lo;
  float hi = s.hi + lo;
  return ff{hi, lo - (hi - s.hi)};
}
// a * s for any float s: error-free product of the high word (fma), so the result keeps
// float-float precision (for s = 3, say, a.hi * s alone would round at 2^-25)
__device__ __forceinline__ ff ff_mul_f(ff a, float s) {
  const float p = __fmul_rn(a.hi, s), e = __fmaf_rn(a.hi, s, -p);
  const float lo = __fmaf_rn(a.lo, s, e);
  const float hi = __fadd_rn(p, lo);
  return ff{hi, lo - (hi - p)};
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  float hi = __fadd_rn(p, e);
  return ff{hi, e - (hi - p)};
}
// a / b from an approximate reciprocal (__fdividef: a few ulp) and one float-float correction
// step: q1 = a.hi / b.hi (approx.), r = a - q1 b (float-float), q2 = r.hi / b.hi (approx.);
// relative error ~2^-44, at a fraction of the cost of two IEEE divisions.
__device__ __forceinline__ ff ff_div_fast(ff a, ff b) {
  const float rb = __fdividef(1.f, b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  const ff    r  = ff_add(a, ff_neg(ff_mul(ff{q1, 0.f}, b)));
  const float q2 = __fmul_rn(r.hi, rb);
  const float h  = __fadd_rn(q1, q2);
  return ff{h, q2 - (h - q1)};
}
// Running float-float sum of products p + e (p rounded, e its error and low-order terms):
// high words by an error-free two-sum, low words added, one renormalisation at the end.
struct ffacc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float p, float e) {
    const float s = hi + p, z = s - hi;
    lo += ((hi - (s - z)) + (p - z)) + e;
    hi = s;
  }
  __device__ __forceinline__ void add_sq(ff w) { // + w^2
    const float p = __fmul_rn(w.hi, w.hi);
    add(p, __fadd_rn(__fmaf_rn(w.hi, w.hi, -p), __fmul_rn(__fmul_rn(2.f, w.hi), w.lo)));
  }
  __device__ __forceinline__ void add_mul_f(ff w, float y) { // + w y
    const float p = __fmul_rn(w.hi, y);
    add(p, __fadd_rn(__fmaf_rn(w.hi, y, -p), __fmul_rn(w.lo, y)));
  }
  __device__ __forceinline__ ff get() const {
    const float h = hi + lo;
    return ff{h, lo - (h - hi)};
  }
};
__device__ __forceinline__ ff ff_from_double(double x) {
  float hi = (float) x;
  return ff{hi, (float) (x - (double) hi)};
}

// 2^e as a float from its exponent bits (no libm call): exact for -126 <= e <= 127; below that
// the scale (and the contribution it multiplies, under 2^-126 of the operands' units) flushes to
// zero, above it the result is +inf.
__device__ __forceinline__ float oz_pow2(int e) {
  return e < -126 ? 0.f : __int_as_float((min(e, 128) + 127) << 23);
}

// Horner fold of S exact level sums (most significant first) into an unnormalised float-float
// X = sum_l L[l] 2^{7 (S - 1 - l)}.  Each level is an integer multiple of one power of two g (the
// element's row-scale product, carried by the BF16 digits), |L| < 2^24 g.  A step is Fast2Sum of
// a = 128 hi (exact) and b = L[l]: s = fl(a + b), z = fl(s - a), e = b - z.  It is error-free
// here in either order of |a|, |b|: for |a| >= |b| by Dekker's theorem; for |a| < |b| both are
// integer multiples of g below 2^24 g, so the rounding error of s is 0 or +-g and s - a = b + error
// is a multiple of g below 2^24 g, held exactly.  fma forms the 128 hi products without rounding
// (4 operations per level; the first level's low word is e itself).  The result is exact for
// S <= 4; at S = 5 the low-word update can round (relative < 2^-46).  The caller renormalises
// once, after its last addition.
template<int S, int W = 16>
__device__ __forceinline__ ff oz_horner(const uint32_t (&L)[S][W], int e) {
  float hi = __uint_as_float(L[0][e]), lo = 0.f;
#pragma unroll
  for(int l = 1; l < S; l++) {
    const float b = __uint_as_float(L[l][e]);
    const float s = fmaf(hi, 128.f, b), z = fmaf(hi, -128.f, s);
    lo            = l == 1 ? b - z : fmaf(lo, 128.f, b - z);
    hi            = s;
  }
  return ff{hi, lo};
}

// The same fold rounded to FP32 (one rounding per level step): for partial arrays stored in FP32,
// whose element error is then a few FP32 roundings, far below the truncation of one or two digit
// planes.
template<int S, int W = 16>
__device__ __forceinline__ float oz_horner_f32(const uint32_t (&L)[S][W], int e) {
  float x = __uint_as_float(L[0][e]);
#pragma unroll
  for(int l = 1; l < S; l++) x = __fmaf_rn(x, 128.f, __uint_as_float(L[l][e]));
  return x;
}

// ---------------------------------------------------------------------------------- slicing
// Rows of a dense FP64 array [R][K] -> S digit planes [S][R][Kp] (Kp >= K, zero padded) and
// exponents e[R].  One warp per row.  Row r ~ 2^e[r] sum_p d_p 2^{-7 (p + 1)} with integer digits
// |d_0| <= 127, |d_p| <= 64.  BF16 planes hold d_p 2^e[r] (exact: 7 significant bits), so every
// product in a contraction's dot product for output (y, n) carries the same power of two
// 2^(e_y + e_n) and the level sums stay exact integer multiples of it; the epilogues need no row
// or column scale.  Rows under 2^-126 flush to zero digits.  INT8 planes hold d_p and the kernels
// that read them scale by the exponents.
template<typename T>
__device__ __forceinline__ T oz_digit(double d, int e);
template<>
__device__ __forceinline__ __nv_bfloat16 oz_digit<__nv_bfloat16>(double d, int e) {
  return __float2bfloat16_rn((float) d * oz_pow2(e));
}
template<>
__device__ __forceinline__ int8_t oz_digit<int8_t>(double d, int) {
  return (int8_t) (int) d;
}

// Row r of the source is x[r * ld .. r * ld + K) (ld = K for a dense array; larger to slice a
// column range of each row).
template<typename T>
__global__ void oz_slice_rows_kernel(const double* __restrict__ x, long long R, int K, int Kp, int S,
                                     T* __restrict__ out, long long plane, int* __restrict__ exps, long long ld) {
  const int       lane = threadIdx.x & 31;
  const long long warps = (long long) gridDim.x * (blockDim.x >> 5);
  for(long long r = (long long) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += warps) {
    const double* row = x + r * ld;
    double        mx  = 0.0;
    for(int k = lane; k < K; k += 32) mx = fmax(mx, fabs(row[k]));
#pragma unroll
    for(int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    int e = 0;
    if(mx > 0.0) frexp(mx * (1.0 + 1.0 / 128.0), &e); // mx (1 + 2^-7) < 2^e
    if(lane == 0) exps[r] = e;
    for(int k = lane; k < Kp; k += 32) {
      double y = k < K ? ldexp(row[k], -e) : 0.0;
      for(int p = 0; p < S; p++) {
        y        = y * 128.0;
        double d = rint(y);
        y        = y - d;
        out[(long long) p * plane + r * Kp + k] = oz_digit<T>(d, e);
      }
    }
  }
}

// ---------------------------------------------------------------------------------- GEMM
// One term: sum over kappa of A(m, kappa) B(n, kappa), each operand given as digit planes.
// Row r of an operand lives at plane base + rid(r) * Kp, rid(r) = (r / q) * h + (r % q) * l.
struct OzRows {
  long long h, l;
  int       q;
};
__host__ __device__ inline long long oz_rid(const OzRows& m, long long r) { return (r / m.q) * m.h + (r % m.q) * m.l; }
inline OzRows oz_plain() { return OzRows{0, 1, 1 << 30}; }
inline OzRows oz_swapped(int q) { return OzRows{1, q, q}; } // r = x q + y -> y q + x

struct OzTerm {
  const void* A;       // digit planes of A: plane stride planeA elements
  const int*  eA;      // exponents, indexed by rid (nullptr: BF16 digits that carry their row scale)
  OzRows      ma;
  long long   planeA;
  const void* B;
  const int*  eB;
  OzRows      mb;
  long long   planeB;
  int         Kp;      // padded contraction length (multiple of the k chunk)
  float       sign;
};

struct OzJob {
  OzTerm    t[2];
  int       nterms;
  float2*   C; // ff output [M][N]
  long long M, N;
  int       accumulate; // 0: C = result, 1: C += result
};

struct OzBatch {
  OzJob job[3];
  int   S; // slices used (<= planes stored)
};

} // namespace ccsdt
