// Shared device/host helpers for the (T) kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccsdt {

// Row address map: element (r, kappa) of an operand lives at
//   base[(r / q) * s_hi + (r % q) * s_lo + kappa]
// which covers plain rows (q = 1 << 30) and the transposed-pair rows that the
// permuted contractions need (r = x * v + y addressing the (y, x) pair).
struct RowMap {
  long long s_hi, s_lo;
  int       q;
};

__host__ __device__ inline long long row_addr(const RowMap& m, long long r) {
  return (r / m.q) * m.s_hi + (r % m.q) * m.s_lo;
}

inline RowMap plain_rows(long long stride) { return RowMap{0, stride, 1 << 30}; }
// rows r = x * q + y  ->  (y * q + x) * stride
inline RowMap swapped_pair_rows(int q, long long stride) {
  return RowMap{stride, (long long) q * stride, q};
}

// Error-free transformation a + b = s + e (Knuth TwoSum).
__host__ __device__ inline void two_sum(double a, double b, double& s, double& e) {
  s        = a + b;
  double z = s - a;
  e        = (a - (s - z)) + (b - z);
}

// Compensated accumulator (value + running error).
struct CSum {
  double s = 0.0, c = 0.0;
  __host__ __device__ inline void add(double x) {
    double t, e;
    two_sum(s, x, t, e);
    s = t;
    c += e;
  }
  __host__ __device__ inline void merge(const CSum& o) {
    add(o.s);
    c += o.c;
  }
  __host__ __device__ inline double value() const { return s + c; }
};

} // namespace ccsdt
