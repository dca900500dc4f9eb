// Minimal stand-in for the TAMM / HPTT symbols that ExaChem's CPU (T) headers use,
// so that those headers (exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp and the
// singles/doubles1/doubles2 gather headers it includes) compile unmodified here.
//
// TEST INFRASTRUCTURE ONLY: this shim is part of the oracle build (oracle/_ref),
// never of the product library.
//
// What is provided and which reference call it serves:
//   Index / IndexVector          tile ids (ccsd_t_all_fused_singles.hpp:193,200)
//   Tensor<T>::get(ids, buf)     dense block read, row-major, last index fastest
//                                (singles.hpp:200,304; doubles1.hpp:222,237,282;
//                                 doubles2.hpp:215,230,335)
//   LRUCache<K,V>::log_access    always reports a miss, so every block is re-read
//                                (singles.hpp:193; doubles1.hpp:209,274; doubles2.hpp:208,326)
//   TimerGuard                   RAII accumulator of seconds (singles.hpp:198)
//   hptt::create_plan(...)       B = alpha * transpose(A, perm) + beta * B with the
//                                row-major (numpy.transpose) meaning of perm
//                                (singles.hpp:208,310; doubles1.hpp:229,244,288;
//                                 doubles2.hpp:222,236,341)
//   exachem::cholesky_2e::V2Tensors<T>  holder of v2ijab / v2ijka / v2iabc
//                                (cholesky/v2tensors.hpp:18-33)
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <iostream>
#include <map>
#include <string>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <tuple>
#include <utility>
#include <vector>

namespace tamm {

using Index       = std::size_t;
using IndexVector = std::vector<Index>;

// Dense tiled tensor: every mode has a list of tile extents; the full array is
// stored row-major (mode 0 slowest).  get() copies one block, row-major.
template<typename T>
class Tensor {
public:
  Tensor() = default;
  Tensor(std::vector<std::vector<std::size_t>> tiles_per_mode): tiles_(std::move(tiles_per_mode)) {
    extent_.resize(tiles_.size());
    offs_.resize(tiles_.size());
    std::size_t total = 1;
    for(std::size_t m = 0; m < tiles_.size(); m++) {
      std::size_t s = 0;
      for(auto t: tiles_[m]) {
        offs_[m].push_back(s);
        s += t;
      }
      extent_[m] = s;
      total *= s;
    }
    data_.assign(total, T(0));
  }
  std::size_t rank() const { return tiles_.size(); }
  std::size_t extent(std::size_t m) const { return extent_[m]; }
  T*          data() { return data_.data(); }

  // element access with full (untiled) indices, row-major
  T& at(const std::size_t* idx) {
    std::size_t lin = 0;
    for(std::size_t m = 0; m < extent_.size(); m++) lin = lin * extent_[m] + idx[m];
    return data_[lin];
  }

  void get(const IndexVector& bid, std::vector<T>& buf) const {
    const std::size_t r = tiles_.size();
    if(bid.size() != r) throw std::runtime_error("shim Tensor::get: rank mismatch");
    std::vector<std::size_t> bext(r), boff(r);
    std::size_t              n = 1;
    for(std::size_t m = 0; m < r; m++) {
      if(bid[m] >= tiles_[m].size()) throw std::runtime_error("shim Tensor::get: tile id out of range");
      bext[m] = tiles_[m][bid[m]];
      boff[m] = offs_[m][bid[m]];
      n *= bext[m];
    }
    if(buf.size() < n) buf.resize(n);
    std::vector<std::size_t> c(r, 0);
    for(std::size_t e = 0; e < n; e++) {
      std::size_t lin = 0;
      for(std::size_t m = 0; m < r; m++) lin = lin * extent_[m] + (boff[m] + c[m]);
      buf[e] = data_[lin];
      for(std::size_t m = r; m-- > 0;) {
        if(++c[m] < bext[m]) break;
        c[m] = 0;
      }
    }
  }

private:
  std::vector<std::vector<std::size_t>> tiles_;
  std::vector<std::vector<std::size_t>> offs_;
  std::vector<std::size_t>              extent_;
  std::vector<T>                        data_;
};

} // namespace tamm

using tamm::Index;
using tamm::IndexVector;
using tamm::Tensor;

// Cache that never hits: the reference then reads and transposes every block,
// which gives the same packed buffers as a hit would.
template<typename K, typename V>
class LRUCache {
public:
  explicit LRUCache(std::size_t = 0) {}
  std::pair<bool, V&> log_access(const IndexVector&) { return {false, scratch_}; }

private:
  V scratch_;
};

class TimerGuard {
public:
  explicit TimerGuard(double* acc): acc_(acc), t0_(std::chrono::steady_clock::now()) {}
  ~TimerGuard() {
    *acc_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }

private:
  double*                               acc_;
  std::chrono::steady_clock::time_point t0_;
};

namespace hptt {

enum SelectionMethod { ESTIMATE = 0, MEASURE = 1, PATIENT = 2, CRAZY = 3 };

// Out-of-place permutation B = alpha * A^perm + beta * B.  With useRowMajor
// the arrays are row-major and output mode j is input mode perm[j], i.e. the
// same as numpy.transpose(A, perm).
template<typename T>
class Plan {
public:
  Plan(const int* perm, int dim, T alpha, const T* A, const int* size, T beta, T* B, bool rowMajor)
    : perm_(perm, perm + dim), size_(size, size + dim), alpha_(alpha), beta_(beta), A_(A), B_(B),
      rowMajor_(rowMajor) {}
  void execute() {
    if(!rowMajor_) throw std::runtime_error("shim hptt: only row-major plans are supported");
    const int                dim = (int) perm_.size();
    std::vector<std::size_t> astride(dim), bsize(dim);
    std::size_t              n = 1;
    for(int m = dim; m-- > 0;) {
      astride[m] = n;
      n *= (std::size_t) size_[m];
    }
    for(int j = 0; j < dim; j++) bsize[j] = (std::size_t) size_[perm_[j]];
    std::vector<std::size_t> c(dim, 0);
    for(std::size_t e = 0; e < n; e++) {
      std::size_t src = 0;
      for(int j = 0; j < dim; j++) src += c[j] * astride[perm_[j]];
      B_[e] = alpha_ * A_[src] + (beta_ == T(0) ? T(0) : beta_ * B_[e]);
      for(int j = dim; j-- > 0;) {
        if(++c[j] < bsize[j]) break;
        c[j] = 0;
      }
    }
  }

private:
  std::vector<int> perm_, size_;
  T                alpha_, beta_;
  const T*         A_;
  T*               B_;
  bool             rowMajor_;
};

template<typename T>
std::shared_ptr<Plan<T>> create_plan(const int* perm, int dim, T alpha, const T* A, const int* sizeA,
                                     const int* /*outerSizeA*/, T beta, T* B,
                                     const int* /*outerSizeB*/, SelectionMethod, int /*numThreads*/,
                                     const int* /*threadIds*/, bool useRowMajor) {
  return std::make_shared<Plan<T>>(perm, dim, alpha, A, sizeA, beta, B, useRowMajor);
}

// the reference passes an int literal as alpha for the t1 transpose (singles.hpp:208)
template<typename T>
std::shared_ptr<Plan<T>> create_plan(const int* perm, int dim, int alpha, const T* A, const int* sizeA,
                                     const int* outerSizeA, int beta, T* B, const int* outerSizeB,
                                     SelectionMethod m, int nt, const int* tid, bool useRowMajor) {
  return create_plan<T>(perm, dim, T(alpha), A, sizeA, outerSizeA, T(beta), B, outerSizeB, m, nt,
                        tid, useRowMajor);
}

} // namespace hptt

namespace exachem::cholesky_2e {
template<typename T>
class V2Tensors {
public:
  tamm::Tensor<T> v2ijab; // hhpp
  tamm::Tensor<T> v2ijka; // hhhp
  tamm::Tensor<T> v2iabc; // hppp
};
} // namespace exachem::cholesky_2e
