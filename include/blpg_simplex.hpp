// blpg_simplex.hpp — C++ mirror of the reference's host class over the C ABI.
//
// Reference: class Simplex (BLPG-Solver/src/simplex.cuh:37-83).  Same names,
// argument meaning and call order: construct with the batch size, set the
// shared constraints, ComputeLP with one objective row per LP (max sense),
// then read results.  Differences: the status codes are GLPK's (5 optimal,
// 6 unbounded, 4 infeasible, 1 pivot cap; the reference reports only 2 or 6,
// simplex.cu:451-461); errors throw std::runtime_error with the library's
// message instead of being ignored (simplex.cu:21-31); no cudaDeviceReset.
// Header-only; link with -lblpg.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "blpg.h"

namespace blpg {

// Dense row-major matrix with the accessors the reference's math::matrix
// offers to the solver path (A(i, j), size1(), size2(), resize).
template <typename T>
class matrix {
 public:
  matrix() = default;
  matrix(size_t r, size_t c) : r_(r), c_(c), v_(r * c) {}
  void resize(size_t r, size_t c) {
    r_ = r;
    c_ = c;
    v_.assign(r * c, T());
  }
  T& operator()(size_t i, size_t j) { return v_[i * c_ + j]; }
  const T& operator()(size_t i, size_t j) const { return v_[i * c_ + j]; }
  size_t size1() const { return r_; }
  size_t size2() const { return c_; }
  const T* data() const { return v_.data(); }
  T* data() { return v_.data(); }

 private:
  size_t r_ = 0, c_ = 0;
  std::vector<T> v_;
};

class Simplex {
 public:
  // Simplex(N_S, multipleBatch) — simplex.cu:387-400.  multipleBatch is kept
  // for signature parity; one call takes any batch size.
  explicit Simplex(unsigned int N_S, unsigned int multipleBatch = 0)
      : number_of_LPs_(N_S), multipleBatchOn_(multipleBatch) {
    blpg_options_init(&opt_);
  }

  // setConstratint (sic) — simplex.cu:463: one A, b shared by every LP.
  void setConstratint(const matrix<double>& A, const std::vector<double>& b) {
    A_ = A;
    b_ = b;
  }

  // ComputeLP — simplex.cu:552: C holds one objective row per LP (max sense).
  // number_of_streams is accepted for parity; the library's persistent launch
  // per size class replaces the reference's stream split.
  void ComputeLP(const matrix<double>& C, unsigned int number_of_streams = 1) {
    (void)number_of_streams;
    const int32_t k = (int32_t)C.size1();
    if (A_.size1() == 0 || (size_t)C.size2() != A_.size2())
      throw std::runtime_error("ComputeLP: setConstratint first, with as many columns as C");
    m_.assign(k, (int32_t)A_.size1());
    n_.assign(k, (int32_t)A_.size2());
    offA_.assign(k, 0);
    offb_.assign(k, 0);
    offc_.resize(k);
    for (int32_t i = 0; i < k; ++i) offc_[i] = (int64_t)i * (int64_t)C.size2();
    blpg_batch bt{k, m_.data(), n_.data(), offA_.data(), offb_.data(), offc_.data(),
                  A_.data(), b_.data(), C.data()};
    status_.assign(k, 0);
    result_.assign(k, 0.0);
    blpg_result res{status_.data(), result_.data(), nullptr, nullptr, nullptr, nullptr};
    const int32_t rc = blpg_solve_batch(&bt, &opt_, &res);
    if (rc != BLPG_OK) throw std::runtime_error(std::string("blpg: ") + blpg_last_error());
  }

  std::vector<double> getResultAll() const { return result_; }
  std::vector<int> getStatusAll() const { return std::vector<int>(status_.begin(), status_.end()); }
  double getResult(int n) const { return result_.at((size_t)(n - 1)); }  // 1-based
  int getStatus(int n) const { return status_.at((size_t)(n - 1)); }
  int getNo_OF_Simplx() const { return (int)number_of_LPs_; }

  // Options beyond the reference (precision, pivot cap, tuning).
  blpg_options& options() { return opt_; }

 private:
  unsigned int number_of_LPs_;
  unsigned int multipleBatchOn_;
  blpg_options opt_;
  matrix<double> A_;
  std::vector<double> b_;
  std::vector<int32_t> m_, n_, status_;
  std::vector<int64_t> offA_, offb_, offc_;
  std::vector<double> result_;
};

}  // namespace blpg
