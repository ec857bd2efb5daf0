// Fortran-style multi-dimensional arrays for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY. The oracle restates the reference Fortran line by
// line; giving every array its Fortran bounds (arbitrary lower bounds,
// column-major storage, first index fastest) keeps that restatement readable and
// lets each loop follow the cited reference loop directly.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <initializer_list>
#include <utility>
#include <vector>

#ifndef ORACLE_BOUNDS_CHECK
#define ORACLE_BOUNDS_CHECK 1
#endif

template <class T>
class FArr {
 public:
  FArr() = default;
  explicit FArr(std::initializer_list<std::pair<int, int>> bounds) { init(bounds); }

  void init(std::initializer_list<std::pair<int, int>> bounds) {
    rank_ = 0;
    long stride = 1;
    off_ = 0;
    for (const auto& b : bounds) {
      lo_[rank_] = b.first;
      hi_[rank_] = b.second;
      str_[rank_] = stride;
      long ext = (long)b.second - b.first + 1;
      if (ext < 0) ext = 0;
      off_ -= (long)b.first * stride;
      stride *= ext;
      ++rank_;
    }
    v_.assign((size_t)stride, T());
  }

  template <class... I>
  inline T& operator()(I... idx) {
    return v_[pos(idx...)];
  }
  template <class... I>
  inline const T& operator()(I... idx) const {
    return v_[pos(idx...)];
  }

  void fill(const T& x) { std::fill(v_.begin(), v_.end(), x); }
  size_t size() const { return v_.size(); }
  T* data() { return v_.data(); }
  const T* data() const { return v_.data(); }
  bool allocated() const { return rank_ > 0; }
  int lo(int r) const { return lo_[r]; }
  int hi(int r) const { return hi_[r]; }

 private:
  template <class... I>
  inline long pos(I... idx) const {
    const int ii[] = {static_cast<int>(idx)...};
    long p = off_;
    for (int r = 0; r < (int)sizeof...(I); ++r) {
#if ORACLE_BOUNDS_CHECK
      if (ii[r] < lo_[r] || ii[r] > hi_[r]) {
        std::fprintf(stderr, "oracle: index %d out of bounds [%d,%d] in dim %d\n", ii[r], lo_[r],
                     hi_[r], r);
        std::abort();
      }
#endif
      p += (long)ii[r] * str_[r];
    }
    return p;
  }

  std::vector<T> v_;
  int rank_ = 0;
  int lo_[8] = {0}, hi_[8] = {0};
  long str_[8] = {0};
  long off_ = 0;
};
