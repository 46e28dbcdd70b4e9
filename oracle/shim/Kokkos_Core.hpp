// Minimal Kokkos API stand-in -- TEST INFRASTRUCTURE ONLY.
//
// Kokkos itself (an empty, unpinned git submodule of the reference) is not
// available.  This header provides exactly the API subset that the
// reference's hot-path headers use, so that SimInfo.h, States.h, Update.h,
// RiemannSolvers.h, BoundaryConditions.h, ThermalConduction.h, Viscosity.h,
// ComputeDt.h and (with Kokkos_Random.hpp) Init.h compile UNMODIFIED with
// g++ -fopenmp into oracle/_ref/:
//
//   View<double****>   host LayoutRight (k,j,i,var), zero-initialised,
//                      reference counted only outside parallel regions
//                      (Kokkos disables tracking inside dispatch too)
//   deep_copy          whole-view copy, extents must match
//   Array<T,N>         aggregate with operator[]
//   MDRangePolicy<Rank<3>>, parallel_for, parallel_reduce(Max x3)
//                      OpenMP over (k,j) with i innermost
//   fabs/fmax          (Kokkos_MathematicalFunctions.hpp)
//
// Only the semantics the reference relies on are reproduced; nothing here is
// Kokkos source.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <omp.h>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}

template <class T, size_t N>
struct Array {
  T m_data[N];
  T& operator[](size_t i) { return m_data[i]; }
  const T& operator[](size_t i) const { return m_data[i]; }
  static constexpr size_t size() { return N; }
};

namespace Impl {
// Set inside parallel dispatch: View copies made there do not touch the
// reference count (as in Kokkos, where tracking is disabled in dispatch).
inline bool& in_dispatch() {
  static thread_local bool flag = false;
  return flag;
}
struct DispatchGuard {
  DispatchGuard() { in_dispatch() = true; }
  ~DispatchGuard() { in_dispatch() = false; }
};
struct ViewRecord {
  long count;
  double* data;
  std::string label;
};
}  // namespace Impl

template <class DataType>
class View;

// Rank-4 double view, LayoutRight: index ((i0*n1 + i1)*n2 + i2)*n3 + i3.
template <>
class View<double****> {
 public:
  View() = default;
  View(const std::string& label, size_t n0, size_t n1 = 0, size_t n2 = 0, size_t n3 = 0)
      : n_{n0, n1, n2, n3} {
    const size_t total = n0 * n1 * n2 * n3;
    rec_ = new Impl::ViewRecord{1, new double[total ? total : 1](), label};
    data_ = rec_->data;
  }
  View(const View& o) : data_(o.data_), n_{o.n_[0], o.n_[1], o.n_[2], o.n_[3]} {
    if (!Impl::in_dispatch() && o.rec_) {
      rec_ = o.rec_;
      ++rec_->count;
    }
  }
  View& operator=(const View& o) {
    if (this == &o) return *this;
    release();
    data_ = o.data_;
    for (int r = 0; r < 4; ++r) n_[r] = o.n_[r];
    if (!Impl::in_dispatch() && o.rec_) {
      rec_ = o.rec_;
      ++rec_->count;
    }
    return *this;
  }
  ~View() { release(); }
  double& operator()(size_t i0, size_t i1, size_t i2, size_t i3) const {
    return data_[((i0 * n_[1] + i1) * n_[2] + i2) * n_[3] + i3];
  }
  size_t extent(int r) const { return n_[r]; }
  size_t size() const { return n_[0] * n_[1] * n_[2] * n_[3]; }
  double* data() const { return data_; }
  std::string label() const { return rec_ ? rec_->label : std::string(); }

 private:
  void release() {
    if (rec_ && --rec_->count == 0) {
      delete[] rec_->data;
      delete rec_;
    }
    rec_ = nullptr;
  }
  double* data_ = nullptr;
  size_t n_[4] = {0, 0, 0, 0};
  Impl::ViewRecord* rec_ = nullptr;
};

template <class V>
void deep_copy(const V& dst, const V& src) {
  for (int r = 0; r < 4; ++r)
    if (dst.extent(r) != src.extent(r))
      throw std::runtime_error("Kokkos shim: deep_copy extents mismatch (" + dst.label() + " <- " +
                               src.label() + ")");
  std::memcpy(dst.data(), src.data(), sizeof(double) * dst.size());
}

template <unsigned N>
struct Rank {};

template <class R>
struct MDRangePolicy;

template <>
struct MDRangePolicy<Rank<3>> {
  long b[3] = {0, 0, 0};
  long e[3] = {0, 0, 0};
  MDRangePolicy() = default;
  MDRangePolicy(std::initializer_list<long> lo, std::initializer_list<long> hi) {
    int r = 0;
    for (long v : lo) b[r++] = v;
    r = 0;
    for (long v : hi) e[r++] = v;
  }
};

template <class F>
void parallel_for(const std::string&, const MDRangePolicy<Rank<3>>& p, const F& f) {
  const long b0 = p.b[0], b1 = p.b[1], b2 = p.b[2];
  const long e0 = p.e[0], e1 = p.e[1], e2 = p.e[2];
#pragma omp parallel
  {
    Impl::DispatchGuard guard;
#pragma omp for collapse(2) schedule(static)
    for (long k = b2; k < e2; ++k)
      for (long j = b1; j < e1; ++j)
        for (long i = b0; i < e0; ++i) f((int)i, (int)j, (int)k);
  }
}

template <class T>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
};

// Three Max reducers, the only parallel_reduce form the hot path uses
// (ComputeDt.h:28-54).  Each reducer starts from the lowest double.
template <class F>
void parallel_reduce(const std::string&, const MDRangePolicy<Rank<3>>& p, const F& f, Max<double> r0,
                     Max<double> r1, Max<double> r2) {
  const double lowest = std::numeric_limits<double>::lowest();
  double g0 = lowest, g1 = lowest, g2 = lowest;
  const long b0 = p.b[0], b1 = p.b[1], b2 = p.b[2];
  const long e0 = p.e[0], e1 = p.e[1], e2 = p.e[2];
#pragma omp parallel
  {
    Impl::DispatchGuard guard;
    double l0 = lowest, l1 = lowest, l2 = lowest;
#pragma omp for collapse(2) schedule(static)
    for (long k = b2; k < e2; ++k)
      for (long j = b1; j < e1; ++j)
        for (long i = b0; i < e0; ++i) f((int)i, (int)j, (int)k, l0, l1, l2);
#pragma omp critical
    {
      if (l0 > g0) g0 = l0;
      if (l1 > g1) g1 = l1;
      if (l2 > g2) g2 = l2;
    }
  }
  r0.ref = g0;
  r1.ref = g1;
  r2.ref = g2;
}

}  // namespace Kokkos

#include "Kokkos_MathematicalFunctions.hpp"
