// Minimal stand-in for Kokkos' random pool -- TEST INFRASTRUCTURE ONLY.
//
// Init.h (the reference's problem generators) draws the H84 / C91
// perturbations from Kokkos::Random_XorShift64_Pool<> (Init.h:13, 114, 139,
// 257).  Kokkos is an empty submodule of the reference, so this header
// provides the API subset Init.h uses -- construction from a seed,
// get_state(), free_state(), drand(start, end) -- so that Init.h compiles
// unmodified.  The generator is the published xorshift64* recurrence (shift
// triple 12, 25, 27, multiplier 2685821657736338717), one state per OpenMP
// thread.  The seeding and the assignment of states to threads are this
// shim's own, not Kokkos': the values drawn are NOT the reference's, and the
// fixtures built with this header never compare the perturbation fields.
#pragma once

#include <cstdint>
#include <vector>
#include <omp.h>

namespace Kokkos {

class Random_XorShift64 {
 public:
  explicit Random_XorShift64(uint64_t s = 1) : state_(s ? s : 1) {}
  uint64_t urand64() {
    state_ ^= state_ >> 12;
    state_ ^= state_ << 25;
    state_ ^= state_ >> 27;
    return state_ * 2685821657736338717ull;
  }
  // uniform in [start, end): top 53 bits of a draw
  double drand(double start, double end) {
    const double u = (double)(urand64() >> 11) * (1.0 / 9007199254740992.0);
    return start + u * (end - start);
  }
  uint64_t state_;
};

template <class DeviceType = void>
class Random_XorShift64_Pool {
 public:
  explicit Random_XorShift64_Pool(uint64_t seed) {
    const int n = omp_get_max_threads();
    states_.resize(n);
    for (int t = 0; t < n; ++t) {
      uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(t + 1);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      states_[t] = z ^ (z >> 31);
    }
  }
  Random_XorShift64 get_state() const { return Random_XorShift64(states_[omp_get_thread_num()]); }
  void free_state(const Random_XorShift64& g) const { states_[omp_get_thread_num()] = g.state_; }

 private:
  mutable std::vector<uint64_t> states_;
};

}  // namespace Kokkos
