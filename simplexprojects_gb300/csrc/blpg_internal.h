// Internal declarations shared by the host translation units of libblpg.so.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <string>

#include "../../include/blpg.h"

namespace blpg {

// Record a printf-style message for blpg_last_error() and return `code`.
int32_t fail(int32_t code, const char* fmt, ...);

// Counter-based random stream (SplitMix64).  LP k of a workload draws from
// Rng(seed + k), so every LP can be regenerated independently.  All floating
// point here is plain IEEE arithmetic compiled without contraction, so x86
// and Arm hosts produce bit-identical workloads.
struct Rng {
  uint64_t s;
  static uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) : s(mix(seed)) {}
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // Uniform on [0, 1) with 53 random bits.
  double u01() { return (double)(next() >> 11) * 0x1.0p-53; }
  double uniform(double a, double b) {
    double w = (b - a) * u01();
    return a + w;
  }
  // Uniform integer on [0, k).
  int32_t below(int32_t k) {
    int32_t v = (int32_t)(u01() * (double)k);
    return v < k ? v : k - 1;
  }
  double normal();  // N(0, 1), Marsaglia's polar method
};

// Natural log and exp from range reduction and series only (no libm), so the
// generator does not depend on the host's libm rounding.
double det_log(double x);
double det_exp(double x);

}  // namespace blpg
