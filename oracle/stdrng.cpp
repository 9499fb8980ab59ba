// Test infrastructure (the oracle), not part of the product.
//
// The reference draws its random test matrix and its column shuffle from the
// C++ standard library (libstdc++): std::default_random_engine seeded with
// --seed feeding std::normal_distribution<double>{0,1} (or
// std::uniform_real_distribution<double>{-1,1}) in column-major order
// (src/Halko.cpp:15-23, src/RSVD.hpp:20-59), and std::shuffle of 0..M-1 with a
// default-constructed std::default_random_engine (src/RSVD.hpp:61-78).  The
// oracle calls the same library routines here so that its inputs are
// bit-identical to the reference's.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <random>

extern "C" {

void oracle_random_omega(int seed, int gaussian, int64_t rows, int64_t cols, double* out) {
  std::default_random_engine rng{};
  rng.seed(seed);
  const int64_t n = rows * cols;
  if (gaussian) {
    std::normal_distribution<double> dist{0, 1};
    for (int64_t i = 0; i < n; ++i) out[i] = dist(rng);
  } else {
    std::uniform_real_distribution<double> dist{-1, 1};
    for (int64_t i = 0; i < n; ++i) out[i] = dist(rng);
  }
}

void oracle_shuffle_columns(int64_t n, int32_t* out) {
  std::iota(out, out + n, 0);
  auto rng = std::default_random_engine{};
  std::shuffle(out, out + n, rng);
}

}  // extern "C"
