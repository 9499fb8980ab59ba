// Host-side random streams of the operator, drawn with the C++ standard
// library exactly as the reference does: the test matrix Omega from
// std::default_random_engine seeded with --seed through
// std::normal_distribution<double>{0,1} (or uniform_real_distribution{-1,1})
// in column-major order (src/Halko.cpp:15-23, src/RSVD.hpp:20-59), and the
// in-core SNP shuffle of src/RSVD.hpp:61-70 (std::shuffle of 0..M-1 with a
// default-constructed engine).
//
// Built with FP contraction into fused multiply-adds (pcaone_gb300/build.py),
// as the reference's -march=native / -mcpu=native build contracts the polar
// method's arithmetic: the drawn matrix equals the reference's bit for bit.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <random>

namespace pcaone {

void host_random_omega(int seed, int gaussian, int64_t rows, int64_t cols, double* out_colmajor) {
  std::default_random_engine rng{};
  rng.seed(seed);
  const int64_t n = rows * cols;
  if (gaussian) {
    std::normal_distribution<double> dist{0, 1};
    for (int64_t i = 0; i < n; ++i) out_colmajor[i] = dist(rng);
  } else {
    std::uniform_real_distribution<double> dist{-1, 1};
    for (int64_t i = 0; i < n; ++i) out_colmajor[i] = dist(rng);
  }
}

void host_shuffle_columns(int64_t n, int32_t* out) {
  std::iota(out, out + n, 0);
  auto rng = std::default_random_engine{};
  std::shuffle(out, out + n, rng);
}

}  // namespace pcaone
