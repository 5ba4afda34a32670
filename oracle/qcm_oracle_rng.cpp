// Seeded Gaussian start vector of the reference: a fresh
// std::default_random_engine(seed) drawing from std::normal_distribution(0,1)
// (src_util/vector_num.cpp:114-119, distribution at
// src_ed/Hamiltonian/Lanczos.cpp:7).  Normalization is left to the caller.
// Test infrastructure only.
#include <cstddef>
#include <random>

extern "C" void qo_seeded_normal(size_t n, unsigned seed, double* out) {
  std::normal_distribution<double> dist(0.0, 1.0);
  std::default_random_engine gen(seed);
  for (size_t i = 0; i < n; ++i) out[i] = dist(gen);
}
