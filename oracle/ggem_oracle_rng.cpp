// ggem_oracle_rng.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference draws its Brownian noise with std::default_random_engine and
// std::normal_distribution<double> (random_generator.h:195,
// random_generator.C:43-67), reseeding once from `random_seed`
// (copss.C:1389 -> random_generator.C:96-99) and building a fresh
// distribution object per vector (random_generator.C:53-54).  This oracle
// makes exactly those library calls, so it reproduces the reference stream
// on the same C++ standard library.
#include <cstdint>
#include <random>

#include "ggem_oracle.h"

extern "C" void orc_std_normal_vector(uint64_t seed, int64_t skip_vectors,
                                      int64_t n, double mean, double stddev,
                                      double *out) {
  std::default_random_engine gen;
  gen.seed(static_cast<std::size_t>(seed));
  for (int64_t v = 0; v <= skip_vectors; ++v) {
    std::normal_distribution<double> dist(mean, stddev);
    dist.reset();
    for (int64_t i = 0; i < n; ++i) {
      const double x = dist(gen);
      if (v == skip_vectors) out[i] = x;
    }
  }
}
