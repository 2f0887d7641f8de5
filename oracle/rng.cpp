// rng.cpp — ORACLE (test infrastructure only; never linked into the product).
//
// The reference draws its probes with libstdc++'s std::mt19937 and distributions; calling the
// same standard-library templates reproduces its draws exactly.  Paths inside jiang18/slemm.
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

extern "C" {

// src/reml.cpp:597-605 — Rademacher probes: V starts at +1; for column j, row i, a draw
// runif(rng) < 0.5 sets −1; columns are then normalised to unit norm (FP32).  V is n×n_V
// column-major.
void oracle_rademacher(int seed, int64_t n, int n_V, float* V)
{
  std::mt19937 rng(seed + 54321);
  std::uniform_real_distribution<float> runif(0.0, 1.0);
  for (int j = 0; j < n_V; ++j) {
    for (int64_t i = 0; i < n; ++i) V[j * n + i] = (runif(rng) < 0.5) ? -1.0f : 1.0f;
  }
  for (int j = 0; j < n_V; ++j) {
    float s = 0.0f;   // Eigen's colwise().norm() accumulates in FP32
    for (int64_t i = 0; i < n; ++i) s += V[j * n + i] * V[j * n + i];
    float nrm = std::sqrt(s);
    for (int64_t i = 0; i < n; ++i) V[j * n + i] /= nrm;
  }
}

// src/reml.cpp:795-809 — MC draws of LMC_REML: u (m×n_MC, column by column) first, then the
// residual draws e (n×n_MC, column by column) from the same generator.
void oracle_lmc_draws(int seed, int64_t m, int64_t n, int n_MC, float* u, float* e)
{
  std::mt19937 rng(seed + 54321);
  std::normal_distribution<float> rnorm(0.0, 1.0);
  for (int j = 0; j < n_MC; ++j)
    for (int64_t i = 0; i < m; ++i) u[j * m + i] = rnorm(rng);
  for (int j = 0; j < n_MC; ++j)
    for (int64_t i = 0; i < n; ++i) e[j * n + i] = rnorm(rng);
}

}  // extern "C"
