// rng.cpp — ORACLE (test infrastructure only; never linked into the product).
//
// The reference draws its probes with libstdc++'s std::mt19937 and distributions; calling the
// same standard-library templates reproduces its draws exactly.  Paths inside jiang18/slemm.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
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

// src/reml.cpp:919-925 — --lmm marker sample: SNPs with gm·n > 20 and (2 − gm)·n > 20 in file
// order, shuffled by std::random_shuffle (libstdc++, std::rand); the reference never seeds rand,
// so its state is the C library's initial one (= srand(1)).  Writes the first min(nqf, count)
// indices; returns that number.
int oracle_lmm_variants(const float* gm, int64_t m, int64_t n, int nqf, int64_t* out)
{
  std::vector<int> variants;
  for (int i = 0; i < (int)m; ++i)
    if (gm[i] * n > 20 && (2 - gm[i]) * n > 20) variants.push_back(i);
  std::srand(1);
  std::random_shuffle(variants.begin(), variants.end());
  const int k = std::min(nqf, (int)variants.size());
  for (int i = 0; i < k; ++i) out[i] = variants[i];
  return k;
}

// The C library's rand() sequence after srand(seed) (count values).
void oracle_libc_rand(unsigned seed, int count, int* out)
{
  std::srand(seed);
  for (int i = 0; i < count; ++i) out[i] = std::rand();
}

}  // extern "C"
