// window.cu — iterative window weighting of the GREML SNP weights (`--iter_weighting`,
// src/option.cpp:437-530), host driver over the REML drivers of reml.cu.
//
// 1. Equal-weight GREML: DF-REML when --lrt and n < 5000 (:444-448), else MC-REML (:449-451).
// 2. snpvar_j = 2·maf_j(1 − maf_j)·b_j² from that fit's SNP-BLUP, normalised to mean 1 (:458-464).
// 3. Fixed-effect SNPs (:466-497): while the largest remaining snpvar exceeds sig_chisq, take that
//    SNP (first maximum), centre its count vector over the kept individuals, and keep it if it is
//    the first or if its residual after least squares on the SNPs already kept retains more than
//    indep_r2 of its squared norm.  Count vectors come from the packed copy on the GPU.
// 4. Window weights (:505-511): mean of snpvar over window_size + 1 neighbours (clamped at both
//    ends), mapped through 0.001/(0.001 + 0.999·exp(−x/2)); fixed SNPs get weight 0 (:523);
//    persnp ← persnp ∘ weights, normalised to mean 1 (:526-527).
// 5. Window-weighted GREML with the fixed SNPs appended to the covariates (DF-REML with --lrt,
//    else MC-REML), and each fixed SNP's BLUP entry replaced by its BLUE (:538).
// Sums over SNPs or individuals are carried in FP64 and rounded to FP32 once.
#include "internal.h"

#include <algorithm>
#include <numeric>

namespace slemm {

void reml_sldf(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
               const float* persnp, const slemm_reml_opts& o, float* Py_out, float* blup_out,
               float* blue_out, float* var_blue_out, slemm_reml_result* res);
void reml_lmc(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
              const float* persnp, const slemm_reml_opts& o, float* Py_out, float* blup_out,
              float* blue_out, slemm_reml_result* res);

// snpvar (normalised) and the window weights of src/option.cpp:458-464, 505-511.
static void window_weights(const float* maf, const float* blup, int64_t m, int window, std::vector<float>& snpvar,
                           std::vector<float>& wts)
{
  snpvar.resize(m);
  double s = 0.0;
  for (int64_t j = 0; j < m; ++j) {
    snpvar[j] = 2.0f * maf[j] * (1.0f - maf[j]) * blup[j] * blup[j];
    s += snpvar[j];
  }
  const float mean = (float)(s / (double)m);
  for (int64_t j = 0; j < m; ++j) snpvar[j] /= mean;
  std::vector<double> cs(m + 1, 0.0);
  for (int64_t j = 0; j < m; ++j) cs[j + 1] = cs[j] + snpvar[j];
  const int64_t half = window / 2;
  wts.resize(m);
  for (int64_t j = 0; j < m; ++j) {
    int64_t lo, hi;
    if (j < half) lo = 0, hi = window + 1;
    else if (j > m - half - 1) lo = m - window - 1, hi = m;
    else lo = j - half, hi = j - half + window + 1;
    const float x = (float)((cs[hi] - cs[lo]) / (double)(hi - lo));
    wts[j] = 0.001f / (0.001f + 0.999f * std::exp(x * -0.5f));
  }
}

// Solves the s×s SPD system A x = b in place (Cholesky, FP64); false if A is not positive definite.
static bool chol_solve(std::vector<double> A, int s, std::vector<double>& b)
{
  for (int j = 0; j < s; ++j) {
    double d = A[(size_t)j * s + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * s + k] * A[(size_t)j * s + k];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    A[(size_t)j * s + j] = d;
    for (int i = j + 1; i < s; ++i) {
      double v = A[(size_t)i * s + j];
      for (int k = 0; k < j; ++k) v -= A[(size_t)i * s + k] * A[(size_t)j * s + k];
      A[(size_t)i * s + j] = v / d;
    }
  }
  for (int i = 0; i < s; ++i) {
    double v = b[i];
    for (int k = 0; k < i; ++k) v -= A[(size_t)i * s + k] * b[k];
    b[i] = v / A[(size_t)i * s + i];
  }
  for (int i = s - 1; i >= 0; --i) {
    double v = b[i];
    for (int k = i + 1; k < s; ++k) v -= A[(size_t)k * s + i] * b[k];
    b[i] = v / A[(size_t)i * s + i];
  }
  return true;
}

// src/option.cpp:466-497.  Returns the fixed SNPs and their centred count columns (n × s).
static void clump(slemm_geno* g, const std::vector<float>& snpvar, float sig_chisq, float indep_r2,
                  std::vector<int64_t>& idx, std::vector<float>& cols)
{
  const int64_t n = g->n, m = (int64_t)snpvar.size();
  std::vector<float> tmp = snpvar, yv(n);
  idx.clear();
  cols.clear();
  for (;;) {
    const int64_t j = std::max_element(tmp.begin(), tmp.end()) - tmp.begin();   // first maximum
    if (!(tmp[j] > sig_chisq)) break;
    tmp[j] = 0.0f;
    int st = slemm_gpu_genotype_rows(g, &j, 1, yv.data(), n, SLEMM_MEM_HOST);
    if (st != SLEMM_OK) SLEMM_THROW(st, "genotype row decode failed");
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += yv[i];
    const float mean = (float)(s / (double)n);
    for (int64_t i = 0; i < n; ++i) yv[i] -= mean;
    bool keep = idx.empty();
    if (!keep) {
      const int k = (int)idx.size();
      std::vector<double> A((size_t)k * k, 0.0), b(k, 0.0);
      for (int a = 0; a < k; ++a) {
        const float* ca = cols.data() + (size_t)a * n;
        for (int c2 = 0; c2 <= a; ++c2) {
          const float* cb = cols.data() + (size_t)c2 * n;
          double d = 0.0;
          for (int64_t i = 0; i < n; ++i) d += (double)ca[i] * cb[i];
          A[(size_t)a * k + c2] = A[(size_t)c2 * k + a] = d;
        }
        double d = 0.0;
        for (int64_t i = 0; i < n; ++i) d += (double)ca[i] * yv[i];
        b[a] = d;
      }
      if (!chol_solve(A, k, b)) SLEMM_THROW(SLEMM_ERR_NUMERIC, "fixed-SNP Gram matrix is not positive definite");
      double rss = 0.0, yy = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        double r = yv[i];
        for (int a = 0; a < k; ++a) r -= b[a] * cols[(size_t)a * n + i];
        rss += r * r;
        yy += (double)yv[i] * yv[i];
      }
      keep = rss / yy > indep_r2;
    }
    if (keep) {
      idx.push_back(j);
      cols.insert(cols.end(), yv.begin(), yv.end());
    }
  }
  (void)m;
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_reml_iter_weighting(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                                             const float* y, const float* persnp, const float* maf,
                                             const slemm_reml_opts* opts, const slemm_window_opts* wo, float* Py,
                                             float* snp_blup, float* blue, float* var_blue, float* persnp_out,
                                             int64_t* fixed_idx, int* n_fixed, slemm_reml_result* res)
{
  return guarded([&] {
    CHECK_ARG(g && X && y && persnp && maf && opts && wo && Py && snp_blup && blue && n_fixed && res, "null argument");
    CHECK_ARG(ldx >= g->n && c >= 1, "bad covariate matrix");
    const int64_t n = g->n, m = g->m;
    CHECK_ARG(wo->window_size >= 0 && wo->window_size % 2 == 0, "window_size must be even and >= 0");
    CHECK_ARG(m >= wo->window_size + 1, "window_size >= number of SNPs");
    CHECK_ARG(wo->max_fixed >= 0, "max_fixed < 0");
    const int n_mc = wo->n_MC > 0 ? wo->n_MC : std::max(std::min((int)(4e9 / (double)n / (double)n), 30), 3);
    const int n_mc2 = wo->n_MC_final > 0 ? wo->n_MC_final : n_mc;
    // 1. equal-weight GREML
    std::vector<float> ones(m, 1.0f), py1(n), blup1(m), blue1(c), vb1((size_t)c * c);
    slemm_reml_result r1{};
    slemm_reml_opts o1 = *opts;
    if (wo->lrt && n < 5000) {
      reml_sldf(g, rvec, X, ldx, c, y, ones.data(), o1, py1.data(), blup1.data(), blue1.data(), vb1.data(), &r1);
    } else {
      o1.n_V = n_mc;
      reml_lmc(g, rvec, X, ldx, c, y, ones.data(), o1, py1.data(), blup1.data(), blue1.data(), &r1);
    }
    // 2-4. per-SNP variance, fixed SNPs, window weights
    std::vector<float> snpvar, wts, cols;
    std::vector<int64_t> idx;
    window_weights(maf, blup1.data(), m, wo->window_size, snpvar, wts);
    clump(g, snpvar, wo->sig_chisq, wo->indep_r2, idx, cols);
    const int s = (int)idx.size();
    CHECK_ARG(s <= wo->max_fixed, "more fixed-effect SNPs (" + std::to_string(s) + ") than max_fixed");
    CHECK_ARG(c + s <= SLEMM_MAX_COVARIATES,
              "covariates plus fixed-effect SNPs exceed SLEMM_MAX_COVARIATES (" + std::to_string(c + s) + ")");
    for (int64_t j : idx) wts[j] = 0.0f;
    std::vector<float> p2(m);
    double ps = 0.0;
    for (int64_t j = 0; j < m; ++j) {
      p2[j] = persnp[j] * wts[j];
      ps += p2[j];
    }
    const float pmean = (float)(ps / (double)m);
    CHECK_ARG(pmean > 0.0f, "all window-weighted SNP weights are zero");
    for (int64_t j = 0; j < m; ++j) p2[j] /= pmean;
    // 5. window-weighted GREML with the fixed SNPs as covariates
    const int c2 = c + s;
    std::vector<float> X2((size_t)n * c2);
    for (int a = 0; a < c; ++a) std::copy(X + (size_t)a * ldx, X + (size_t)a * ldx + n, X2.begin() + (size_t)a * n);
    std::copy(cols.begin(), cols.end(), X2.begin() + (size_t)c * n);
    slemm_reml_opts o2 = *opts;
    if (wo->lrt) {
      reml_sldf(g, rvec, X2.data(), n, c2, y, p2.data(), o2, Py, snp_blup, blue, var_blue, res);
    } else {
      o2.n_V = n_mc2;
      reml_lmc(g, rvec, X2.data(), n, c2, y, p2.data(), o2, Py, snp_blup, blue, res);
    }
    for (int i = 0; i < s; ++i) snp_blup[idx[i]] = blue[c + i];
    res->first_iters_V = r1.iters_V;
    res->first_n_criterion = r1.n_criterion;
    *n_fixed = s;
    if (fixed_idx) std::copy(idx.begin(), idx.end(), fixed_idx);
    if (persnp_out) std::copy(p2.begin(), p2.end(), persnp_out);
  });
}
