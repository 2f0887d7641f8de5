// reml.cu — REML drivers on the GPU operators: DF-REML (SLDF_REML, src/reml.cpp:549-690) and
// MC-REML (LMC_REML, src/reml.cpp:730-883).
//
// All vectors of length n or m stay in HBM; the host keeps the FP64 scalars (Lanczos/CG
// coefficients, golden-section and secant state, c×c covariate algebra).  Probe draws come
// from libstdc++'s std::mt19937 with the reference's distributions and draw order, so the GPU
// engine sees the reference's probes.
#include "internal.h"
#include "reduce.cuh"

#include <chrono>
#include <memory>
#include <random>

namespace slemm {

// ---- host dense helpers (FP64) ---------------------------------------------------------------
// Column-pivoted Householder QR of an n×c column-major matrix (the reference uses Eigen's
// ColPivHouseholderQR, src/reml.cpp:583-588).  Returns Q (n×rank), R·Pᵀ (rank×c) and the rank
// under Eigen's rule |R_ii| > eps_f32·min(n,c)·|R_00|.
struct QRHost {
  std::vector<double> Q;     // n×rank
  std::vector<double> RPt;   // rank×c (column-major)
  int rank = 0;
};

static QRHost qr_colpiv(const std::vector<double>& A0, int64_t n, int c)
{
  std::vector<double> A(A0);
  std::vector<int> perm(c);
  std::vector<double> tau(c, 0.0);
  for (int j = 0; j < c; ++j) perm[j] = j;
  auto col = [&](int j) { return A.data() + (size_t)j * n; };
  const int kmax = (int)std::min<int64_t>(n, c);
  for (int k = 0; k < kmax; ++k) {
    // pivot: largest remaining column norm
    int p = k;
    double best = -1.0;
    for (int j = k; j < c; ++j) {
      double s = 0.0;
      const double* a = col(j);
      for (int64_t i = k; i < n; ++i) s += a[i] * a[i];
      if (s > best) {
        best = s;
        p = j;
      }
    }
    if (p != k) {
      std::swap_ranges(col(k), col(k) + n, col(p));
      std::swap(perm[k], perm[p]);
    }
    double* a = col(k);
    const double nrm = std::sqrt(best);
    if (nrm == 0.0) {
      tau[k] = 0.0;
      continue;
    }
    const double alpha = a[k] >= 0 ? -nrm : nrm;
    const double v0 = a[k] - alpha;
    // v = [1, a[k+1..]/v0], tau = (alpha - a_k)/alpha ... use explicit 2/(vᵀv)
    for (int64_t i = k + 1; i < n; ++i) a[i] /= v0;
    double vtv = 1.0;
    for (int64_t i = k + 1; i < n; ++i) vtv += a[i] * a[i];
    tau[k] = 2.0 / vtv;
    a[k] = alpha;
    for (int j = k + 1; j < c; ++j) {
      double* b = col(j);
      double s = b[k];
      for (int64_t i = k + 1; i < n; ++i) s += a[i] * b[i];
      s *= tau[k];
      b[k] -= s;
      for (int64_t i = k + 1; i < n; ++i) b[i] -= s * a[i];
    }
  }
  QRHost r;
  const double maxpiv = kmax ? std::fabs(A[0]) : 0.0;
  const double thr = 1.1920928955078125e-07 * kmax * maxpiv;
  int rank = 0;
  for (int k = 0; k < kmax; ++k)
    if (std::fabs(A[(size_t)k * n + k]) > thr) ++rank;
  r.rank = rank;
  // Q = H_0 … H_{kmax−1} · I[:, :rank]
  r.Q.assign((size_t)n * rank, 0.0);
  for (int j = 0; j < rank; ++j) {
    double* q = r.Q.data() + (size_t)j * n;
    q[j] = 1.0;
    for (int k = kmax - 1; k >= 0; --k) {
      if (tau[k] == 0.0) continue;
      const double* v = col(k);
      double s = q[k];
      for (int64_t i = k + 1; i < n; ++i) s += v[i] * q[i];
      s *= tau[k];
      q[k] -= s;
      for (int64_t i = k + 1; i < n; ++i) q[i] -= s * v[i];
    }
  }
  // R·Pᵀ: column perm[j] of the result = column j of R (upper triangle)
  r.RPt.assign((size_t)rank * c, 0.0);
  for (int j = 0; j < c; ++j)
    for (int i = 0; i < rank && i <= j; ++i) r.RPt[(size_t)perm[j] * rank + i] = A[(size_t)j * n + i];
  return r;
}

// log|det M| and M^{-1} for a small c×c matrix (partial-pivot LU), column-major.
static double logabsdet(std::vector<double> M, int c, std::vector<double>* inv = nullptr)
{
  std::vector<int> piv(c);
  double ld = 0.0;
  for (int k = 0; k < c; ++k) {
    int p = k;
    for (int i = k + 1; i < c; ++i)
      if (std::fabs(M[(size_t)k * c + i]) > std::fabs(M[(size_t)k * c + p])) p = i;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < c; ++j) std::swap(M[(size_t)j * c + k], M[(size_t)j * c + p]);
    const double d = M[(size_t)k * c + k];
    ld += std::log(std::fabs(d));
    for (int i = k + 1; i < c; ++i) {
      M[(size_t)k * c + i] /= d;
      for (int j = k + 1; j < c; ++j) M[(size_t)j * c + i] -= M[(size_t)k * c + i] * M[(size_t)j * c + k];
    }
  }
  if (inv) {
    inv->assign((size_t)c * c, 0.0);
    for (int col = 0; col < c; ++col) {
      std::vector<double> b(c, 0.0);
      b[col] = 1.0;
      for (int k = 0; k < c; ++k) std::swap(b[k], b[piv[k]]);
      for (int i = 0; i < c; ++i)
        for (int j = 0; j < i; ++j) b[i] -= M[(size_t)j * c + i] * b[j];
      for (int i = c - 1; i >= 0; --i) {
        for (int j = i + 1; j < c; ++j) b[i] -= M[(size_t)j * c + i] * b[j];
        b[i] /= M[(size_t)i * c + i];
      }
      for (int i = 0; i < c; ++i) (*inv)[(size_t)col * c + i] = b[i];
    }
  }
  return ld;
}

// Solves the symmetric positive definite system M x = b (Cholesky), c small.
static std::vector<double> spd_solve(std::vector<double> M, int c, std::vector<double> b)
{
  for (int j = 0; j < c; ++j) {
    double s = M[(size_t)j * c + j];
    for (int k = 0; k < j; ++k) s -= M[(size_t)k * c + j] * M[(size_t)k * c + j];
    if (!(s > 0)) SLEMM_THROW(SLEMM_ERR_NUMERIC, "matrix not positive definite in BLUE solve");
    const double d = std::sqrt(s);
    M[(size_t)j * c + j] = d;
    for (int i = j + 1; i < c; ++i) {
      double t = M[(size_t)j * c + i];
      for (int k = 0; k < j; ++k) t -= M[(size_t)k * c + i] * M[(size_t)k * c + j];
      M[(size_t)j * c + i] = t / d;
    }
  }
  for (int i = 0; i < c; ++i) {
    for (int k = 0; k < i; ++k) b[i] -= M[(size_t)k * c + i] * b[k];
    b[i] /= M[(size_t)i * c + i];
  }
  for (int i = c - 1; i >= 0; --i) {
    for (int k = i + 1; k < c; ++k) b[i] -= M[(size_t)i * c + k] * b[k];
    b[i] /= M[(size_t)i * c + i];
  }
  return b;
}

// ---- small device kernels ---------------------------------------------------------------------
__global__ void scale_rows_kernel(float* __restrict__ X, int64_t ld, int64_t rows, int k,
                                  const float* __restrict__ s, int sqrt_of_s)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= rows) return;
  const float f = sqrt_of_s ? sqrtf(s[i]) : s[i];
  X[(int64_t)c * ld + i] *= f;
}

static void scale_rows(slemm_geno* g, float* X, int64_t ld, int64_t rows, int k, const float* s,
                       bool sq = false)
{
  dim3 gr((unsigned)ceil_div(rows, 256), k);
  scale_rows_kernel<<<gr, 256, 0, g->stream>>>(X, ld, rows, k, s, sq ? 1 : 0);
  LAUNCH_CHECK();
}

// Py[:,0] = PV[:,0]; Py[:,c] = PV[:,c] + st·PV[:,n_MC+c]   (src/reml.cpp:716-717)
__global__ void lmc_combine_kernel(const float* __restrict__ PV, float* __restrict__ Py, int64_t n,
                                   int n_MC, float st)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  if (c == 0) Py[i] = PV[i];
  else Py[(int64_t)c * n + i] = PV[(int64_t)c * n + i] + st * PV[(int64_t)(n_MC + c) * n + i];
}

// y_out[i] = r[i]·y[i] − s·rv[i]·p[i]  helper for the LMC BLUE residual (src/reml.cpp:872-874)
__global__ void lmc_resid_kernel(const float* __restrict__ y, const float* __restrict__ zb,
                                 const float* __restrict__ rvec, const float* __restrict__ Py, float tau1,
                                 int64_t n, float* __restrict__ out)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = zb[i] + tau1 * (rvec[i] * Py[i]);
  out[i] = y[i] - v;
}

static std::vector<double> d2h(slemm_geno* g, const double* d, size_t cnt)
{
  std::vector<double> h(cnt);
  CUDA_TRY(cudaMemcpyAsync(h.data(), d, cnt * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  CUDA_TRY(cudaStreamSynchronize(g->stream));
  return h;
}

// Common set-up of both drivers: rr, Q (rank check), gm, gw (src/reml.cpp:574-622, 757-781).
struct Setup {
  std::vector<float> rr, gm, gw;
  QRHost qr;
  int c = 0;
};

static Setup reml_setup(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                        const float* persnp)
{
  const int64_t n = g->n, m = g->m;
  CHECK_ARG(c >= 1 && c <= SLEMM_MAX_COVARIATES, "number of covariates must be in [1, SLEMM_MAX_COVARIATES]");
  Setup S;
  S.rr.resize(n);
  for (int64_t i = 0; i < n; ++i) {
    const float r = rvec ? rvec[i] : 1.0f;
    if (!(r > 0.f) || !std::isfinite(r)) SLEMM_THROW(SLEMM_ERR_NUMERIC, "error variance weight must be > 0");
    S.rr[i] = 1.0f / std::sqrt(r);   // Eigen rsqrt
  }
  std::vector<double> A((size_t)n * c);
  for (int j = 0; j < c; ++j)
    for (int64_t i = 0; i < n; ++i) {
      const float xv = X[(size_t)j * ldx + i];
      if (!std::isfinite(xv)) SLEMM_THROW(SLEMM_ERR_NUMERIC, "non-finite covariate");
      A[(size_t)j * n + i] = (double)(S.rr[i] * xv);
    }
  S.qr = qr_colpiv(A, n, c);
  if (S.qr.rank != c) SLEMM_THROW(SLEMM_ERR_RANK, "Fixed-effects design matrix is not of full rank.");
  S.c = c;
  // gm = nz_bits/float(n) from the GPU popcounts (bit-exact integers)
  std::vector<int64_t> pc(m);
  {
    int st = slemm_gpu_genotype_counts(g, pc.data(), nullptr, nullptr, nullptr);
    if (st != SLEMM_OK) SLEMM_THROW(st, "genotype counts failed");
  }
  S.gm.resize(m);
  for (int64_t j = 0; j < m; ++j) S.gm[j] = (int)pc[j] / (float)n;
  // gw = 1/(gm(2−gm)/2) / m · persnp/mean(persnp)  in FP32
  float psum = 0.f;
  for (int64_t j = 0; j < m; ++j) psum += persnp[j];
  const float pmean = psum / (float)m;
  S.gw.resize(m);
  for (int64_t j = 0; j < m; ++j) {
    const float v = S.gm[j] * (2.0f - S.gm[j]) / 2.0f;
    S.gw[j] = (1.0f / v) / (float)m * (persnp[j] / pmean);
    if (!std::isfinite(S.gw[j]))
      SLEMM_THROW(SLEMM_ERR_NUMERIC, "monomorphic SNP " + std::to_string(j) + " gives an infinite weight");
  }
  int st = slemm_gpu_set_weights(g, S.gm.data(), S.gw.data(), S.rr.data());
  if (st != SLEMM_OK) SLEMM_THROW(st, "set_weights failed");
  std::vector<float> Qf((size_t)n * c);
  for (size_t i = 0; i < Qf.size(); ++i) Qf[i] = (float)S.qr.Q[i];
  st = slemm_gpu_set_projection(g, Qf.data(), n, c);
  if (st != SLEMM_OK) SLEMM_THROW(st, "set_projection failed");
  return S;
}

// Orthonormal basis of the columns of an n×c matrix (column-pivoted Householder QR, FP64); returns
// the numerical rank and Q (n×rank).
int orthonormal_columns(const std::vector<double>& A, int64_t n, int c, std::vector<double>& Q)
{
  QRHost r = qr_colpiv(A, n, c);
  Q = std::move(r.Q);
  return r.rank;
}

static void upload(slemm_geno* g, float* d, const float* h, size_t cnt)
{
  CUDA_TRY(cudaMemcpyAsync(d, h, cnt * sizeof(float), cudaMemcpyHostToDevice, g->stream));
}

// The search's evaluation points and criterion values into the result (the first SLEMM_TRACE_MAX).
static void store_trace(slemm_reml_result* res, const std::vector<std::pair<float, double>>& tr)
{
  res->n_points = (int)std::min<size_t>(tr.size(), SLEMM_TRACE_MAX);
  for (int q = 0; q < res->n_points; ++q) {
    res->h2_points[q] = tr[q].first;
    res->f_points[q] = tr[q].second;
  }
}

// ================================================================================================
// DF-REML
// ================================================================================================
struct Criterion {
  double slogLL, vg, ve, lrt;
};

void reml_sldf(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
               const float* persnp, const slemm_reml_opts& o, float* Py_out, float* blup_out,
               float* blue_out, float* var_blue_out, slemm_reml_result* res)
{
  const auto t_start = std::chrono::steady_clock::now();
  auto stamp = [&]() {
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  };
  const int64_t n = g->n, m = g->m;
  const bool verbose = o.verbose != 0;
  if (verbose) printf("\nStarted stochastic Lanczos DF-REML.\n");
  cudaStream_t st = g->stream;
  const int n_V = o.n_V;
  CHECK_ARG(n_V >= 1, "n_V must be >= 1");
  CHECK_ARG(c >= 1 && c <= SLEMM_MAX_COVARIATES, "number of covariates must be in [1, SLEMM_MAX_COVARIATES]");
  // One block [y_proj | Q | V] (t = 1 + c + n_V) through one Lanczos recurrence: column 0 uses
  // the projected operator (seed_y, H0_quadform_mv), the rest the plain one (seed_Q and seed_V,
  // H0_ldet_mv); each of the three groups keeps its own stopping rule, as the reference's three
  // L_Seed calls do (src/reml.cpp:627-631).
  const int tQV = 1 + c + n_V;
  DevBuf d_y(g->stream), d_QV(g->stream), d_X(g->stream), d_tmp(g->stream);
  d_y.ensure((size_t)n * sizeof(float));
  d_QV.ensure((size_t)n * tQV * sizeof(float));
  d_X.ensure((size_t)n * tQV * sizeof(float));
  // scalars: projection coefficients (up to c×c) first, one more value from offset c·c
  d_tmp.ensure((size_t)std::max<int64_t>(n, m) * 4 * sizeof(double) + ((size_t)c * c + 64) * sizeof(double));
  // Rademacher probes (src/reml.cpp:597-605), the reference's mt19937 draws generated on the GPU;
  // launched first so that the host set-up below runs while they are drawn
  rademacher_device(o.seed, n, n_V, d_QV.as<float>() + (size_t)(1 + c) * n, n, g->stream);
  Setup S = reml_setup(g, rvec, X, ldx, c, persnp);
  // y_proj = (I − QQᵀ)(rr∘y)   (src/reml.cpp:591-592), FP64 on the host
  std::vector<float> yproj(n);
  {
    std::vector<double> ry(n);
    for (int64_t i = 0; i < n; ++i) ry[i] = (double)(S.rr[i] * y[i]);
    for (int l = 0; l < c; ++l) {
      const double* q = S.qr.Q.data() + (size_t)l * n;
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += q[i] * ry[i];
      for (int64_t i = 0; i < n; ++i) ry[i] -= s * q[i];
    }
    for (int64_t i = 0; i < n; ++i) yproj[i] = (float)ry[i];
  }
  if (verbose) printf("Projected covariates out of phenotypes.\nGenerating %d Rademacher probing vectors.\n", n_V);
  std::vector<float> QV((size_t)n * (1 + c));
  std::copy(yproj.begin(), yproj.end(), QV.begin());
  for (size_t i = 0; i < (size_t)n * c; ++i) QV[(size_t)n + i] = (float)S.qr.Q[i];
  upload(g, d_y.as<float>(), yproj.data(), n);
  upload(g, d_QV.as<float>(), QV.data(), (size_t)n * (1 + c));
  const double t_a = stamp();
  double* d_scal = d_tmp.as<double>();

  const float tau0 = (1.0f - o.s2max) / o.s2max;
  if (verbose) printf("\nPerforming Lanczos decomposition for phenotypes, covariates and Rademacher vectors:\n");
  slemm_lseed* seed = lanczos_seed_device(g, SLEMM_OP_LDET, tau0, d_QV.as<float>(), tQV, o.tol_L, o.maxit,
                                          verbose, {1, c, n_V}, 5, 1);
  std::unique_ptr<slemm_lseed, void (*)(slemm_lseed*)> hold(seed, lseed_free);
  constexpr int GY = 0, GQ = 1, GV = 2;
  const double t_b = stamp();
  const int nld = lseed_iters(seed, GV);
  // Jacobi matrices of the probes (columns 1+c ... c+n_V), src/reml.cpp:638-646
  std::vector<double> dl((size_t)n_V * nld), bt((size_t)n_V * (nld + 1));
  {
    const double* D = lseed_delta(seed);
    const double* B = lseed_beta(seed);
    for (int j = 0; j < nld; ++j)
      for (int p = 0; p < n_V; ++p) dl[(size_t)j * n_V + p] = D[(size_t)j * tQV + 1 + c + p];
    for (int j = 0; j <= nld; ++j)
      for (int p = 0; p < n_V; ++p) bt[(size_t)j * n_V + p] = B[(size_t)j * tQV + 1 + c + p];
  }
  // Gauss quadrature nodes and weights of every probe (FP64, host threads)
  std::vector<double> DV((size_t)n_V * nld), W2((size_t)n_V * nld);
  tridiag_eig_host(dl.data(), bt.data(), n_V, nld, DV.data(), W2.data());

  // Moments of the stored basis: every shifted solve the criterion needs is a combination
  // X = Σ_i coef_i·V_i of the seed vectors (V_0 = the right-hand side), so yᵀX and QᵀX follow
  // from the inner products y·V_i[:,0] and Q_k·V_i[:,1+l], computed once here in one pass.
  const int Jy = lseed_iters(seed, GY), JQ = lseed_iters(seed, GQ);
  const int Jm = std::max(Jy, JQ);
  std::vector<std::pair<int, int>> pairs;
  pairs.push_back({0, 0});
  for (int k = 0; k < c; ++k)
    for (int l = 0; l < c; ++l) pairs.push_back({1 + k, 1 + l});
  const int npairs = (int)pairs.size();
  std::vector<double> mom;
  lanczos_moments(seed, pairs, Jm, mom);
  const double ySy = mom[0];
  int n_eval = 0;
  std::vector<std::pair<float, double>> trace;
  // REML_criterion (src/reml.cpp:457-489)
  auto criterion = [&](float ss) -> Criterion {
    ++n_eval;
    const float tau = (1 - ss) / ss;
    const float sigma = tau - tau0;
    std::vector<double> cy, cq;
    const int sy = solve_coeffs(seed, (double)sigma, 1e-6, GY, cy);
    double yPy = 0.0;
    for (int i = 0; i < sy; ++i) yPy += cy[i] * mom[(size_t)i * npairs];
    Criterion r;
    r.vg = yPy / (double)(n - c);
    r.ve = r.vg * tau;
    double ldet_H = 0.0;   // SLQ_LDet (src/reml.cpp:440-451)
    for (size_t q = 0; q < DV.size(); ++q) ldet_H += W2[q] * std::log(DV[q] + sigma);
    ldet_H = ldet_H * (double)n / (double)n_V;
    r.lrt = (double)n * std::log(ySy / yPy) - ldet_H;
    const int sq = solve_coeffs(seed, (double)sigma, 1e-6, GQ, cq);
    std::vector<double> M((size_t)c * c, 0.0);   // M[k][l] = Q_kᵀ X_l, row-major
    for (int i = 0; i < sq; ++i)
      for (int k = 0; k < c; ++k)
        for (int l = 0; l < c; ++l)
          M[(size_t)k * c + l] += cq[(size_t)i * c + l] * mom[(size_t)i * npairs + 1 + k * c + l];
    r.slogLL = (double)(n - c) * std::log(ySy / yPy) - logabsdet(M, c) - ldet_H;
    trace.push_back({ss, r.slogLL});
    return r;
  };
  // REML_GSS (src/reml.cpp:493-547)
  const double invphi = 0.618033988749894848204586834365638117720309179805762862135;
  const double invphi2 = 0.381966011250105151795413165634361882279690820194237137864;
  float a = o.s2min, b = o.s2max;
  if (verbose) printf("\nDoing golden section search in (%g, %g)\n", a, b);
  float h = b - a;
  int nitr = (h < o.tol_VC) ? 1 : (int)std::ceil(std::log(o.tol_VC / h) / std::log(invphi));
  if (verbose) printf("%d iterations:\n", nitr);
  float cc = (float)(a + invphi2 * h), dd = (float)(a + invphi * h);
  Criterion fc = criterion(cc), fd = criterion(dd), last = fd;
  for (int i = 0; i < nitr; ++i) {
    double fm;
    if (fc.slogLL > fd.slogLL) {
      b = dd;
      dd = cc;
      fd = fc;
      h = (float)(h * invphi);
      cc = (float)(a + invphi2 * h);
      fc = criterion(cc);
      last = fc;
      fm = fc.slogLL;
    } else {
      a = cc;
      cc = dd;
      fc = fd;
      h = (float)(h * invphi);
      dd = (float)(a + invphi * h);
      fd = criterion(dd);
      last = fd;
      fm = fd.slogLL;
    }
    if (verbose) printf("Itr %d: h2 in (%g, %g) and 2logLL = %g\n", i + 1, a, b, fm);
  }
  if (verbose) printf("\nCompleted golden section search.\n");
  const float vg = (float)last.vg, ve = (float)last.ve, lrt = (float)last.lrt;
  const float tau1 = ve / vg;

  const double t_c = stamp();
  // Py = rr∘(I−QQᵀ)L_Solve(seed_y, y_proj, τ1−τ0)   (src/reml.cpp:659-661)
  float* d_Py = d_X.as<float>();
  lanczos_solve_device(seed, (double)(tau1 - tau0), 1e-6, d_Py, n, GY);
  proj_coeffs(g, d_Py, n, 1, d_scal);
  proj_apply(g, d_Py, n, 1, d_scal);
  scale_rows(g, d_Py, n, n, 1, g->rr.as<float>());
  // snp_blup = W Z_cᵀ Py  (src/reml.cpp:662)
  DevBuf d_b(g->stream);
  d_b.ensure((size_t)m * sizeof(float));
  op_device(g, SLEMM_OP_WRMATVEC, 0.f, d_Py, n, 1, d_b.as<float>(), m);
  CUDA_TRY(cudaMemcpyAsync(Py_out, d_Py, n * sizeof(float), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(blup_out, d_b.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
  check_device_error(g);
  if (verbose) printf("\nVg,%g\nVe,%g\nh2,%g\nLRT,%g\n", vg, ve, vg / (vg + ve), lrt);

  // BLUE and var(BLUE) (src/reml.cpp:674-677): with rr∘X = Q·qrR,
  //   XᵀH⁻¹X = qrRᵀ (Qᵀ S) qrR and (H⁻¹X)ᵀy = qrRᵀ Sᵀ(rr∘y), S = L_Solve(seed_Q, Q, τ1−τ0)
  float* d_S = d_X.as<float>();
  lanczos_solve_device(seed, (double)(tau1 - tau0), 1e-6, d_S, n, GQ);
  proj_coeffs(g, d_S, n, c, d_scal);
  std::vector<double> QtS = d2h(g, d_scal, (size_t)c * c);
  {
    std::vector<float> ry(n);
    for (int64_t i = 0; i < n; ++i) ry[i] = S.rr[i] * y[i];
    upload(g, d_y.as<float>(), ry.data(), n);
  }
  std::vector<double> Sty(c);
  for (int l = 0; l < c; ++l) {
    col_dots(g, d_S + (size_t)l * n, n, d_y.as<float>(), n, n, 1, d_scal + (size_t)c * c);
    Sty[l] = d2h(g, d_scal + (size_t)c * c, 1)[0];
  }
  const std::vector<double>& R = S.qr.RPt;   // c×c
  std::vector<double> XtHX((size_t)c * c, 0.0), rhs(c, 0.0), T((size_t)c * c, 0.0);
  for (int i = 0; i < c; ++i)          // T = (QᵀS)·R
    for (int j = 0; j < c; ++j) {
      double s = 0.0;
      for (int k = 0; k < c; ++k) s += QtS[(size_t)i * c + k] * R[(size_t)j * c + k];   // (QᵀS)[i][k] is row-major
      T[(size_t)j * c + i] = s;
    }
  for (int i = 0; i < c; ++i)          // XtHX = Rᵀ T
    for (int j = 0; j < c; ++j) {
      double s = 0.0;
      for (int k = 0; k < c; ++k) s += R[(size_t)i * c + k] * T[(size_t)j * c + k];
      XtHX[(size_t)j * c + i] = s;
    }
  for (int i = 0; i < c; ++i) {        // rhs = Rᵀ (Sᵀ rr∘y)
    double s = 0.0;
    for (int k = 0; k < c; ++k) s += R[(size_t)i * c + k] * Sty[k];
    rhs[i] = s;
  }
  // symmetrise (the product is symmetric in exact arithmetic)
  for (int i = 0; i < c; ++i)
    for (int j = 0; j < i; ++j) {
      const double v = 0.5 * (XtHX[(size_t)j * c + i] + XtHX[(size_t)i * c + j]);
      XtHX[(size_t)j * c + i] = XtHX[(size_t)i * c + j] = v;
    }
  std::vector<double> blue = spd_solve(XtHX, c, rhs);
  std::vector<double> inv;
  logabsdet(XtHX, c, &inv);
  for (int i = 0; i < c; ++i) blue_out[i] = (float)blue[i];
  if (var_blue_out)
    for (size_t q = 0; q < (size_t)c * c; ++q) var_blue_out[q] = (float)(inv[q] * vg);
  if (verbose) {
    printf("\nCompleted stochastic Lanczos DF-REML.\n");
    if (o.s2max - vg / (vg + ve) < o.tol_VC)
      printf("\nWarning: the h2 estimate is virtually the same as the max you specified.\nRerun with a higher --max_heritability.\n");
  }
  if (res) {
    res->vg = vg;
    res->ve = ve;
    res->h2 = vg / (vg + ve);
    res->lrt = lrt;
    res->iters_y = lseed_iters(seed, GY);
    res->iters_Q = lseed_iters(seed, GQ);
    res->iters_V = nld;
    res->n_criterion = n_eval;
    store_trace(res, trace);
    res->seconds = stamp();
    res->t_setup = t_a;
    res->t_seed = t_b - t_a;
    res->t_search = t_c - t_b;
    res->t_final = res->seconds - t_c;
  }
}

// ================================================================================================
// MC-REML
// ================================================================================================
void reml_lmc(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
              const float* persnp, const slemm_reml_opts& o, float* Py_out, float* blup_out,
              float* blue_out, slemm_reml_result* res)
{
  const auto t_start = std::chrono::steady_clock::now();
  auto stamp = [&]() {
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  };
  const int64_t n = g->n, m = g->m;
  const bool verbose = o.verbose != 0;
  if (verbose) printf("\nStarted Lanczos MC-REML.\n");
  Setup S = reml_setup(g, rvec, X, ldx, c, persnp);
  cudaStream_t st = g->stream;
  const int n_MC = o.n_V;
  CHECK_ARG(n_MC >= 1, "n_MC must be >= 1");
  const int tV = 1 + 2 * n_MC;
  // draws: u (m×n_MC) then e (n×n_MC) from one generator (src/reml.cpp:795-809)
  std::vector<float> u((size_t)m * n_MC), V((size_t)n * tV);
  {
    if (verbose) printf("Generating %d MC samples for genetic effects.\n", n_MC);
    std::mt19937 rng(o.seed + 54321);
    std::normal_distribution<float> rnorm(0.0, 1.0);
    for (int j = 0; j < n_MC; ++j)
      for (int64_t i = 0; i < m; ++i) u[(size_t)j * m + i] = rnorm(rng);
    if (verbose) printf("Generating %d MC samples for residuals.\n", n_MC);
    for (int j = 1 + n_MC; j < tV; ++j)
      for (int64_t i = 0; i < n; ++i) V[(size_t)j * n + i] = rnorm(rng);
  }
  for (int64_t i = 0; i < n; ++i) V[i] = y[i];
  DevBuf d_V(g->stream), d_u(g->stream), d_PV(g->stream), d_Py(g->stream), d_ub(g->stream),
      d_tmp(g->stream), d_aux(g->stream);
  d_V.ensure((size_t)n * tV * sizeof(float));
  d_u.ensure((size_t)m * n_MC * sizeof(float));
  d_PV.ensure((size_t)n * tV * sizeof(float));
  d_Py.ensure((size_t)n * (1 + n_MC) * sizeof(float));
  d_ub.ensure((size_t)m * (1 + n_MC) * sizeof(float));
  // scratch: c×tV projection coefficients first, then 4·tV norms from offset c·tV
  const size_t scal_off = (size_t)c * tV;
  d_tmp.ensure((scal_off + 4 * (size_t)tV) * sizeof(double));
  double* d_scal = d_tmp.as<double>();
  upload(g, d_V.as<float>(), V.data(), (size_t)n * tV);
  upload(g, d_u.as<float>(), u.data(), (size_t)m * n_MC);
  // u *= sqrt(gw); V[:,1:1+n_MC] = Z_c u   (src/reml.cpp:801-802)
  scale_rows(g, d_u.as<float>(), m, m, n_MC, g->w.as<float>(), true);
  op_device(g, SLEMM_OP_MATVEC, 0.f, d_u.as<float>(), m, n_MC, d_V.as<float>() + n, n);
  // V[:, :1+n_MC] *= rr; V −= QQᵀV   (src/reml.cpp:812-813)
  if (verbose) printf("Projecting covariates out of phenotypes and MC samples.\n");
  scale_rows(g, d_V.as<float>(), n, n, 1 + n_MC, g->rr.as<float>());
  proj_coeffs(g, d_V.as<float>(), n, tV, d_scal);
  proj_apply(g, d_V.as<float>(), n, tV, d_scal);

  const double t_a = stamp();
  const float tau0 = (1.0f - o.s2max) / o.s2max;
  if (verbose) printf("\nPerforming Lanczos decomposition:\n");
  slemm_lseed* seed_V = lanczos_seed_device(g, SLEMM_OP_QUADFORM, tau0, d_V.as<float>(), tV, 10 * o.tol_L,
                                            o.maxit, verbose, {}, 5);
  std::unique_ptr<slemm_lseed, void (*)(slemm_lseed*)> hold(seed_V, lseed_free);
  int n_eval = 0;
  std::vector<std::pair<float, double>> trace;
  // REML_first_order (src/reml.cpp:696-728); leaves rr-scaled Py in d_Py
  auto first_order = [&](float ss) -> float {
    ++n_eval;
    const float tau = (1 - ss) / ss;
    const float sigma = tau - tau0;
    lanczos_solve_device(seed_V, (double)sigma, 1e-6, d_PV.as<float>(), n, 0);
    dim3 gr((unsigned)ceil_div(n, 256), 1 + n_MC);
    lmc_combine_kernel<<<gr, 256, 0, st>>>(d_PV.as<float>(), d_Py.as<float>(), n, n_MC, std::sqrt(tau));
    LAUNCH_CHECK();
    proj_coeffs(g, d_Py.as<float>(), n, 1 + n_MC, d_scal);
    proj_apply(g, d_Py.as<float>(), n, 1 + n_MC, d_scal);
    col_dots(g, d_Py.as<float>(), n, nullptr, 0, n, 1 + n_MC, d_scal + scal_off);              // ‖e‖²
    scale_rows(g, d_Py.as<float>(), n, n, 1 + n_MC, g->rr.as<float>());
    op_device(g, SLEMM_OP_RMATVEC, 0.f, d_Py.as<float>(), n, 1 + n_MC, d_ub.as<float>(), m);
    scale_rows(g, d_ub.as<float>(), m, m, 1 + n_MC, g->w.as<float>(), true);
    col_dots(g, d_ub.as<float>(), m, nullptr, 0, m, 1 + n_MC, d_scal + scal_off + (1 + n_MC));   // ‖u‖²
    std::vector<double> h = d2h(g, d_scal + scal_off, 2 * (1 + n_MC));
    double e0 = h[0], u0 = h[1 + n_MC], es = 0.0, us = 0.0;
    for (int q = 1; q <= n_MC; ++q) {
      es += h[q];
      us += h[1 + n_MC + q];
    }
    const float f = (float)std::log((u0 / e0) / (us / es));
    trace.push_back({ss, (double)f});
    return f;
  };
  const double t_b = stamp();
  if (verbose) printf("\nSecant iterations:\n");
  float s2 = o.s2max / 2;
  float log_tau1 = std::log((1 - s2) / s2);
  float f1 = first_order(s2);
  if (verbose) printf("  Iter 1: h2=%.4f log((1-h2)/h2)=%.4f funct=%.4f\n", s2, log_tau1, f1);
  s2 = (f1 < 0) ? o.s2max / 4 : o.s2max;
  float log_tau2 = std::log((1 - s2) / s2);
  float f2 = first_order(s2);
  if (verbose) printf("  Iter 2: h2=%.4f log((1-h2)/h2)=%.4f funct=%.4f\n", s2, log_tau2, f2);
  for (int si = 3; si <= 9; ++si) {
    float lt = (log_tau1 * f2 - log_tau2 * f1) / (f2 - f1);
    if (lt > 9) lt = 9;
    else if (lt < -9) lt = -9;
    if (std::fabs(lt - log_tau2) < 0.002) break;
    s2 = 1 / (std::exp(lt) + 1);
    f1 = f2;
    f2 = first_order(s2);
    log_tau1 = log_tau2;
    log_tau2 = lt;
    if (verbose) printf("  Iter %d: h2=%.4f log((1-h2)/h2)=%.4f funct=%.4f\n", si, s2, lt, f2);
  }
  if (verbose && std::fabs(f2) > 0.005)
    printf("\nWarning: secant iterations not converged. h2 close to 0 or small sample size?\n");
  const double t_c = stamp();
  // Py = PyMC[:,0]; vg = y·Py/(n−c); ve = τ1·vg   (src/reml.cpp:855-858)
  float* d_Py0 = d_Py.as<float>();
  {
    std::vector<float> hy(y, y + n);
    upload(g, d_PV.as<float>(), hy.data(), n);
  }
  col_dots(g, d_PV.as<float>(), n, d_Py0, n, n, 1, d_scal);
  const double yPy = d2h(g, d_scal, 1)[0];
  const float vg = (float)(yPy / (double)(n - c));
  const float tau1 = (1 - s2) / s2;
  const float ve = tau1 * vg;
  // snp_blup = W Z_cᵀ Py
  op_device(g, SLEMM_OP_WRMATVEC, 0.f, d_Py0, n, 1, d_ub.as<float>(), m);
  CUDA_TRY(cudaMemcpyAsync(Py_out, d_Py0, n * sizeof(float), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(blup_out, d_ub.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
  // BLUE: y − (Z_c b + τ1·R∘Py), then (XᵀX)⁻¹Xᵀ(·)   (src/reml.cpp:872-875)
  float* d_zb = d_V.as<float>();   // reuse
  op_device(g, SLEMM_OP_MATVEC, 0.f, d_ub.as<float>(), m, 1, d_zb, n);
  {
    std::vector<float> rv(n);
    for (int64_t i = 0; i < n; ++i) rv[i] = rvec ? rvec[i] : 1.0f;
    d_aux.ensure((size_t)n * 2 * sizeof(float));
    upload(g, d_aux.as<float>(), rv.data(), n);
    lmc_resid_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(d_PV.as<float>(), d_zb, d_aux.as<float>(), d_Py0,
                                                                  tau1, n, d_aux.as<float>() + n);
    LAUNCH_CHECK();
  }
  std::vector<float> resid(n);
  CUDA_TRY(cudaMemcpyAsync(resid.data(), d_aux.as<float>() + n, n * sizeof(float), cudaMemcpyDeviceToHost, st));
  check_device_error(g);
  {
    std::vector<double> XtX((size_t)c * c, 0.0), Xtr(c, 0.0);
    for (int a = 0; a < c; ++a) {
      const float* xa = X + (size_t)a * ldx;
      for (int b = 0; b <= a; ++b) {
        const float* xb = X + (size_t)b * ldx;
        double s = 0.0;
        for (int64_t i = 0; i < n; ++i) s += (double)xa[i] * xb[i];
        XtX[(size_t)b * c + a] = XtX[(size_t)a * c + b] = s;
      }
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += (double)xa[i] * resid[i];
      Xtr[a] = s;
    }
    std::vector<double> blue = spd_solve(XtX, c, Xtr);
    for (int a = 0; a < c; ++a) blue_out[a] = (float)blue[a];
  }
  if (verbose) {
    printf("\nVg,%g\nVe,%g\nh2,%g\n", vg, ve, s2);
    printf("\nCompleted Lanczos MC-REML.\n");
    if (s2 > o.s2max)
      printf("\nWarning: the h2 estimate is larger than the max you specified.\nCan rerun with a higher --max_heritability to gain accuracy.\n");
  }
  if (res) {
    res->vg = vg;
    res->ve = ve;
    res->h2 = s2;
    res->lrt = 0.f;
    res->iters_y = res->iters_Q = 0;
    res->iters_V = lseed_iters(seed_V, 0);
    res->n_criterion = n_eval;
    store_trace(res, trace);
    res->seconds = stamp();
    res->t_setup = t_a;
    res->t_seed = t_b - t_a;
    res->t_search = t_c - t_b;
    res->t_final = res->seconds - t_c;
  }
}

}  // namespace slemm

using namespace slemm;

// ================================================================================================
// REML log-likelihood gradient
// ================================================================================================
// In the rr-transformed space (ỹ = rr∘y, X̃ = rr∘X, Z̃ = rr∘Z_c) the model of the DF-REML path is
//   Ṽ = σ_g²·Z̃WZ̃ᵀ + σ_e²·I,   W_j = gw_j·w_{window_j},
// gw the reference's per-SNP weights (src/reml.cpp:613-622) and w one weight per window of SNPs
// (1 outside every window).  ℓ = −½[log|Ṽ| + log|X̃ᵀṼ⁻¹X̃| + ỹᵀP̃ỹ] has
//   ∂ℓ/∂θ = −½[tr(P̃·∂Ṽ/∂θ) − ỹᵀP̃(∂Ṽ/∂θ)P̃ỹ].
// With H = Z̃WZ̃ᵀ + τI (τ = σ_e²/σ_g²), P̃ = P_H/σ_g² where P_H = (I−QQᵀ)H̃⁺(I−QQᵀ) is the projected
// solve of the DF-REML path (H0_quadform_mv at shift τ).  Traces take the reference's normalised
// Rademacher probes v (tr(A) ≈ (n/n_V)·Σ_v vᵀAv, src/reml.cpp:597-605); per SNP
//   a_j = (z̃_jᵀP_Hỹ)²,   b_j = (n/n_V)·Σ_v (z̃_jᵀP_Hv)(z̃_jᵀv),
// and
//   ∂ℓ/∂σ_g² = −½[Σ_j W_j·b_j/σ_g² − Σ_j W_j·a_j/σ_g⁴]
//   ∂ℓ/∂σ_e² = −½[tr(P_H)/σ_g² − ‖P_Hỹ‖²/σ_g⁴],   tr(P_H) ≈ (n/n_V)·Σ_v vᵀP_Hv
//   ∂ℓ/∂w_k  = −½·Σ_{j ∈ window k} gw_j·[b_j − a_j/σ_g²].
// The per-SNP terms of every window come from one packed product Z̃ᵀ[P_Hỹ | P_HV | V] (column-
// scaled FP16 hi+lo), the transposed product the operators use, reduced per window on the device in
// FP64 (grad_window_kernel).
// Per-SNP terms of the gradient from T = Z̃ᵀ[P_Hỹ | P_HV | V] (column-major, m rows), computed in
// FP64 where they are reduced: a_j = t_{0,j}², b_j = scale·Σ_v t_{1+v,j}·t_{1+n_V+v,j}.
__device__ __forceinline__ void grad_terms(const float* __restrict__ T, int64_t m, int n_V, double scale, int64_t j,
                                           double& a, double& b)
{
  const double t0 = T[j];
  double s = 0.0;
  for (int v = 0; v < n_V; ++v) s = fma((double)T[(int64_t)(1 + v) * m + j], (double)T[(int64_t)(1 + n_V + v) * m + j], s);
  a = t0 * t0;
  b = s * scale;
}

// The adjoint's reduction, fused with the per-SNP terms: blocks [0, n_runs) each reduce one run of
// consecutive SNPs of one window (runs[3r …] = first SNP, end, window), part[2r …] = Σ gw_j·(a_j, b_j);
// blocks from n_runs each reduce a chunk of all m SNPs weighted by W_j (the handle's weights,
// gw·wwin), glob[2b …] = Σ W_j·(a_j, b_j).  The partials are summed in a fixed order afterwards, so
// the gradient is bit-reproducible.
constexpr int kGradChunk = 8192;
__global__ void __launch_bounds__(256)
grad_window_kernel(const float* __restrict__ T, int64_t m, int n_V, double scale, const float* __restrict__ gw,
                   const float* __restrict__ W, const int64_t* __restrict__ runs, int n_runs,
                   double* __restrict__ part, double* __restrict__ glob)
{
  __shared__ double sh[32];
  int64_t j0, j1;
  const float* wt;
  double* dst;
  if ((int)blockIdx.x < n_runs) {
    j0 = runs[3 * (int64_t)blockIdx.x];
    j1 = runs[3 * (int64_t)blockIdx.x + 1];
    wt = gw;
    dst = part + 2 * (int64_t)blockIdx.x;
  } else {
    const int64_t b = (int64_t)blockIdx.x - n_runs;
    j0 = b * kGradChunk;
    j1 = min64(m, j0 + kGradChunk);
    wt = W;
    dst = glob + 2 * b;
  }
  double sa = 0.0, sb = 0.0;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    double a, b;
    grad_terms(T, m, n_V, scale, j, a, b);
    const double w = (double)wt[j];
    sa = fma(w, a, sa);
    sb = fma(w, b, sb);
  }
  sa = block_sum_d(sa, sh);
  sb = block_sum_d(sb, sh);
  if (threadIdx.x == 0) {
    dst[0] = sa;
    dst[1] = sb;
  }
}

// grad[0] = −½(Σ W·b/σ_g² − Σ W·a/σ_g⁴) from the chunk partials (thread 0), and for window q
// (thread q + 1) grad[2 + q] = −½(Σ gw·b − Σ gw·a/σ_g²) over its runs, taken in SNP order from the
// CSR lists wrun_off / wrun.  grad[1] is the host's (it needs no per-SNP term).
__global__ void grad_window_final_kernel(const double* __restrict__ part, const double* __restrict__ glob, int nglob,
                                         const int* __restrict__ wrun_off, const int* __restrict__ wrun, int n_win,
                                         double sg2, double* __restrict__ grad)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    double sa = 0.0, sb = 0.0;
    for (int b = 0; b < nglob; ++b) {
      sa += glob[2 * b];
      sb += glob[2 * b + 1];
    }
    grad[0] = -0.5 * (sb / sg2 - sa / (sg2 * sg2));
  } else if (t <= n_win) {
    const int q = t - 1;
    double ga = 0.0, gb = 0.0;
    for (int r = wrun_off[q]; r < wrun_off[q + 1]; ++r) {
      ga += part[2 * (int64_t)wrun[r]];
      gb += part[2 * (int64_t)wrun[r] + 1];
    }
    grad[2 + q] = -0.5 * (gb - ga / sg2);
  }
}

void reml_grad(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
               const float* persnp, const int32_t* window, int n_win, const float* wwin, double sg2,
               double se2, int n_V, int seed, float tol, double* grad)
{
  const int64_t n = g->n, m = g->m;
  cudaStream_t st = g->stream;
  const int t = 1 + n_V, k = 1 + 2 * n_V;
  DevBuf d_B(st), d_X(st), d_U(st), d_T(st), d_s(st);
  d_B.ensure((size_t)n * t * sizeof(float));
  // probes straight into the block, drawn while the host set-up runs
  rademacher_device(seed, n, n_V, d_B.as<float>() + n, n, st);
  Setup S = reml_setup(g, rvec, X, ldx, c, persnp);
  std::vector<float> W(m);
  for (int64_t j = 0; j < m; ++j) W[j] = S.gw[j] * ((window && window[j] >= 0) ? wwin[window[j]] : 1.0f);
  {
    const int s2 = slemm_gpu_set_weights(g, S.gm.data(), W.data(), S.rr.data());
    if (s2 != SLEMM_OK) SLEMM_THROW(s2, "set_weights failed");
  }
  // ỹ_proj = (I − QQᵀ)(rr∘y) on the host in FP64, as the DF-REML path
  std::vector<float> yproj(n);
  {
    std::vector<double> ry(n);
    for (int64_t i = 0; i < n; ++i) ry[i] = (double)(S.rr[i] * y[i]);
    for (int l = 0; l < c; ++l) {
      const double* q = S.qr.Q.data() + (size_t)l * n;
      double sum = 0.0;
      for (int64_t i = 0; i < n; ++i) sum += q[i] * ry[i];
      for (int64_t i = 0; i < n; ++i) ry[i] -= sum * q[i];
    }
    for (int64_t i = 0; i < n; ++i) yproj[i] = (float)ry[i];
  }
  upload(g, d_B.as<float>(), yproj.data(), n);
  // U's last n_V columns keep the raw probes; the block's get projected
  d_U.ensure((size_t)n * k * sizeof(float));
  CUDA_TRY(cudaMemcpyAsync(d_U.as<float>() + (size_t)(1 + n_V) * n, d_B.as<float>() + n, (size_t)n * n_V * sizeof(float),
                           cudaMemcpyDeviceToDevice, st));
  // scalars: c×t projection coefficients, then the trace and norm dots from offset c·t
  const size_t qoff = (size_t)std::max(c, 1) * t;
  double* d_scal = (double*)d_s.ensure(qoff * sizeof(double) + 2 * (size_t)t * sizeof(double));
  proj_coeffs(g, d_B.as<float>() + n, n, n_V, d_scal);
  proj_apply(g, d_B.as<float>() + n, n, n_V, d_scal);
  // P_H[ỹ | V] by one projected Lanczos seed at shift τ, solved at σ = 0 (groups ỹ, probes)
  const float tau = (float)(se2 / sg2);
  slemm_lseed* sd = lanczos_seed_device(g, SLEMM_OP_QUADFORM, tau, d_B.as<float>(), t, tol, 600, false, {1, n_V}, 5, t);
  std::unique_ptr<slemm_lseed, void (*)(slemm_lseed*)> hold(sd, lseed_free);
  d_X.ensure((size_t)n * t * sizeof(float));
  lanczos_solve_device(sd, 0.0, 1e-6, d_X.as<float>(), n, 0);
  lanczos_solve_device(sd, 0.0, 1e-6, d_X.as<float>() + n, n, 1);
  proj_coeffs(g, d_X.as<float>(), n, t, d_scal);
  proj_apply(g, d_X.as<float>(), n, t, d_scal);
  // tr(P_H) ≈ (n/n_V)·Σ_v vᵀP_Hv and ‖P_Hỹ‖²
  double* d_dots = d_scal + qoff;
  col_dots(g, d_U.as<float>() + (size_t)(1 + n_V) * n, n, d_X.as<float>() + n, n, n, n_V, d_dots);
  col_dots(g, d_X.as<float>(), n, nullptr, 0, n, 1, d_dots + n_V);
  const std::vector<double> dots = d2h(g, d_dots, (size_t)n_V + 1);
  double vPv = 0.0;
  for (int v = 0; v < n_V; ++v) vPv += dots[v];
  const double trP = vPv * (double)n / (double)n_V, pyy = dots[n_V];
  // Z̃ᵀ[P_Hỹ | P_HV | V]: rr∘ on the rows, then the transposed packed product
  CUDA_TRY(cudaMemcpyAsync(d_U.as<float>(), d_X.as<float>(), (size_t)n * t * sizeof(float), cudaMemcpyDeviceToDevice,
                           st));
  scale_rows(g, d_U.as<float>(), n, n, k, g->rr.as<float>());
  d_T.ensure((size_t)m * k * sizeof(float));
  const int prec = g->prec;
  g->prec = SLEMM_PREC_FP16X2;
  try {
    op_device(g, SLEMM_OP_RMATVEC, 0.f, d_U.as<float>(), n, k, d_T.as<float>(), m);
  } catch (...) {
    g->prec = prec;
    throw;
  }
  g->prec = prec;
  // Per-window reduction on the device, fused with the per-SNP terms: runs of consecutive SNPs of
  // one window (one run per window when windows are contiguous), reduced by one block each; only
  // the 2 + n_win gradient entries come back.
  std::vector<int64_t> runs;   // first SNP, end, window
  if (window) {
    for (int64_t j = 0; j < m;) {
      const int q = window[j];
      int64_t e = j + 1;
      while (e < m && window[e] == q) ++e;
      if (q >= 0) runs.insert(runs.end(), {j, e, (int64_t)q});
      j = e;
    }
  }
  const int n_runs = (int)(runs.size() / 3);
  std::vector<int> wrun_off((size_t)std::max(n_win, 0) + 1, 0), wrun(n_runs);
  for (int r = 0; r < n_runs; ++r) ++wrun_off[runs[3 * r + 2] + 1];
  for (int q = 0; q < n_win; ++q) wrun_off[q + 1] += wrun_off[q];
  {
    std::vector<int> fill(wrun_off.begin(), wrun_off.end() - 1);
    for (int r = 0; r < n_runs; ++r) wrun[fill[runs[3 * r + 2]]++] = r;   // a window's runs in SNP order
  }
  const int nglob = (int)ceil_div(m, kGradChunk);
  DevBuf d_gw(st), d_runs(st), d_wrun(st), d_part(st), d_grad(st);
  d_gw.ensure((size_t)m * sizeof(float));
  d_runs.ensure(std::max<size_t>(runs.size(), 1) * sizeof(int64_t));
  d_wrun.ensure(((size_t)n_win + 1 + n_runs) * sizeof(int));
  double* part = (double*)d_part.ensure(2 * ((size_t)n_runs + nglob) * sizeof(double));
  double* d_g = (double*)d_grad.ensure(((size_t)n_win + 2) * sizeof(double));
  upload(g, d_gw.as<float>(), S.gw.data(), m);
  if (n_runs) {
    CUDA_TRY(cudaMemcpyAsync(d_runs.p, runs.data(), runs.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_wrun.as<int>() + n_win + 1, wrun.data(), (size_t)n_runs * sizeof(int),
                             cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(cudaMemcpyAsync(d_wrun.p, wrun_off.data(), ((size_t)n_win + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  grad_window_kernel<<<(unsigned)(n_runs + nglob), 256, 0, st>>>(d_T.as<float>(), m, n_V, (double)n / (double)n_V,
                                                                   d_gw.as<float>(), g->w.as<float>(),
                                                                   d_runs.as<int64_t>(), n_runs, part,
                                                                   part + 2 * (size_t)n_runs);
  LAUNCH_CHECK();
  grad_window_final_kernel<<<(unsigned)ceil_div(n_win + 1, 256), 256, 0, st>>>(
      part, part + 2 * (size_t)n_runs, nglob, d_wrun.as<int>(), d_wrun.as<int>() + n_win + 1, n_win, sg2, d_g);
  LAUNCH_CHECK();
  const std::vector<double> gv = d2h(g, d_g, (size_t)n_win + 2);
  check_device_error(g);
  grad[0] = gv[0];
  grad[1] = -0.5 * (trP / sg2 - pyy / (sg2 * sg2));
  for (int q = 0; q < n_win; ++q) grad[2 + q] = gv[2 + q];
}

extern "C" {

int slemm_gpu_reml_sldf(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
                        const float* persnp, const slemm_reml_opts* opts, float* Py, float* snp_blup,
                        float* blue, float* var_blue, slemm_reml_result* res)
{
  return guarded([&] {
    CHECK_ARG(g && X && y && persnp && opts && Py && snp_blup && blue, "null argument");
    CHECK_ARG(ldx >= g->n, "ldx < n");
    CHECK_ARG(opts->s2max > opts->s2min && opts->s2min > 0 && opts->s2max < 1, "bad h2 bounds");
    reml_sldf(g, rvec, X, ldx, c, y, persnp, *opts, Py, snp_blup, blue, var_blue, res);
  });
}

int slemm_gpu_reml_lmc(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
                       const float* persnp, const slemm_reml_opts* opts, float* Py, float* snp_blup,
                       float* blue, slemm_reml_result* res)
{
  return guarded([&] {
    CHECK_ARG(g && X && y && persnp && opts && Py && snp_blup && blue, "null argument");
    CHECK_ARG(ldx >= g->n, "ldx < n");
    CHECK_ARG(opts->s2max > 0 && opts->s2max < 1, "bad h2 bound");
    reml_lmc(g, rvec, X, ldx, c, y, persnp, *opts, Py, snp_blup, blue, res);
  });
}

int slemm_gpu_reml_grad(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
                        const float* persnp, const int32_t* window, int n_win, const float* wwin, double sigma_g2,
                        double sigma_e2, int n_V, int seed, float tol, double* grad)
{
  return guarded([&] {
    CHECK_ARG(g && X && y && persnp && grad, "null argument");
    CHECK_ARG(ldx >= g->n && c >= 1 && c <= SLEMM_MAX_COVARIATES, "bad covariate matrix");
    CHECK_ARG(n_win >= 0 && (n_win == 0 || (window && wwin)), "windows given without their weights");
    CHECK_ARG(sigma_g2 > 0.0 && sigma_e2 > 0.0 && std::isfinite(sigma_g2) && std::isfinite(sigma_e2),
              "variance components must be positive");
    CHECK_ARG(n_V >= 1 && n_V <= 256, "n_V out of [1, 256]");
    CHECK_ARG(tol > 0.f, "tol must be positive");
    for (int q = 0; q < n_win; ++q) CHECK_ARG(wwin[q] > 0.f && std::isfinite(wwin[q]), "window weights must be > 0");
    if (window)
      for (int64_t j = 0; j < g->m; ++j) CHECK_ARG(window[j] >= -1 && window[j] < n_win, "window index out of range");
    reml_grad(g, rvec, X, ldx, c, y, persnp, window, n_win, wwin, sigma_g2, sigma_e2, n_V, seed, tol, grad);
  });
}

}  // extern "C"
