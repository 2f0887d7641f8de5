// lmm.cu — GWAS step 1 quadratic forms (`--lmm` with real markers, src/reml.cpp:919-981): the
// per-marker statistics of the .gstat.txt file that slemm_gamma.py and slemm_gwa.py read.
//
// Marker sample (:919-925): markers with gm·n > 20 and (2 − gm)·n > 20 in file order, shuffled by
// libstdc++'s std::random_shuffle (for i = 1 … N−1: swap(v[i], v[rand() % (i+1)])) driven by the C
// library's rand() in its initial state — glibc's TYPE_3 additive-feedback generator
// (r_i = r_{i−3} + r_{i−31} mod 2^32, output r_i ≫ 1, state from the seed by the Park–Miller
// recurrence 16807·r mod 2^31−1, first 310 outputs discarded), restated here with seed 1.
//
// For the first num_qf markers x (centred counts): xPy = xᵀPy; v = (I − QQᵀ)(rr∘x);
// xPx = vᵀ(H0 + τ1 I)⁻¹v through one projected Lanczos seed on all v and one solve at shift 0;
// xSx = ‖v‖²; xBx = (xSx − zᵀ(ZᵀZ + τ1·diag(1/gw))⁻¹z)/τ1 where Z holds the projected, rr-scaled
// centred counts of the window_size markers around x (clamped at both ends) and z = Zᵀv.
//
// GB300 mapping: ZᵀZ and z come out of one packed tensor-core product per window,
// Z_wdᵀ[U | rr∘v] with U = rr∘(I − QQᵀ)(rr∘Cc) — the centred counts Cc are read from the packed
// copy, never materialised as a dense Z — using column-scaled FP16 hi+lo (≈ FP32 accuracy, like the
// reference's SGEMM).  The windows' systems are then factored together, one CTA per window:
// blocked FP32 Cholesky in global memory (L2-resident), then two steps of iterative refinement
// with FP64 residuals, so the quadratic form is limited by the Gram's own accuracy, not by the
// FP32 factorisation.
#include "internal.h"
#include "reduce.cuh"
#include "dense.cuh"

#include <algorithm>
#include <memory>

namespace slemm {

// ---- C library rand() and std::random_shuffle, restated -----------------------------------------
namespace {
struct LibcRand {
  uint32_t r[34];
  int i = 0;   // ring position
  explicit LibcRand(uint32_t seed)
  {
    std::vector<int64_t> v(344);
    v[0] = seed;
    for (int k = 1; k < 31; ++k) {
      const int64_t hi = v[k - 1] / 127773, lo = v[k - 1] % 127773;
      int64_t w = 16807 * lo - 2836 * hi;   // 16807·r mod (2^31 − 1) without overflow (Schrage)
      if (w < 0) w += 2147483647;
      v[k] = w;
    }
    for (int k = 31; k < 34; ++k) v[k] = v[k - 31];
    std::vector<uint32_t> u(v.begin(), v.begin() + 34);
    for (int k = 34; k < 344; ++k) u.push_back(u[k - 31] + u[k - 3]);
    for (int k = 0; k < 34; ++k) r[k] = u[310 + k];   // the last 34 words of the warm-up
  }
  int next()
  {
    // r holds words k−34 … k−1 (ring); word k = word k−31 + word k−3
    const uint32_t w = r[(i + 34 - 31) % 34] + r[(i + 34 - 3) % 34];
    r[i] = w;
    i = (i + 1) % 34;
    return (int)(w >> 1);
  }
};
}  // namespace

// src/reml.cpp:919-925: the sampled markers (first min(num_qf, count)).
static std::vector<int64_t> lmm_variants(const std::vector<float>& gm, int64_t n, int num_qf)
{
  std::vector<int> v;
  for (int i = 0; i < (int)gm.size(); ++i)
    if (gm[i] * (float)n > 20.0f && (2.0f - gm[i]) * (float)n > 20.0f) v.push_back(i);
  LibcRand rnd(1);
  for (size_t i = 1; i < v.size(); ++i) {
    const size_t j = (size_t)rnd.next() % (i + 1);
    if (i != j) std::swap(v[i], v[j]);
  }
  const int k = std::min<int>(num_qf, (int)v.size());
  return std::vector<int64_t>(v.begin(), v.begin() + k);
}

// y ← L⁻¹y then y ← L⁻ᵀy (FP64 vector in shared memory, FP32 factor), one CTA.
__device__ void chol_apply(const float* __restrict__ L, int s, int64_t lda, double* y)
{
  // forward: the thread that owns no row waits; columns processed in order
  for (int j = 0; j < s; ++j) {
    if (threadIdx.x == 0) y[j] /= (double)L[(int64_t)j * lda + j];
    __syncthreads();
    const double yj = y[j];
    for (int i = j + 1 + threadIdx.x; i < s; i += blockDim.x) y[i] -= (double)L[(int64_t)j * lda + i] * yj;
    __syncthreads();
  }
  // backward: y_j = (y_j − Σ_{i>j} L_ij y_i)/L_jj, dot products by block reduction
  __shared__ double red[32];
  for (int j = s - 1; j >= 0; --j) {
    double part = 0.0;
    for (int i = j + 1 + threadIdx.x; i < s; i += blockDim.x) part += (double)L[(int64_t)j * lda + i] * y[i];
    const double tot = block_sum_d(part, red);
    if (threadIdx.x == 0) y[j] = (y[j] - tot) / (double)L[(int64_t)j * lda + j];
    __syncthreads();
  }
}

// One CTA per system b: A_b = A + b·strideA + off[b] (s×s, ld lda, lower triangle used) plus
// diag(d_b) is copied to F_b, factored, and q_b = z_bᵀx (z_b = column s of A_b) with x refined
// twice against FP64 residuals of the original system.
__global__ void __launch_bounds__(kCholThreads)
spd_quadform_kernel(const float* __restrict__ A, int64_t lda, int64_t strideA, const int64_t* __restrict__ off,
                    const float* __restrict__ d, int s, float* __restrict__ F, double* __restrict__ q,
                    int* __restrict__ status)
{
  extern __shared__ double sm[];   // x (s), r (s)
  __shared__ float S[kCholB][kCholB + 1];
  __shared__ int bad;
  __shared__ double red[32];
  const int b = blockIdx.x;
  const float* Ab = A + (int64_t)b * strideA + off[b];
  const float* db = d + (int64_t)b * s;
  const float* zb = Ab + (int64_t)s * lda;
  float* Fb = F + (int64_t)b * s * s;
  double* x = sm;
  double* r = sm + s;
  if (threadIdx.x == 0) bad = 0;
  for (int64_t q2 = threadIdx.x; q2 < (int64_t)s * s; q2 += blockDim.x) {
    const int i = (int)(q2 % s), j = (int)(q2 / s);
    if (i >= j) Fb[(int64_t)j * s + i] = Ab[(int64_t)j * lda + i] + (i == j ? db[i] : 0.f);
  }
  __syncthreads();
  const bool ok = chol_blocked(Fb, s, s, S, &bad);
  if (!ok) {
    if (threadIdx.x == 0) {
      q[b] = 0.0;
      atomicOr(status, 1);
    }
    return;
  }
  for (int i = threadIdx.x; i < s; i += blockDim.x) x[i] = (double)zb[i];
  __syncthreads();
  chol_apply(Fb, s, s, x);
  for (int it = 0; it < 2; ++it) {
    // r = z − (A + D)x in FP64, symmetric A from its lower triangle
    for (int i = threadIdx.x; i < s; i += blockDim.x) {
      double acc = (double)zb[i] - (double)db[i] * x[i];
      for (int j = 0; j < s; ++j) {
        const float a = (i >= j) ? Ab[(int64_t)j * lda + i] : Ab[(int64_t)i * lda + j];
        acc -= (double)a * x[j];
      }
      r[i] = acc;
    }
    __syncthreads();
    chol_apply(Fb, s, s, r);
    for (int i = threadIdx.x; i < s; i += blockDim.x) x[i] += r[i];
    __syncthreads();
  }
  double part = 0.0;
  for (int i = threadIdx.x; i < s; i += blockDim.x) part += (double)zb[i] * x[i];
  const double tot = block_sum_d(part, red);
  if (threadIdx.x == 0) q[b] = tot;
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_lmm_quadforms(slemm_geno* g, const float* Py, float tau1, float tol_L, int num_qf,
                                       int window_size, int64_t* variants, float* xPy, float* xPx, float* xBx,
                                       float* xSx, int* count)
{
  return guarded([&] {
    CHECK_ARG(g && Py && variants && xPy && xPx && xBx && xSx && count, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_lmm_quadforms reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    CHECK_ARG(g->weights_set, "set_weights must be called first");
    CHECK_ARG(num_qf >= 1 && num_qf <= 300, "num_qf_markers out of [1, 300]");
    CHECK_ARG(tau1 > 0.f && std::isfinite(tau1), "tau1 must be positive");
    const int64_t n = g->n, m = g->m;
    CHECK_ARG(window_size >= 2 && window_size % 2 == 0 && window_size <= 5000 && window_size <= m,
              "window_size must be even, in [2, 5000] and <= m");
    cudaStream_t st = g->stream;
    std::vector<float> gm(m), gw(m);
    CUDA_TRY(cudaMemcpyAsync(gm.data(), g->gm.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(gw.data(), g->w.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const std::vector<int64_t> var = lmm_variants(gm, n, num_qf);
    const int k = (int)var.size();
    *count = k;
    if (k == 0) return;
    std::copy(var.begin(), var.end(), variants);
    const int64_t K_tiles = g->n_pad / kTileK;
    // centred counts of the sampled markers, x'Py, then v = P(rr∘x)
    DevBuf d_rows(st), d_V(st), d_X(st), d_py(st), d_sc(st);
    d_rows.ensure(k * sizeof(int64_t));
    CUDA_TRY(cudaMemcpyAsync(d_rows.p, var.data(), k * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    float* V = (float*)d_V.ensure((size_t)n * k * sizeof(float));
    float* X = (float*)d_X.ensure((size_t)n * k * sizeof(float));
    float* py = (float*)d_py.ensure(n * sizeof(float));
    double* sc = (double*)d_sc.ensure((size_t)4 * k * sizeof(double));
    DevBuf d_qt(st);
    double* qtv = (double*)d_qt.ensure((size_t)g->c * std::max(k, window_size + 1) * sizeof(double));
    CUDA_TRY(cudaMemcpyAsync(py, Py, n * sizeof(float), cudaMemcpyHostToDevice, st));
    centred_rows_kernel<<<dim3((unsigned)ceil_div(n, 256), k), 256, 0, st>>>(
        g->G.as<uint32_t>(), K_tiles, d_rows.as<int64_t>(), 0, g->gm.as<float>(), nullptr, n, V, n);
    LAUNCH_CHECK();
    col_dots(g, V, n, py, 0, n, k, sc);   // every column against Py
    scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), k), 256, 0, st>>>(V, n, g->rr.as<float>(), n);
    LAUNCH_CHECK();
    proj_coeffs(g, V, n, k, qtv);
    proj_apply(g, V, n, k, qtv);
    // x'Px through one projected Lanczos seed and a solve at shift 0; x'Sx = ‖v‖²
    slemm_lseed* S = lanczos_seed_device(g, SLEMM_OP_QUADFORM, tau1, V, k, tol_L, 600, false, {}, 5, 0);
    std::unique_ptr<slemm_lseed, void (*)(slemm_lseed*)> hold(S, lseed_free);
    lanczos_solve_device(S, 0.0, 1e-6, X, n, 0);
    col_dots(g, V, n, X, n, n, k, sc + k);
    col_dots(g, V, n, nullptr, 0, n, k, sc + 2 * k);
    // windows: [ZᵀZ | Zᵀv] from the packed copy, one product per marker
    const int ws = window_size;
    DevBuf d_U(st), d_gram(st), d_F(st), d_d(st), d_q(st), d_status(st);
    float* U = (float*)d_U.ensure((size_t)n * (ws + 1) * sizeof(float));
    const int64_t rows_max = round_up(ws, kPadRows) + kPadRows;
    float* gram = (float*)d_gram.ensure((size_t)k * rows_max * (ws + 1) * sizeof(float));
    std::vector<int64_t> wstart(k);
    std::vector<float> dd((size_t)k * ws);
    for (int c = 0; c < k; ++c) {
      const int64_t j = var[c];
      int64_t wds;
      if (j < ws / 2) wds = 0;
      else if (j > m - ws / 2) wds = m - ws;
      else wds = j - ws / 2;
      wstart[c] = wds;
      for (int t = 0; t < ws; ++t) dd[(size_t)c * ws + t] = tau1 / gw[wds + t];
      // U = rr∘P(rr∘Cc) for the window's markers, then column ws = rr∘v
      centred_rows_kernel<<<dim3((unsigned)ceil_div(n, 256), ws), 256, 0, st>>>(
          g->G.as<uint32_t>(), K_tiles, nullptr, wds, g->gm.as<float>(), g->rr.as<float>(), n, U, n);
      LAUNCH_CHECK();
      proj_coeffs(g, U, n, ws, qtv);
      proj_apply(g, U, n, ws, qtv);
      CUDA_TRY(cudaMemcpyAsync(U + (size_t)ws * n, V + (size_t)c * n, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
      scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), ws + 1), 256, 0, st>>>(U, n, g->rr.as<float>(), n);
      LAUNCH_CHECK();
      const int64_t r0 = wds / kPadRows * kPadRows;
      const int64_t r1 = std::min<int64_t>(round_up(wds + ws, kPadRows), g->m_pad);
      rows_product(g, r0, r1 - r0, U, n, ws + 1, gram + (size_t)c * rows_max * (ws + 1), rows_max, SLEMM_PREC_FP16X2);
      // this window's Gram starts at row wds − r0 of its block
      wstart[c] = wds - r0;
    }
    check_device_error(g);
    // batched solves: q_c = zᵀ(ZᵀZ + D)⁻¹z
    float* F = (float*)d_F.ensure((size_t)k * ws * ws * sizeof(float));
    float* dvec = (float*)d_d.ensure((size_t)k * ws * sizeof(float));
    double* q = (double*)d_q.ensure(k * sizeof(double));
    int* status = (int*)d_status.ensure(sizeof(int));
    CUDA_TRY(cudaMemcpyAsync(dvec, dd.data(), dd.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    const size_t smem = (size_t)2 * ws * sizeof(double);
    CUDA_TRY(cudaFuncSetAttribute(spd_quadform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DevBuf d_off(st);
    CUDA_TRY(cudaMemcpyAsync(d_off.ensure(k * sizeof(int64_t)), wstart.data(), k * sizeof(int64_t),
                             cudaMemcpyHostToDevice, st));
    spd_quadform_kernel<<<k, kCholThreads, smem, st>>>(gram, rows_max, rows_max * (ws + 1), d_off.as<int64_t>(), dvec,
                                                       ws, F, q, status);
    LAUNCH_CHECK();
    std::vector<double> h(3 * k), hq(k);
    int hs = 0;
    CUDA_TRY(cudaMemcpyAsync(h.data(), sc, 3 * k * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(hq.data(), q, k * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (hs) SLEMM_THROW(SLEMM_ERR_NUMERIC, "a window's ZᵀZ + τ1·diag(1/gw) is not positive definite in FP32");
    for (int c = 0; c < k; ++c) {
      xPy[c] = (float)h[c];
      xPx[c] = (float)h[k + c];
      xSx[c] = (float)h[2 * k + c];
      xBx[c] = (float)((h[2 * k + c] - hq[c]) / (double)tau1);
    }
  });
}
