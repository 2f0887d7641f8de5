// wls.cu — SNP effects by weighted least squares (`--wls`, src/wls.cpp:4-129).
//
// With Z̃ = (I − QQᵀ)(rr∘(Cnt − 1·gmᵀ)) (gm = popcount/n, Q an orthonormal basis of rr∘X):
//   b = (Z̃ᵀZ̃ + 1e-4·mean(diag Z̃ᵀZ̃)·I)⁻¹ Z̃ᵀ y_proj,   y_proj = (I − QQᵀ)(rr∘y),
// solved by Cholesky in FP32 like the reference's LLT on its FP32 blocks.
//
// GB300 mapping.  Z̃ᵀZ̃ = Cc ᵀ·U with U = rr∘(I − QQᵀ)(rr∘Cc) (P is a symmetric projection), so the
// Gram comes, 1024 columns at a time, out of the packed tensor-core product over the SNP rows at or
// below the block (the lower part is all the factorisation reads) with column-scaled FP16 hi+lo
// (≈ FP32, like the reference's SGEMM), and Z̃ᵀy_proj = Ccᵀ(rr∘y_proj) likewise.  The m×m system
// is factored in place by a tiled right-looking Cholesky (128×128 tiles): one CTA factors the
// diagonal tile, one CTA per tile below solves the panel, and a shared-memory tiled FP32
// SYRK/GEMM updates the trailing lower triangle; the triangular solves are blocked the same way.
#include "internal.h"
#include "reduce.cuh"
#include "dense.cuh"

#include <cmath>

namespace slemm {

constexpr int kT = 128;   // Cholesky tile

// One CTA: the tk×tk diagonal tile at (k0, k0) of A (ld lda) becomes its Cholesky factor.
__global__ void __launch_bounds__(kCholThreads)
potrf_tile_kernel(float* __restrict__ A, int64_t lda, int64_t k0, int tk, int* __restrict__ status)
{
  __shared__ float S[kCholB][kCholB + 1];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  if (!chol_blocked(A + k0 * lda + k0, tk, lda, S, &bad) && threadIdx.x == 0) atomicOr(status, 1);
}

// Panel: for the row tile starting at r = k0 + tk + 128·blockIdx.x, X·L_kkᵀ = A[r…, k0…k0+tk) in
// place; one thread per row, L_kk and the rows in shared memory.
__global__ void __launch_bounds__(kT)
trsm_panel_kernel(float* __restrict__ A, int64_t lda, int64_t m, int64_t k0, int tk)
{
  extern __shared__ float sm[];
  float* L = sm;                          // tk × tk, row-major L[j*kT + t]
  float* X = sm + kT * kT;                // 128 rows × (kT+1)
  const int64_t r0 = k0 + tk + (int64_t)kT * blockIdx.x;
  for (int q = threadIdx.x; q < tk * tk; q += blockDim.x) {
    const int j = q / tk, t = q % tk;
    L[j * kT + t] = (t <= j) ? A[(k0 + t) * lda + k0 + j] : 0.f;
  }
  const int rows = (int)min64(kT, m - r0);
  for (int q = threadIdx.x; q < rows * tk; q += blockDim.x) {
    const int i = q % rows, t = q / rows;
    X[i * (kT + 1) + t] = A[(k0 + t) * lda + r0 + i];
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (i < rows) {
    float* x = X + i * (kT + 1);
    for (int j = 0; j < tk; ++j) {
      float a = x[j];
      for (int t = 0; t < j; ++t) a -= x[t] * L[j * kT + t];
      x[j] = a / L[j * kT + j];
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < rows * tk; q += blockDim.x) {
    const int ii = q % rows, t = q / rows;
    A[(k0 + t) * lda + r0 + ii] = X[ii * (kT + 1) + t];
  }
}

// Trailing update: lower tile pair (ti ≥ tj) of the rows/columns after c0 = k0 + tk:
// A[I, J] −= P_I·P_Jᵀ with P = A[·, k0 … k0+tk).  128×128 output tile, 8×8 per thread.
__global__ void __launch_bounds__(256)
syrk_update_kernel(float* __restrict__ A, int64_t lda, int64_t m, int64_t k0, int tk)
{
  __shared__ float Pa[16][kT + 4];
  __shared__ float Pb[16][kT + 4];
  // triangular index → (ti, tj), tj ≤ ti
  const int64_t q = blockIdx.x;
  int64_t ti = (int64_t)((std::sqrt(8.0 * (double)q + 1.0) - 1.0) / 2.0);
  while ((ti + 1) * (ti + 2) / 2 <= q) ++ti;
  while (ti * (ti + 1) / 2 > q) --ti;
  const int64_t tj = q - ti * (ti + 1) / 2;
  const int64_t c0 = k0 + tk;
  const int64_t I0 = c0 + ti * kT, J0 = c0 + tj * kT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[8][8] = {};
  for (int u0 = 0; u0 < tk; u0 += 16) {
    for (int e = threadIdx.x; e < 16 * kT; e += 256) {
      const int uu = e / kT, r = e % kT;
      const int64_t col = k0 + u0 + uu;
      const bool cu = (u0 + uu) < tk;
      Pa[uu][r] = (cu && I0 + r < m) ? A[col * lda + I0 + r] : 0.f;
      Pb[uu][r] = (cu && J0 + r < m) ? A[col * lda + J0 + r] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int uu = 0; uu < 16; ++uu) {
      float a[8], b[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        a[v] = Pa[uu][ty + 16 * v];
        b[v] = Pb[uu][tx + 16 * v];
      }
#pragma unroll
      for (int v = 0; v < 8; ++v)
#pragma unroll
        for (int w = 0; w < 8; ++w) acc[v][w] = fmaf(a[v], b[w], acc[v][w]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int v = 0; v < 8; ++v)
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      const int64_t i = I0 + ty + 16 * v, j = J0 + tx + 16 * w;
      if (i < m && j < m && i >= j) A[j * lda + i] -= acc[v][w];
    }
}

// Forward step on tile k: y_k ← L_kk⁻¹ y_k (one warp), then y_i −= L_ik·y_k for every row below.
__global__ void trsv_fwd_diag_kernel(const float* __restrict__ A, int64_t lda, int64_t k0, int tk, double* __restrict__ y)
{
  const int lane = threadIdx.x;
  for (int i = 0; i < tk; ++i) {
    double s = 0.0;
    for (int t = lane; t < i; t += 32) s += (double)A[(k0 + t) * lda + k0 + i] * y[k0 + t];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) y[k0 + i] = (y[k0 + i] - s) / (double)A[(k0 + i) * lda + k0 + i];
    __syncwarp();
  }
}
__global__ void trsv_fwd_update_kernel(const float* __restrict__ A, int64_t lda, int64_t m, int64_t k0, int tk,
                                       double* __restrict__ y)
{
  const int64_t i = k0 + tk + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int t = 0; t < tk; ++t) s += (double)A[(k0 + t) * lda + i] * y[k0 + t];
  y[i] -= s;
}
// Backward step on tile k: x_k ← L_kk⁻ᵀ x_k (one warp), then x_j −= L_kjᵀ·x_k for every j < k0.
__global__ void trsv_bwd_diag_kernel(const float* __restrict__ A, int64_t lda, int64_t k0, int tk, double* __restrict__ x)
{
  const int lane = threadIdx.x;
  for (int i = tk - 1; i >= 0; --i) {
    double s = 0.0;
    for (int t = i + 1 + lane; t < tk; t += 32) s += (double)A[(k0 + i) * lda + k0 + t] * x[k0 + t];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[k0 + i] = (x[k0 + i] - s) / (double)A[(k0 + i) * lda + k0 + i];
    __syncwarp();
  }
}
__global__ void trsv_bwd_update_kernel(const float* __restrict__ A, int64_t lda, int64_t k0, int tk, double* __restrict__ x)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k0) return;
  double s = 0.0;
  for (int t = 0; t < tk; ++t) s += (double)A[j * lda + k0 + t] * x[k0 + t];
  x[j] -= s;
}

__global__ void diag_kernel(const float* __restrict__ A, int64_t lda, int64_t m, float* __restrict__ d)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) d[i] = A[i * lda + i];
}
__global__ void add_diag_kernel(float* __restrict__ A, int64_t lda, int64_t m, float v)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) A[i * lda + i] += v;
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_wls(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c, const float* y,
                             float* snp_blup)
{
  return guarded([&] {
    CHECK_ARG(g && X && y && snp_blup, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_wls reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    const int64_t n = g->n, m = g->m;
    CHECK_ARG(c >= 1 && c <= SLEMM_MAX_COVARIATES && ldx >= n, "bad covariate matrix");
    cudaStream_t st = g->stream;
    // rr, Q, y_proj on the host (FP64 QR); gm from the exact popcounts
    std::vector<float> rr(n);
    for (int64_t i = 0; i < n; ++i) {
      const float r = rvec ? rvec[i] : 1.0f;
      CHECK_ARG(r > 0.f && std::isfinite(r), "error variance weight must be > 0");
      rr[i] = 1.0f / std::sqrt(r);
    }
    std::vector<double> A((size_t)n * c), Qd;
    for (int j = 0; j < c; ++j)
      for (int64_t i = 0; i < n; ++i) A[(size_t)j * n + i] = (double)(X[(size_t)j * ldx + i] * rr[i]);
    CHECK_ARG(orthonormal_columns(A, n, c, Qd) == c, "Fixed-effects design matrix is not of full rank.");
    std::vector<float> yp(n);
    {
      std::vector<double> v(n);
      for (int64_t i = 0; i < n; ++i) v[i] = (double)(rr[i] * y[i]);
      for (int l = 0; l < c; ++l) {
        const double* q = Qd.data() + (size_t)l * n;
        double s = 0.0;
        for (int64_t i = 0; i < n; ++i) s += q[i] * v[i];
        for (int64_t i = 0; i < n; ++i) v[i] -= s * q[i];
      }
      for (int64_t i = 0; i < n; ++i) yp[i] = (float)(rr[i] * (float)v[i]);   // rr∘y_proj
    }
    std::vector<int64_t> pc(m);
    int stc = slemm_gpu_genotype_counts(g, pc.data(), nullptr, nullptr, nullptr);
    if (stc != SLEMM_OK) SLEMM_THROW(stc, "genotype counts failed");
    std::vector<float> gm(m), ones(m, 1.0f), Qf((size_t)n * c);
    for (int64_t j = 0; j < m; ++j) gm[j] = (int)pc[j] / (float)n;
    for (size_t i = 0; i < Qf.size(); ++i) Qf[i] = (float)Qd[i];
    stc = slemm_gpu_set_weights(g, gm.data(), ones.data(), rr.data());
    if (stc != SLEMM_OK) SLEMM_THROW(stc, "set_weights failed");
    stc = slemm_gpu_set_projection(g, Qf.data(), n, c);
    if (stc != SLEMM_OK) SLEMM_THROW(stc, "set_projection failed");
    // Z̃ᵀZ̃ (lower part) and Z̃ᵀy_proj
    const int64_t lda = m;
    DevBuf d_A(st), d_U(st), d_qt(st), d_y(st), d_b(st), d_d(st), d_st(st), d_x(st);
    float* Am = (float*)d_A.ensure((size_t)lda * m * sizeof(float));
    const int kc = 1024;
    float* U = (float*)d_U.ensure((size_t)n * kc * sizeof(float));
    double* qt = (double*)d_qt.ensure((size_t)c * kc * sizeof(double));
    const int64_t K_tiles = g->n_pad / kTileK;
    for (int64_t j0 = 0; j0 < m; j0 += kc) {
      const int k = (int)std::min<int64_t>(kc, m - j0);
      centred_rows_kernel<<<dim3((unsigned)ceil_div(n, 256), k), 256, 0, st>>>(
          g->G.as<uint32_t>(), K_tiles, nullptr, j0, g->gm.as<float>(), g->rr.as<float>(), n, U, n);
      LAUNCH_CHECK();
      proj_coeffs(g, U, n, k, qt);
      proj_apply(g, U, n, k, qt);
      scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), k), 256, 0, st>>>(U, n, g->rr.as<float>(), n);
      LAUNCH_CHECK();
      const int64_t r0 = j0 / kPadRows * kPadRows;
      rows_product(g, r0, g->m_pad - r0, U, n, k, Am + j0 * lda + r0, lda, SLEMM_PREC_FP16X2);
    }
    float* dy = (float*)d_y.ensure(n * sizeof(float));
    float* b = (float*)d_b.ensure(g->m_pad * sizeof(float));
    CUDA_TRY(cudaMemcpyAsync(dy, yp.data(), n * sizeof(float), cudaMemcpyHostToDevice, st));
    rows_product(g, 0, g->m_pad, dy, n, 1, b, g->m_pad, SLEMM_PREC_FP16X2);
    check_device_error(g);
    // ridge: 1e-4·mean(diag) (src/wls.cpp:123)
    float* dd = (float*)d_d.ensure(m * sizeof(float));
    diag_kernel<<<(unsigned)ceil_div(m, 256), 256, 0, st>>>(Am, lda, m, dd);
    LAUNCH_CHECK();
    std::vector<float> hd(m);
    CUDA_TRY(cudaMemcpyAsync(hd.data(), dd, m * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    double ds = 0.0;
    for (float v : hd) ds += v;
    const float ridge = 1e-4f * (float)(ds / (double)m);
    add_diag_kernel<<<(unsigned)ceil_div(m, 256), 256, 0, st>>>(Am, lda, m, ridge);
    LAUNCH_CHECK();
    // tiled Cholesky
    int* status = (int*)d_st.ensure(sizeof(int));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    const size_t smem_trsm = (size_t)(kT * kT + kT * (kT + 1)) * sizeof(float);
    CUDA_TRY(cudaFuncSetAttribute(trsm_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_trsm));
    for (int64_t k0 = 0; k0 < m; k0 += kT) {
      const int tk = (int)std::min<int64_t>(kT, m - k0);
      potrf_tile_kernel<<<1, kCholThreads, 0, st>>>(Am, lda, k0, tk, status);
      LAUNCH_CHECK();
      const int64_t rest = m - k0 - tk;
      if (rest <= 0) break;
      const int64_t nt = ceil_div(rest, kT);
      trsm_panel_kernel<<<(unsigned)nt, kT, smem_trsm, st>>>(Am, lda, m, k0, tk);
      LAUNCH_CHECK();
      syrk_update_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, st>>>(Am, lda, m, k0, tk);
      LAUNCH_CHECK();
    }
    // L Lᵀ x = b
    double* x = (double*)d_x.ensure(m * sizeof(double));
    {
      std::vector<float> hb(m);
      CUDA_TRY(cudaMemcpyAsync(hb.data(), b, m * sizeof(float), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      std::vector<double> hx(hb.begin(), hb.end());
      CUDA_TRY(cudaMemcpyAsync(x, hx.data(), m * sizeof(double), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    }
    for (int64_t k0 = 0; k0 < m; k0 += kT) {
      const int tk = (int)std::min<int64_t>(kT, m - k0);
      trsv_fwd_diag_kernel<<<1, 32, 0, st>>>(Am, lda, k0, tk, x);
      LAUNCH_CHECK();
      if (m - k0 - tk > 0) {
        trsv_fwd_update_kernel<<<(unsigned)ceil_div(m - k0 - tk, 256), 256, 0, st>>>(Am, lda, m, k0, tk, x);
        LAUNCH_CHECK();
      }
    }
    for (int64_t k0 = (m - 1) / kT * kT; k0 >= 0; k0 -= kT) {
      const int tk = (int)std::min<int64_t>(kT, m - k0);
      trsv_bwd_diag_kernel<<<1, 32, 0, st>>>(Am, lda, k0, tk, x);
      LAUNCH_CHECK();
      if (k0 > 0) {
        trsv_bwd_update_kernel<<<(unsigned)ceil_div(k0, 256), 256, 0, st>>>(Am, lda, k0, tk, x);
        LAUNCH_CHECK();
      }
    }
    std::vector<double> hx(m);
    int hs = 0;
    CUDA_TRY(cudaMemcpyAsync(hx.data(), x, m * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (hs) SLEMM_THROW(SLEMM_ERR_NUMERIC, "Z̃ᵀZ̃ + ridge is not positive definite in FP32");
    for (int64_t j = 0; j < m; ++j) snp_blup[j] = (float)hx[j];
  });
}
