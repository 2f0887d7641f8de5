// dense.cuh — small dense helpers of the GWAS drivers (lmm.cu, gwa.cu): centred count rows decoded
// from the packed copy, row scaling, and a one-CTA blocked Cholesky factorisation.  Everything has
// internal linkage (each including translation unit gets its own copy).
#pragma once

#include "common.h"

namespace slemm {
namespace {

// out[c·ld + i] = (count(row rows[c], i) − gm[rows[c]])·(rr ? rr[i] : 1) for i < n (FP32).
__global__ void centred_rows_kernel(const uint32_t* __restrict__ G, int64_t K_tiles, const int64_t* __restrict__ rows,
                                    int64_t row0, const float* __restrict__ gm, const float* __restrict__ rr, int64_t n,
                                    float* __restrict__ out, int64_t ld)
{
  const int c = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t j = rows ? rows[c] : row0 + c;
  const int64_t mt = j / 128, r = j % 128, kt = i / 64, e = i % 64;
  const uint32_t w = G[((mt * K_tiles + kt) * 128 + r) * 4 + e / 16];
  const int q = (int)(e % 16);
  const int sh = (q & 1) ? 16 + (q & ~1) : q;
  float x = (float)((w >> sh) & 3u) - gm[j];
  if (rr) x *= rr[i];
  out[(int64_t)c * ld + i] = x;
}

// X[i, c] *= rr[i]
__global__ void scale_rows_rr_kernel(float* __restrict__ X, int64_t ld, const float* __restrict__ rr, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) X[(int64_t)blockIdx.y * ld + i] *= rr[i];
}

// ---- batched SPD solve: q_b = z_bᵀ(A_b + diag(d_b))⁻¹z_b ----------------------------------------
constexpr int kCholB = 32;
constexpr int kCholThreads = 512;

// In place: the lower triangle of A (s×s, column-major, lda) becomes its Cholesky factor L.
// Returns false (in every thread) if a pivot is not positive.
__device__ bool chol_blocked(float* __restrict__ A, int s, int64_t lda, float (*S)[kCholB + 1], int* bad)
{
  const int tid = threadIdx.x;
  for (int kb = 0; kb < s; kb += kCholB) {
    const int nb = min(kCholB, s - kb);
    // 1. diagonal block in shared memory, unblocked
    for (int q = tid; q < nb * nb; q += blockDim.x) {
      const int i = q % nb, j = q / nb;
      S[i][j] = A[(int64_t)(kb + j) * lda + kb + i];
    }
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
      if (tid == 0) {
        const float d = S[j][j];
        if (!(d > 0.f)) *bad = 1;
        S[j][j] = sqrtf(fmaxf(d, 1e-30f));
      }
      __syncthreads();
      const float djj = S[j][j];
      for (int i = j + 1 + tid; i < nb; i += blockDim.x) S[i][j] /= djj;
      __syncthreads();
      for (int q = tid; q < nb * nb; q += blockDim.x) {
        const int i = q % nb, k = q / nb;
        if (k > j && i >= k) S[i][k] -= S[i][j] * S[k][j];
      }
      __syncthreads();
    }
    for (int q = tid; q < nb * nb; q += blockDim.x) {
      const int i = q % nb, j = q / nb;
      if (i >= j) A[(int64_t)(kb + j) * lda + kb + i] = S[i][j];
    }
    // 2. panel rows below: x·L11ᵀ = a, one thread per row
    for (int i = kb + nb + tid; i < s; i += blockDim.x) {
      float x[kCholB];
#pragma unroll
      for (int j = 0; j < kCholB; ++j) {
        if (j < nb) {
          float a = A[(int64_t)(kb + j) * lda + i];
          for (int t = 0; t < j; ++t) a -= x[t] * S[j][t];
          x[j] = a / S[j][j];
        }
      }
#pragma unroll
      for (int j = 0; j < kCholB; ++j)
        if (j < nb) A[(int64_t)(kb + j) * lda + i] = x[j];
    }
    __syncthreads();
    // 3. trailing lower triangle: A[i][j] −= Σ_t P[i][t]·P[j][t], 4×4 tiles per thread
    const int r0 = kb + nb, t = s - r0;
    const int tiles = (t + 3) / 4;
    for (int q = tid; q < tiles * tiles; q += blockDim.x) {
      const int ti = q % tiles, tj = q / tiles;
      if (tj > ti) continue;
      const int i0 = r0 + 4 * ti, j0 = r0 + 4 * tj;
      float acc[4][4] = {};
      for (int u = 0; u < nb; ++u) {
        const float* col = A + (int64_t)(kb + u) * lda;
        float pi[4], pj[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          pi[a] = (i0 + a < s) ? col[i0 + a] : 0.f;
          pj[a] = (j0 + a < s) ? col[j0 + a] : 0.f;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] += pi[a] * pj[b];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int i = i0 + a, j = j0 + b;
          if (i < s && j < s && i >= j) A[(int64_t)j * lda + i] -= acc[a][b];
        }
    }
    __syncthreads();
  }
  __syncthreads();
  return *bad == 0;
}

}  // namespace
}  // namespace slemm
