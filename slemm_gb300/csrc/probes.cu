// probes.cu — the reference's Rademacher probe block generated on the GPU, draw for draw.
//
// The reference fills V (n×n_V, column by column) with std::mt19937(seed + 54321) and
// uniform_real_distribution<float>(0, 1) < 0.5 → −1, then divides each column by its norm
// (src/reml.cpp:597-605).  With a 32-bit engine, generate_canonical<float> returns
// float(x)/2^32 for the engine output x (rounded to nearest), so a draw is −1 exactly when
// float(x) < 2^31.  The column norm is √n (Σ(±1)² is exact), so every entry is ±1/√n in FP32.
//
// MT19937 (Matsumoto & Nishimura, 1998): 624-word state, initialised by
// s[i] = 1812433253·(s[i−1] ⊕ (s[i−1] ≫ 30)) + i, regenerated 624 words at a time by the twist
// s'[k] = s[k+397] ⊕ (y ≫ 1) ⊕ (y odd ? 0x9908B0DF : 0), y = upper bit of s[k] | lower 31 bits
// of s[k+1] (indices mod 624, using already-regenerated words for k+397 ≥ 624 and for the last
// word's successor), and tempered on output.  The twist's dependencies split into four phases
// that run in parallel inside one CTA: k < 227 (old words only), 227 ≤ k < 454 (needs phase 1),
// 454 ≤ k < 623 (needs phase 2), k = 623 (needs s'[0] and s'[396]).
#include "internal.h"

namespace slemm {

constexpr int kMtN = 624, kMtM = 397;

__device__ __forceinline__ uint32_t mt_twist(uint32_t cur, uint32_t next, uint32_t far)
{
  const uint32_t y = (cur & 0x80000000u) | (next & 0x7fffffffu);
  return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y)
{
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// V[c*ld + i] = ±inv_norm for draw index c·n + i, all n·n_V draws (one CTA of 640 threads).
__global__ void __launch_bounds__(640, 1)
mt_rademacher_kernel(uint32_t seed, int64_t n, int n_V, float* __restrict__ V, int64_t ld, float value)
{
  __shared__ uint32_t s[kMtN];
  const int k = threadIdx.x;
  if (k == 0) {
    s[0] = seed;
    for (int i = 1; i < kMtN; ++i) s[i] = 1812433253u * (s[i - 1] ^ (s[i - 1] >> 30)) + (uint32_t)i;
  }
  __syncthreads();
  const int64_t total = n * (int64_t)n_V;
  for (int64_t base = 0; base < total; base += kMtN) {
    uint32_t nv = 0;
    if (k < kMtN - kMtM) nv = mt_twist(s[k], s[k + 1], s[k + kMtM]);                 // phase 1
    __syncthreads();
    if (k < kMtN - kMtM) s[k] = nv;
    __syncthreads();
    if (k >= kMtN - kMtM && k < 2 * (kMtN - kMtM)) nv = mt_twist(s[k], s[k + 1], s[k - (kMtN - kMtM)]);  // phase 2
    __syncthreads();
    if (k >= kMtN - kMtM && k < 2 * (kMtN - kMtM)) s[k] = nv;
    __syncthreads();
    if (k >= 2 * (kMtN - kMtM) && k < kMtN - 1) nv = mt_twist(s[k], s[k + 1], s[k - (kMtN - kMtM)]);  // phase 3
    __syncthreads();
    if (k >= 2 * (kMtN - kMtM) && k < kMtN - 1) s[k] = nv;
    __syncthreads();
    if (k == kMtN - 1) s[k] = mt_twist(s[kMtN - 1], s[0], s[kMtM - 1]);               // phase 4
    __syncthreads();
    if (k < kMtN) {
      const int64_t idx = base + k;
      if (idx < total) {
        const uint32_t x = mt_temper(s[k]);
        const bool neg = __uint2float_rn(x) < 2147483648.0f;   // float(x)/2^32 < 0.5
        const int64_t c = idx / n, i = idx - c * n;
        V[c * ld + i] = neg ? -value : value;
      }
    }
    __syncthreads();
  }
}

// Fills the device block V (n×n_V, ld) with the reference's normalised Rademacher probes.
void rademacher_device(int seed, int64_t n, int n_V, float* dV, int64_t ld, cudaStream_t st)
{
  const float value = 1.0f / std::sqrt((float)n);   // ±1 / ‖±1‖, both IEEE-rounded in FP32
  mt_rademacher_kernel<<<1, 640, 0, st>>>((uint32_t)(seed + 54321), n, n_V, dV, ld, value);
  LAUNCH_CHECK();
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_rademacher(int seed, int64_t n, int n_V, float* V, int64_t ldv, int mem)
{
  return guarded([&] {
    CHECK_ARG(V != nullptr && n >= 1 && n_V >= 1 && ldv >= n, "bad argument");
    if (mem == SLEMM_MEM_DEVICE) {
      rademacher_device(seed, n, n_V, V, ldv, nullptr);
      CUDA_TRY(cudaStreamSynchronize(nullptr));
      return;
    }
    DevBuf d;
    d.ensure((size_t)n * n_V * sizeof(float));
    rademacher_device(seed, n, n_V, d.as<float>(), n, nullptr);
    CUDA_TRY(cudaMemcpy2D(V, ldv * sizeof(float), d.p, n * sizeof(float), n * sizeof(float), n_V,
                          cudaMemcpyDeviceToHost));
  });
}
