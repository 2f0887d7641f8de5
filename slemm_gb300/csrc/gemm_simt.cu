// gemm_simt.cu — FP32 CUDA-core packed product (the plain FP32 path).
//
// D[s][c][r] = Σ_{K in split s} count[r,K] · B[c][K] for a 128-row tile per CTA: thread t owns
// row t, reads its 16 packed bytes of each tile (the CTA's 128 threads read one contiguous
// 2048-byte tile), decodes exact integer counts to FP32 and multiplies and adds in FP32 like the
// reference's SGEMM (src/reml.cpp:36, 144, 182, 220), one K-tile at a time, folding each tile's
// sum into a double-float accumulator.  B columns are staged in shared memory for kStageTiles
// tiles at a time and read as broadcasts.
#include "common.h"
#include "decode.cuh"
#include "reduce.cuh"

namespace slemm {

constexpr int kStageTiles = 8;                 // 512 K elements per shared-memory stage
constexpr int kStageK = kStageTiles * kTileK;

template <int KC>
__global__ void __launch_bounds__(128)
gemm_simt_kernel(const uint4* __restrict__ A, int64_t M_pad, int64_t K_tiles,
                 const float* __restrict__ B, int64_t K_pad, int c0, int k_total,
                 float* __restrict__ D, int N, int tiles_per_split)
{
  __shared__ __align__(16) float sB[kStageK][KC];
  const int t = threadIdx.x;
  const int64_t mt = blockIdx.x;
  const int s = blockIdx.y;
  const int64_t kt0 = (int64_t)s * tiles_per_split;
  const int64_t kt1 = min64(K_tiles, kt0 + tiles_per_split);
  // Each K-tile's 64 products are summed in FP32 and folded into a double-float sum per column:
  // one FP32 chain over a whole split (10^5 elements at 500,000 individuals) loses ~1e-5 of the
  // result to rounding, 64-element chains ~3e-7.
  DF acc[KC];

  for (int64_t ks = kt0; ks < kt1; ks += kStageTiles) {
    const int ntile = (int)min64(kStageTiles, kt1 - ks);
    // stage B[c0 .. c0+KC)[ks*64 .. +ntile*64)
    __syncthreads();
    for (int idx = t; idx < ntile * kTileK * KC; idx += 128) {
      const int c = idx / (ntile * kTileK);
      const int kk = idx % (ntile * kTileK);
      const int col = c0 + c;
      sB[kk][c] = (col < k_total) ? B[(int64_t)col * K_pad + ks * kTileK + kk] : 0.f;
    }
    __syncthreads();
    uint4 pk[kStageTiles];
#pragma unroll
    for (int u = 0; u < kStageTiles; ++u)
      if (u < ntile) pk[u] = A[((mt * K_tiles + ks + u) * 128 + t)];
#pragma unroll
    for (int u = 0; u < kStageTiles; ++u) {
      if (u >= ntile) break;
      const uint32_t words[4] = {pk[u].x, pk[u].y, pk[u].z, pk[u].w};
      float part[KC];
#pragma unroll
      for (int c = 0; c < KC; ++c) part[c] = 0.f;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float xe, xo;
          f32pair_of(words[w], q, xe, xo);
          const int kk = u * kTileK + w * 16 + 2 * q;
#pragma unroll
          for (int c = 0; c < KC; ++c) part[c] = fmaf(xe, sB[kk][c], fmaf(xo, sB[kk + 1][c], part[c]));
        }
      }
#pragma unroll
      for (int c = 0; c < KC; ++c) df_add(acc[c], part[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < KC; ++c) {
    const int col = c0 + c;
    if (col < k_total) D[((int64_t)s * N + col) * M_pad + mt * 128 + t] = __fadd_rn(acc[c].hi, acc[c].lo);
  }
}

void gemm_simt(const GemmArgs& a, cudaStream_t st)
{
  const int64_t M_tiles = a.M_pad / kTileM, K_tiles = a.K_pad / kTileK;
  const int tps = (int)ceil_div(K_tiles, a.splits);
  dim3 grid((unsigned)M_tiles, (unsigned)a.splits);
  const float* B = static_cast<const float*>(a.B);
  int c0 = 0;
  while (c0 < a.N) {
    const int rem = a.N - c0;
    if (rem >= 8) {
      gemm_simt_kernel<8><<<grid, 128, 0, st>>>((const uint4*)a.A, a.M_pad, K_tiles, B, a.K_pad, c0,
                                                a.N, a.D, a.N, tps);
      c0 += 8;
    } else if (rem >= 4) {
      gemm_simt_kernel<4><<<grid, 128, 0, st>>>((const uint4*)a.A, a.M_pad, K_tiles, B, a.K_pad, c0,
                                                a.N, a.D, a.N, tps);
      c0 += 4;
    } else if (rem >= 2) {
      gemm_simt_kernel<2><<<grid, 128, 0, st>>>((const uint4*)a.A, a.M_pad, K_tiles, B, a.K_pad, c0,
                                                a.N, a.D, a.N, tps);
      c0 += 2;
    } else {
      gemm_simt_kernel<1><<<grid, 128, 0, st>>>((const uint4*)a.A, a.M_pad, K_tiles, B, a.K_pad, c0,
                                                a.N, a.D, a.N, tps);
      c0 += 1;
    }
    LAUNCH_CHECK();
  }
}

}  // namespace slemm
