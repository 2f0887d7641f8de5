// reduce.cuh — accumulation helpers of the row-wise kernels.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the row-wise kernels keep every
// per-element operation in FP32 and carry their sums as unevaluated double-float pairs
// (hi + lo): TwoProd through an FMA gives the exact product error and TwoSum (Knuth) the exact
// addition error, so a pair carries about 48 significant bits — the accuracy of an FP64
// accumulator — while FP64 is used only once per thread and per block.  The explicit _rn
// intrinsics keep the compiler from contracting the error-free transformations into FMAs.
//
// Partials are written per block and summed in one fixed order — by a warp in the consumer
// kernels' preambles (warp_sum_partials) and by one thread in the final reductions
// (sum_partials), with the same arithmetic — so every reader sees the same bits run to run.
#pragma once

#include <cuda_runtime.h>

namespace slemm {

struct DF {
  float hi = 0.f, lo = 0.f;
};

// s += v
__device__ __forceinline__ void df_add(DF& s, float v)
{
  const float t = __fadd_rn(s.hi, v);
  const float bp = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bp)), __fsub_rn(v, bp));
  s.hi = t;
  s.lo = __fadd_rn(s.lo, err);
}

// s += a·b (the product's rounding error goes to the low word)
__device__ __forceinline__ void df_fma(DF& s, float a, float b)
{
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  df_add(s, p);
  s.lo = __fadd_rn(s.lo, e);
}

__device__ __forceinline__ double df_value(const DF& s) { return (double)s.hi + (double)s.lo; }

// hi + lo = d to about 48 bits (hi = fl(d), lo = fl(d − hi))
__device__ __forceinline__ void split_double(double d, float& hi, float& lo)
{
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

// Block sum of one double per thread; the result is valid in thread 0.  sh holds ≥ 32 doubles.
__device__ __forceinline__ double block_sum_d(double v, double* sh)
{
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  return r;
}

// The fixed order of a sum of block partials: lane l of a warp adds part[b] for b ≡ l (mod 32) in
// increasing b, then the 32 lane sums combine by a butterfly (v_l ← v_l + v_(l xor o) for
// o = 16, 8, 4, 2, 1; floating-point addition is commutative, so every lane ends with the same
// value).  A block's preamble reads its column's scalars this way with 32 lanes instead of one
// thread walking a hundred partials.  All 32 lanes of the warp must call it.
__device__ __forceinline__ double warp_sum_partials(const double* __restrict__ part, int nblk)
{
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += part[b];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// The same sum, the same bits, in one thread (the final reductions).
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int nblk)
{
  double v[32];
  for (int l = 0; l < 32; ++l) {
    double s = 0.0;
    for (int b = l; b < nblk; b += 32) s += part[b];
    v[l] = s;
  }
  for (int o = 16; o; o >>= 1) {
    double w[32];
    for (int l = 0; l < 32; ++l) w[l] = v[l] + v[l ^ o];
    for (int l = 0; l < 32; ++l) v[l] = w[l];
  }
  return v[0];
}

// max_b part[b·stride] over b < nblk (0 when nblk = 0), by the 32 lanes of a warp.
__device__ __forceinline__ double warp_max_partials(const double* __restrict__ part, int nblk, int stride = 1,
                                                    double init = 0.0)
{
  const int lane = threadIdx.x & 31;
  double v = init;
  for (int b = lane; b < nblk; b += 32) v = fmax(v, part[(int64_t)b * stride]);
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// V consecutive rows per thread and iteration (V = 4 needs 16-byte aligned addresses).
template <int V>
__device__ __forceinline__ void ldv(const float* p, float (&v)[V])
{
  if constexpr (V == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
  } else {
    v[0] = *p;
  }
}
template <int V>
__device__ __forceinline__ void stv(float* p, const float (&v)[V])
{
  if constexpr (V == 4) *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  else *p = v[0];
}

// Warp 0 evaluates f() once per block (f may use the warp-collective helpers above) and shares
// its double-float split.
template <class F>
__device__ __forceinline__ void block_scalar(F&& f, float* sb, float& hi, float& lo)
{
  if (threadIdx.x < 32) {
    const double v = f();
    if (threadIdx.x == 0) split_double(v, sb[0], sb[1]);
  }
  __syncthreads();
  hi = sb[0];
  lo = sb[1];
}

}  // namespace slemm
