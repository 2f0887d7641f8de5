// decode.cuh — 2-bit packed counts → BF16 / FP16 / FP32 (device helpers shared by the kernels).
//
// A 32-bit word holds 16 counts x ∈ {0,1,2} as 2-bit binary fields (layout in geno.cu): the even
// elements 2q in bits 2q..2q+1 of the low half-word, the odd elements 2q+1 in bits 16+2q.. of the
// high half-word.  For the element pair q (elements 2q, 2q+1) and k = 2·(q mod 4), taking
// src = word (q < 4) or word ≫ 8 (q ≥ 4):
//   (src & (0x00030003 ≪ k)) | 0x43004300
// is a BF16 pair whose halves are exactly 128 + x·2^k (0x4300 is 128; the count lands in the
// mantissa, or for k = 6 and x = 2 carries into the exponent, which is still 256 = 128 + 2·64).
// One BF16 FMA, v·2^−k − 128·2^−k, then gives x exactly.  So a pair costs one AND-OR on the
// integer pipe and one HFMA2 on the FMA pipe (plus one shift per 8 pairs).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace slemm {

__device__ __forceinline__ uint32_t bf16pair_of(uint32_t word, int q)
{
  const uint32_t src = (q < 4) ? word : (word >> 8);
  const int k = 2 * (q & 3);
  const uint32_t bits = (src & (0x00030003u << k)) | 0x43004300u;
  const float sc = 1.0f / (float)(1 << k);
  const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&bits);
  const __nv_bfloat162 r = __hfma2(v, __float2bfloat162_rn(sc), __float2bfloat162_rn(-128.0f * sc));
  return *reinterpret_cast<const uint32_t*>(&r);
}

// The same pair as FP16: (src & (0x00030003 ≪ k)) | 0x64006400 is an FP16 pair whose halves are
// 1024 + x·2^k (0x6400 is 1024, whose mantissa step is 1; x·2^k ≤ 128 stays inside the 10-bit
// mantissa), and one HFMA2, v·2^−k − 1024·2^−k, gives x exactly.
__device__ __forceinline__ uint32_t f16pair_of(uint32_t word, int q)
{
  const uint32_t src = (q < 4) ? word : (word >> 8);
  const int k = 2 * (q & 3);
  const uint32_t bits = (src & (0x00030003u << k)) | 0x64006400u;
  const float sc = 1.0f / (float)(1 << k);
  const __half2 v = *reinterpret_cast<const __half2*>(&bits);
  const __half2 r = __hfma2(v, __float2half2_rn(sc), __float2half2_rn(-1024.0f * sc));
  return *reinterpret_cast<const uint32_t*>(&r);
}

// The pair as FP16 subnormals, by masking alone: an FP16 whose exponent field is zero is
// mantissa·2^−24, so a count x whose 2-bit field sits at bits 2s, 2s+1 of a half-word (s ≤ 4,
// inside the 10-bit mantissa) reads as x·2^(2s−24).  Pairs q = 0 … 4 are masked in place
// (s = q); pairs 5 … 7 from the word shifted right by 10 (s = q − 5).  The product's other
// operand carries the factor 2^−2s of its K position (f16sub_kscale) and the accumulator is
// multiplied by 2^24, so count·operand is the same product, exactly: one LOP per pair and one
// shift per word.
__device__ __forceinline__ int f16sub_shift(int q) { return q < 5 ? q : q - 5; }
__device__ __forceinline__ uint32_t f16sub_pair_of(uint32_t word, int q)
{
  const uint32_t src = (q < 5) ? word : (word >> 10);
  return src & (0x00030003u << (2 * f16sub_shift(q)));
}
// 2^−2s for the element at K index kidx (K-tiles start at multiples of 64; element j of a
// 16-element word is K index ≡ j mod 16, pair q = j / 2).
__device__ __forceinline__ float f16sub_kscale(int64_t kidx)
{
  const int s = f16sub_shift((int)((kidx & 15) >> 1));
  return __uint_as_float((uint32_t)(127 - 2 * s) << 23);
}
__device__ __forceinline__ float f16sub_kunscale(int64_t kidx)
{
  const int s = f16sub_shift((int)((kidx & 15) >> 1));
  return __uint_as_float((uint32_t)(127 + 2 * s) << 23);
}
constexpr float kF16SubUnscale = 16777216.0f;   // 2^24

template <bool F16>
__device__ __forceinline__ uint32_t pair_of(uint32_t word, int q)
{
  if constexpr (F16) return f16sub_pair_of(word, q);
  else return bf16pair_of(word, q);
}

// The 4 BF16 pairs of elements 8h … 8h+7 of a word (h = 0: pairs 0-3, h = 1: pairs 4-7).
__device__ __forceinline__ uint4 bf16x8_of(uint32_t word, int h)
{
  uint4 r;
  r.x = bf16pair_of(word, 4 * h + 0);
  r.y = bf16pair_of(word, 4 * h + 1);
  r.z = bf16pair_of(word, 4 * h + 2);
  r.w = bf16pair_of(word, 4 * h + 3);
  return r;
}

// Exact FP32 counts of element pair q.
__device__ __forceinline__ void f32pair_of(uint32_t word, int q, float& even, float& odd)
{
  const uint32_t p = bf16pair_of(word, q);
  even = __uint_as_float(p << 16);
  odd = __uint_as_float(p & 0xFFFF0000u);
}

// Count of element e (0..15) of a word, as an integer.
__device__ __forceinline__ uint32_t count_at(uint32_t word, int e)
{
  return (word >> ((e & 1) * 16 + 2 * (e >> 1))) & 3u;
}

}  // namespace slemm
