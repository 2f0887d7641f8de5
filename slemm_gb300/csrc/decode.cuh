// decode.cuh — 2-bit plane-encoded counts → BF16 / FP32 (device helpers shared by the kernels).
//
// A 32-bit word holds 16 counts x (layout in geno.cu): for element pair q (elements 2q, 2q+1),
// (word >> q) has nz_even at bit 0, hi_even at bit 8, nz_odd at bit 16, hi_odd at bit 24.
// BF16(x) = nz·0x3F80 + hi·0x0080 (0 → 0x0000, 1 → 0x3F80, 2 → 0x4000), so one AND, one
// shift-AND and one integer multiply-add give the packed BF16 pair of both elements.
#pragma once
#include <cstdint>

namespace slemm {

__device__ __forceinline__ uint32_t bf16pair_of(uint32_t word, int q)
{
  const uint32_t s = word >> q;
  return (s & 0x00010001u) * 0x3F80u + ((s >> 1) & 0x00800080u);
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

}  // namespace slemm
