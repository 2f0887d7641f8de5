// gemm_tc.cu — tcgen05 packed-genotype product for sm_103a.
//
// D[s][n][r] = Σ_{K in split s} count[r,K] · B[n][K].  One CTA owns 256 rows as two 128-row
// tiles, each with its own TMEM accumulator (128 lanes × N FP32 columns), and both consume every
// B tile, so each B byte fetched from L2 feeds twice the MMA work.
//
// Three decoupled shared-memory rings:
//   packed ring (kPk = 8 stages × 2 tiles × 2 KB) ← warp 0: two cp.async.bulk per stage (DRAM);
//   B ring      (nb stages × N·128 B)             ← warp 1: one TMA tile, 128-byte swizzle (L2);
//   A ring      (na stages × 2 × 16 KB BF16)      ← warps 3..10 decode packed → BF16 in the
//                                                   canonical K-major SWIZZLE_128B layout;
// warp 2 allocates TMEM and issues 2 × 4 tcgen05.mma (M=128, N, K=16) per stage, committing to
// the A- and B-ring "empty" barriers; the decoder warps then run the epilogue (tcgen05.ld →
// FP32 partials), one warp per TMEM lane quarter and accumulator.
//
// Every mbarrier wait is bounded by a %globaltimer budget; a wait that gives up sets a bit in
// *err, raises the CTA's abort flag, and the CTA drains the copies and MMAs it issued (again with
// bounded waits), frees its TMEM and returns.  The host reads *err after the operator.
#include "common.h"
#include "decode.cuh"

#include <cuda.h>

namespace slemm {

constexpr int kPk = 8;                 // packed-tile stages
constexpr int kMaxRing = 8;            // barrier array size for the A and B rings
constexpr int kThreads = 352;          // 11 warps
constexpr int kDecWarps = 8;           // warps 3..10
constexpr int kTileA = 16384;          // one 128×64 BF16 tile
constexpr uint64_t kWaitBudgetNs = 2000000000ull;   // 2 s per wait
constexpr size_t kSmemBudget = 227 * 1024;

struct TcSmemLayout {
  int N, na, nb;
  size_t a_off, b_off, pk_off, bar_off, total;
  __host__ __device__ TcSmemLayout(int N_, int na_, int nb_) : N(N_), na(na_), nb(nb_)
  {
    a_off = 0;                                             // na × 2 × 16 KB (1024-aligned)
    b_off = a_off + (size_t)na * 2 * kTileA;               // nb × N·128 B (1024-aligned, N%8==0)
    pk_off = b_off + (size_t)nb * N * 128;                 // kPk × 2 × 2 KB
    bar_off = pk_off + (size_t)kPk * 2 * kTileBytes;       // barriers, TMEM slot, abort flag
    total = bar_off + 512 + 1024;                          // + slack for the 1024-B base alignment
  }
};

// Ring depths for a given N: as deep a B ring as fits after 3 (else 2) A stages.
static TcSmemLayout plan_smem(int N)
{
  for (int na = 3; na >= 2; --na)
    for (int nb = kMaxRing; nb >= 2; --nb) {
      TcSmemLayout L(N, na, nb);
      if (L.total <= kSmemBudget) return L;
    }
  return TcSmemLayout(N, 2, 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; on timeout sets `code` in *err and the CTA abort flag, returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          volatile int* abort_flag)
{
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > kWaitBudgetNs) {
      atomicOr(err, code);
      *abort_flag = 1;
      return false;
    }
  }
}

// Drain-only wait (used on the abort path): bounded, never raises.
__device__ __forceinline__ void mbar_wait_drain(uint64_t* bar, uint32_t parity)
{
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer() - t0 > kWaitBudgetNs) return;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows × 128 B
  d |= (uint64_t)1 << 46;                        // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                        // SWIZZLE_128B
  return d;
}

// Instruction descriptor of kind::f16: BF16 × BF16 → FP32, both K-major, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int N)
{
  return (1u << 4)                      // D format F32
         | (1u << 7)                    // A format BF16
         | (1u << 10)                   // B format BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(128 >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
gemm_tc_kernel(const uint8_t* __restrict__ A, const __grid_constant__ CUtensorMap tmapB,
               float* __restrict__ D, int64_t M_pad, int K_tiles, int tiles_per_split, int N,
               int na, int nb, uint32_t tmem_cols, int* __restrict__ err)
{
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte alignment of the shared-window address (SWIZZLE_128B tiles need it)
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const TcSmemLayout L(N, na, nb);
  uint8_t* sA = smem + L.a_off;
  uint8_t* sB = smem + L.b_off;
  uint8_t* sPk = smem + L.pk_off;
  uint64_t* pk_full = (uint64_t*)(smem + L.bar_off);
  uint64_t* pk_empty = pk_full + kPk;
  uint64_t* b_full = pk_empty + kPk;
  uint64_t* b_empty = b_full + kMaxRing;
  uint64_t* a_full = b_empty + kMaxRing;
  uint64_t* a_empty = a_full + kMaxRing;
  uint64_t* accum = a_empty + kMaxRing;
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t mt0 = (int64_t)blockIdx.x * 2;   // first of the CTA's two 128-row tiles
  const int split = blockIdx.y;
  const int kt0 = split * tiles_per_split;
  const int kt1 = min(K_tiles, kt0 + tiles_per_split);
  const int nk = max(0, kt1 - kt0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kPk; ++s) {
      mbar_init(&pk_full[s], 1);
      mbar_init(&pk_empty[s], kDecWarps);
    }
    for (int s = 0; s < kMaxRing; ++s) {
      mbar_init(&b_full[s], 1);
      mbar_init(&b_empty[s], 1);
      mbar_init(&a_full[s], kDecWarps);
      mbar_init(&a_empty[s], 1);
    }
    mbar_init(accum, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- packed-tile producer (DRAM) ----------------
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nk; ++i) {
        const int s = i % kPk;
        const uint32_t round = (uint32_t)(i / kPk);
        if (i >= kPk && !mbar_wait(&pk_empty[s], (round - 1) & 1, err, 1, abort_flag)) break;
        if (*abort_flag) break;
        mbar_arrive_expect_tx(&pk_full[s], 2u * kTileBytes);
        const int kt = kt0 + i;
        uint8_t* dst = sPk + (size_t)s * 2 * kTileBytes;
        bulk_copy_g2s(dst, A + ((size_t)mt0 * K_tiles + kt) * kTileBytes, kTileBytes, &pk_full[s]);
        bulk_copy_g2s(dst + kTileBytes, A + ((size_t)(mt0 + 1) * K_tiles + kt) * kTileBytes, kTileBytes,
                      &pk_full[s]);
        ++issued;
      }
      if (*abort_flag)   // let issued copies land before the CTA's shared memory is released
        for (int i = max(0, issued - kPk); i < issued; ++i)
          mbar_wait_drain(&pk_full[i % kPk], (uint32_t)(i / kPk) & 1);
    }
  } else if (warp == 1) {
    // ---------------- B producer (L2) ----------------
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)N * 128u;
      int issued = 0;
      for (int i = 0; i < nk; ++i) {
        const int s = i % nb;
        const uint32_t round = (uint32_t)(i / nb);
        if (i >= nb && !mbar_wait(&b_empty[s], (round - 1) & 1, err, 16, abort_flag)) break;
        if (*abort_flag) break;
        mbar_arrive_expect_tx(&b_full[s], bytes);
        tma_load_2d(sB + (size_t)s * N * 128, &tmapB, (kt0 + i) * kTileK, 0, &b_full[s]);
        ++issued;
      }
      if (*abort_flag)
        for (int i = max(0, issued - nb); i < issued; ++i)
          mbar_wait_drain(&b_full[i % nb], (uint32_t)(i / nb) & 1);
    }
  } else if (warp == 2) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(N);
      for (int i = 0; i < nk; ++i) {
        const int sa = i % na, sb = i % nb;
        if (!mbar_wait(&a_full[sa], (uint32_t)(i / na) & 1, err, 2, abort_flag)) break;
        if (!mbar_wait(&b_full[sb], (uint32_t)(i / nb) & 1, err, 32, abort_flag)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(sA + (size_t)sa * 2 * kTileA);
        const uint32_t b0 = smem_u32(sB + (size_t)sb * N * 128);
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            mma_bf16(tmem_base + (uint32_t)(t * N), sw128_desc(a0 + t * kTileA + kk * 32),
                     sw128_desc(b0 + kk * 32), idesc, (i > 0 || kk > 0) ? 1u : 0u);
        mma_commit(&a_empty[sa]);
        mma_commit(&b_empty[sb]);
      }
      mma_commit(accum);   // arrives once every MMA issued above has completed
    }
  } else {
    // ---------------- decoders (thread → one row of the 256), then epilogue ----------------
    const int t = threadIdx.x - 96;        // 0..255
    const int sub = t >> 7, r = t & 127;   // tile 0/1, row in tile
    for (int i = 0; i < nk; ++i) {
      const int sp = i % kPk, sa = i % na;
      bool got = mbar_wait(&pk_full[sp], (uint32_t)(i / kPk) & 1, err, 4, abort_flag);
      if (!__all_sync(0xffffffffu, got)) break;   // warp-uniform exit
      const uint4 pk = *reinterpret_cast<const uint4*>(sPk + ((size_t)sp * 2 + sub) * kTileBytes + r * 16);
      __syncwarp();
      if (lane == 0) mbar_arrive(&pk_empty[sp]);
      if (i >= na) {
        got = mbar_wait(&a_empty[sa], (uint32_t)(i / na - 1) & 1, err, 64, abort_flag);
        if (!__all_sync(0xffffffffu, got)) break;
      }
      uint8_t* rowp = sA + ((size_t)sa * 2 + sub) * kTileA + r * 128;
      const uint32_t words[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int chunk = 2 * w + h;   // 16-byte chunk of the 128-byte row
          *reinterpret_cast<uint4*>(rowp + ((chunk ^ (r & 7)) << 4)) = bf16x8_of(words[w], h);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&a_full[sa]);
    }
    // epilogue: warps 3..6 read accumulator 0, warps 7..10 accumulator 1; each warp owns TMEM
    // lanes 32·(warp%4) … +31 (its rows within the tile)
    const int acc = (warp - 3) >> 2;
    const int lq = warp & 3;
    const int row = lq * 32 + lane;
    const bool got = mbar_wait(accum, 0, err, 8, abort_flag);
    const bool ok = __all_sync(0xffffffffu, got && !*abort_flag);   // tcgen05.ld is warp-wide
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
      float* Dbase = D + ((size_t)split * N) * M_pad + (mt0 + acc) * 128 + row;
      for (int c0 = 0; c0 < N; c0 += 16) {
        uint32_t v[16];
        tmem_ld16(tmem_base + ((uint32_t)(lq * 32) << 16) + (uint32_t)(acc * N + c0), v);
        if (nk == 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = 0u;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) Dbase[(size_t)(c0 + j) * M_pad] = __uint_as_float(v[j]);
      }
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) {
    if (*abort_flag && lane == 0) mbar_wait_drain(accum, 0);   // MMAs finished before freeing TMEM
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(tmem_cols)
                 : "memory");
  }
}

// ---- host side ------------------------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                    const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                    const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled get_encode()
{
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    CUDA_TRY(cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q));
    if (!p || q != cudaDriverEntryPointSuccess)
      SLEMM_THROW(SLEMM_ERR_CUDA, "cuTensorMapEncodeTiled entry point not found");
    fn = (PFN_encodeTiled)p;
  }
  return fn;
}

void gemm_tc(const GemmArgs& a, cudaStream_t st)
{
  CHECK_ARG(a.N >= 16 && a.N <= 256 && a.N % 16 == 0, "TC path needs N in [16,256], N%16==0");
  CHECK_ARG(a.M_pad % (2 * kTileM) == 0 && a.K_pad % 128 == 0, "unpadded operand");
  CHECK_ARG(((uintptr_t)a.A % 16) == 0 && ((uintptr_t)a.B % 16) == 0, "misaligned operand");
  const int64_t M2 = a.M_pad / (2 * kTileM);
  const int K_tiles = (int)(a.K_pad / kTileK);
  const int tps = (int)ceil_div(K_tiles, a.splits);

  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)a.K_pad, (cuuint64_t)a.N};
  const cuuint64_t strides[1] = {(cuuint64_t)a.K_pad * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)a.N};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = get_encode()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(a.B), dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) SLEMM_THROW(SLEMM_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));

  const TcSmemLayout L = plan_smem(a.N);
  CHECK_ARG(L.total <= kSmemBudget, "shared-memory plan exceeds 227 KB");
  static size_t configured = 0;
  if (L.total > configured) {
    CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
    configured = kSmemBudget;
  }
  // two accumulators of N columns: allocate the next power of two ≥ 2N (≤ 512)
  const uint32_t cols = 2 * a.N <= 32 ? 32u : 2 * a.N <= 64 ? 64u : 2 * a.N <= 128 ? 128u : 2 * a.N <= 256 ? 256u : 512u;
  dim3 grid((unsigned)M2, (unsigned)a.splits);
  gemm_tc_kernel<<<grid, kThreads, L.total, st>>>(a.A, map, a.D, a.M_pad, K_tiles, tps, a.N, L.na, L.nb, cols,
                                                  a.err);
  LAUNCH_CHECK();
}

}  // namespace slemm
