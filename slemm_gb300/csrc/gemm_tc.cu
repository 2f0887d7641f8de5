// gemm_tc.cu — tcgen05 packed-genotype product for sm_103a.
//
// D[s][n][r] = Σ_{K in split s} count[r,K] · B[n][K].  One CTA owns SUB (1 or 2) tiles of 128
// rows, each with its own TMEM accumulator (128 lanes × N FP32 columns); every B tile feeds all
// of them.  The decoded counts (the MMA's A operand) never touch shared memory: decoder threads
// turn their row's 16 packed bytes into 32 16-bit pairs in registers and write them into tensor
// memory with tcgen05.st; the MMA reads A from TMEM and B from shared memory.  BF16 pairs cost
// one LOP and one HFMA2 each; FP16 pairs are the counts as FP16 subnormals, one LOP each, with
// the matching power of two per K position in B and 2^24 in the epilogue (decode.cuh).
//
// What limits tcgen05 here is the issuing thread, not the tensor pipe.  Measured on GB300: one
// thread issuing M=128, N=144, K=16 BF16 MMAs back to back keeps the pipe full (72 cycles per
// MMA, 8192 FLOP/clk per SM) whether A comes from TMEM or shared memory, but a barrier wait and
// fence between groups of MMAs leave it idle for ~150 cycles each unless a second thread issues
// meanwhile, and every instruction of the issuing thread competes for issue slots with the decoder
// warps on its SM sub-partition (their integer/FMA work, not their TMEM stores, costs ~100 cycles
// per 576-cycle stage).  So each tile has its own MMA-issuing warp, each stage costs that thread
// one wait, one fence, four MMAs and ONE commit, and its loop is unrolled over the ring so slots,
// parities and descriptor offsets are constants.
//
// Roles (warp w):
//   w = 0          packed-tile producer: per ring slot, one cp.async.bulk of kPkg K-tiles (8 KB)
//                  per tile;
//   w = 1          B producer: one TMA tile (N rows × 64 BF16, 128-byte swizzle) per stage;
//   w = 2 … 1+SUB  MMA issuers, one per tile (w = 2 also allocates TMEM);
//   w = 2+SUB …    kNG groups of 4·SUB decoder warps; group g decodes stages i ≡ g (mod kNG).
//                  Warp w covers TMEM lanes 32·(w mod 4) …, i.e. those rows of its tile.  Group 0
//                  also runs the epilogue (tcgen05.ld → FP32 partials).
//
// Barriers: pk_full/pk_empty per packed slot; st_full per A stage (the decoder warps, plus the B
// copy's expect_tx when B rides on the A stages); b_full per B stage; done[i mod BS] per stage,
// one commit from each MMA thread, which frees both the A stage and the B stage of stage i.
// TMEM columns: accumulators [0, SUB·N), then S stages of SUB × 32 columns of A (64 BF16 of K per
// row).  Every mbarrier wait is bounded by a %globaltimer budget; a wait that gives up sets a bit
// in *err, raises the CTA's abort flag, and the CTA drains what it issued (bounded), frees its
// TMEM and returns.  The host reads *err after the operator.
#include "common.h"
#include "decode.cuh"

#include <cuda.h>

namespace slemm {

// Ring depths, a template quadruple <PK, S, SB, KT>: PK packed slots of kPkg K-tiles each, S A
// (TMEM) stages and SB B (smem) stages, each stage KT K-tiles of 64.  B has its own, deeper ring:
// its tiles come from L2 (every row tile of a split reads the same B) with a latency of ~1500
// cycles under load, so they are requested SB stages ahead instead of only as far ahead as the
// TMEM-bound A ring allows; one decoder warp of each stage waits for its B tile before arriving,
// so the MMA thread still waits on one barrier per stage.  The K-tiles of a row tile are
// contiguous in HBM, so one bulk copy moves a whole slot: one 2 KB copy per K-tile paced the
// kernel at ~750 cycles per K-tile, four K-tiles per copy take a quarter of that.  Wide blocks
// (N > 64) use <4, 3, 6, 1>.  Narrow ones, whose MMAs are short, are paced by the issuing thread's
// fixed cost per stage (wait, fence, commit) rather than by the tensor pipe, so their stages hold
// two K-tiles (eight MMAs per wait and commit; the small accumulators leave TMEM room for three
// such stages): <6, 3, 0, 2>, where SB = 0 puts B on the A stages' own full barrier (the B
// producer's expect_tx), which measured faster for narrow blocks than a separate B ring.
constexpr int kPkg = 4;                // K-tiles per packed slot
constexpr int kNG = 3;                 // decoder groups (each keeps one stage in flight)
constexpr int kMaxThreads = 64 + 2 * 32 + kNG * 2 * 128;   // SUB = 2
// Threads of a one-tile CTA (the narrow plan that runs two CTAs per SM, 256 TMEM columns each).
constexpr int kThreads1 = 64 + 32 + kNG * 128;
// Launch bounds of a plan: TM = 512 TMEM columns per CTA, one CTA per SM; TM = 256, two.
constexpr int tc_max_threads(int TM) { return TM == 512 ? kMaxThreads : kThreads1; }
constexpr int tc_min_blocks(int TM) { return TM == 512 ? 1 : 2; }
constexpr uint64_t kWaitBudgetNs = 2000000000ull;   // 2 s per wait
constexpr size_t kSmemBudget = 227 * 1024;

template <int PK, int S, int SB, int KT>
struct TcPlan {
  int N, sub;
  size_t b_off, pk_off, bar_off, total;
  __host__ __device__ TcPlan(int N_, int sub_) : N(N_), sub(sub_)
  {
    b_off = 0;                                         // BS × KT × N·128 B (1024-aligned, N%8==0)
    pk_off = b_off + (size_t)(SB > 0 ? SB : S) * KT * N * 128;   // PK × sub × kPkg × 2 KB
    bar_off = pk_off + (size_t)PK * sub * kPkg * kTileBytes;
    total = bar_off + 512 + 1024;                      // barriers/slots + 1024-B base alignment
  }
  __host__ __device__ int mma_warp0() const { return 2; }
  __host__ __device__ int dec_warp0() const { return 2 + sub; }
  __host__ __device__ int threads() const { return 32 * (2 + sub + kNG * 4 * sub); }
  // first A column: after the accumulators, 32-column aligned for tcgen05.st
  __host__ __device__ uint32_t acol() const { return (uint32_t)(((sub * N + 31) / 32) * 32); }
};

// Two tiles when their accumulators and S A-stages of KT K-tiles fit the 512 TMEM columns, else one;
// a plan with TM = 256 (two CTAs per SM) always has one tile.
template <int PK, int S, int SB, int KT, int TM = 512>
static TcPlan<PK, S, SB, KT> plan_tc(int N)
{
  if (TM == 512 && (((2 * N + 31) / 32) * 32) + 2 * 32 * KT * S <= 512) return TcPlan<PK, S, SB, KT>(N, 2);
  return TcPlan<PK, S, SB, KT>(N, 1);
}
constexpr int kNarrowN = 64;   // N ≤ 64 uses the deep ring

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

// Bounded wait; on timeout sets `code` in *err and the CTA abort flag, returns false.  The abort
// flag and the timer are looked at only every 64 polls, and `sleep_ns` > 0 makes a waiter back
// off between polls, so waiting warps do not crowd the barrier and shared-memory pipes that the
// MMA-issuing thread depends on.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          volatile int* abort_flag, uint32_t sleep_ns = 0)
{
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (sleep_ns) __nanosleep(sleep_ns);
    if ((it & 63u) == 0) {
      if (*abort_flag) return false;
      if (globaltimer() - t0 > kWaitBudgetNs) {
        atomicOr(err, code);
        *abort_flag = 1;
        return false;
      }
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

// Instruction descriptor of kind::f16: BF16 × BF16 (or FP16 × FP16) → FP32, both K-major, M = 128.
// A and B always have the same type.
__host__ __device__ constexpr uint32_t idesc_f16kind(int N, bool f16)
{
  return (1u << 4)                          // D format F32
         | ((f16 ? 0u : 1u) << 7)           // A format: 0 FP16, 1 BF16
         | ((f16 ? 0u : 1u) << 10)          // B format: 0 FP16, 1 BF16
         | ((uint32_t)(N >> 3) << 17)       // N / 8
         | ((uint32_t)(128 >> 4) << 24);    // M / 16
}

// D[tmem] (+)= A[tmem] · B[smem]
__device__ __forceinline__ void mma_bf16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 8 consecutive TMEM columns (from a multiple of 8) of this warp's 32 lanes; no wait.
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8])
{
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
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

// 32 consecutive TMEM columns of this warp's 32 lanes ← 32 registers per thread.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&v)[32])
{
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
      "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(
          taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
      "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]),
      "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]),
      "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
      : "memory");
}

template <int PK, int S, int SB, int KT, bool F16, int TM>
__global__ void __launch_bounds__(tc_max_threads(TM), tc_min_blocks(TM))
gemm_tc_kernel(const uint8_t* __restrict__ A, const __grid_constant__ CUtensorMap tmapB,
               float* __restrict__ D, int64_t M_pad, int K_tiles, int tiles_per_split, int N, int sub,
               int kp, int pieces, int* __restrict__ err, int withhold)
{
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte alignment of the shared-window address (SWIZZLE_128B tiles need it)
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const TcPlan<PK, S, SB, KT> P(N, sub);
  uint8_t* sB = smem + P.b_off;
  uint8_t* sPk = smem + P.pk_off;
  uint64_t* pk_full = (uint64_t*)(smem + P.bar_off);
  uint64_t* pk_empty = pk_full + PK;
  constexpr int BS = SB > 0 ? SB : S;          // B stages (SB = 0: B rides on the A stages)
  static_assert(BS % S == 0, "the stage-done ring serves both rings");
  static_assert(kPkg % KT == 0, "a stage's K-tiles lie in one packed slot");
  uint64_t* st_full = pk_empty + PK;
  uint64_t* done = st_full + S;                // done[i % BS]: the MMAs of stage i have completed
  uint64_t* b_full = done + BS;
  uint64_t* accum = b_full + BS;
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int dec_warps = sub * 4;               // decoder warps per group
  const int64_t mt0 = (int64_t)blockIdx.x * sub;
  const int split = blockIdx.y;
  const int kt0 = split * tiles_per_split;
  const int kt1 = min(K_tiles, kt0 + tiles_per_split);
  const int nk = max(0, kt1 - kt0);            // K-tiles of this split (a multiple of KT)
  const int ns = nk / KT;                      // stages

  if (threadIdx.x == 0) {
    for (int s = 0; s < PK; ++s) {
      mbar_init(&pk_full[s], 1);
      mbar_init(&pk_empty[s], dec_warps * (kPkg / KT));   // the decoders of each of the slot's stages
    }
    for (int s = 0; s < S; ++s)
      mbar_init(&st_full[s], dec_warps + (SB > 0 ? 0 : 1));   // decoder warps (+ B's expect_tx if SB = 0)
    for (int s = 0; s < BS; ++s) {
      mbar_init(&done[s], sub);                // one commit per MMA-issuing thread
      mbar_init(&b_full[s], 1);                // the B producer's expect_tx (unused if SB = 0)
    }
    mbar_init(accum, sub);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TM)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;
  const uint32_t acol = P.acol();

  if (warp == 0) {
    // ---------------- packed-tile producer (DRAM) ----------------
    if (lane == 0) {
      int issued = 0;
      const int nslots = (nk + kPkg - 1) / kPkg;
      for (int j = 0; j < nslots; ++j) {
        const int s = j % PK;
        const uint32_t round = (uint32_t)(j / PK);
        if (j >= PK && !mbar_wait(&pk_empty[s], (round - 1) & 1, err, 1, abort_flag, 128)) break;
        if (*abort_flag) break;
        const int cnt = min(kPkg, nk - j * kPkg);   // K-tiles in this slot
        const uint32_t bytes = (uint32_t)(cnt * kTileBytes);
        mbar_arrive_expect_tx(&pk_full[s], (uint32_t)sub * bytes);
        const int kt = kt0 + j * kPkg;
        uint8_t* dst = sPk + (size_t)s * sub * kPkg * kTileBytes;
        for (int t = 0; t < sub; ++t)
          bulk_copy_g2s(dst + (size_t)t * kPkg * kTileBytes, A + ((size_t)(mt0 + t) * K_tiles + kt) * kTileBytes, bytes,
                        &pk_full[s]);
        ++issued;
      }
      if (*abort_flag)   // let issued copies land before the CTA's shared memory is released
        for (int j = max(0, issued - PK); j < issued; ++j)
          mbar_wait_drain(&pk_full[j % PK], (uint32_t)(j / PK) & 1);
    }
  } else if (warp == 1) {
    // ---------------- B producer (L2) ----------------
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)N * 128u;   // one K-tile of B
      int issued = 0;
      for (int i = 0; i < ns; ++i) {
        const int s = i % BS;
        const uint32_t round = (uint32_t)(i / BS);
        uint64_t* full = (SB > 0) ? &b_full[s] : &st_full[s];
        if (i >= BS && !mbar_wait(&done[s], (round - 1) & 1, err, 16, abort_flag, 128)) break;
        if (*abort_flag) break;
        if (i == withhold && blockIdx.x == 0 && blockIdx.y == 0) {   // test support: the stage never fills
          ++issued;
          continue;
        }
        mbar_arrive_expect_tx(full, (uint32_t)KT * bytes);
        for (int kk = 0; kk < KT; ++kk)
          tma_load_2d(sB + ((size_t)s * KT + kk) * N * 128, &tmapB, (kt0 + i * KT + kk) * kTileK, 0, full);
        ++issued;
      }
      if (*abort_flag)
        for (int i = max(0, issued - BS); i < issued; ++i)
          mbar_wait_drain((SB > 0) ? &b_full[i % BS] : &st_full[i % BS], (uint32_t)(i / BS) & 1);
    }
  } else if (warp < P.dec_warp0()) {
    // ---------------- MMA issuer for tile t ----------------
    // One issuing thread per tile: MMA issue is effectively blocking, and while one thread
    // waits, fences and commits, the other tile's MMAs keep the tensor pipe fed (one thread for
    // both tiles, or four column-group issuers, measured slower).
    const int t = warp - P.mma_warp0();
    if (lane == 0) {
      const uint32_t idesc = idesc_f16kind(N, F16);
      const uint64_t bdesc0 = sw128_desc(smem_u32(sB));
      const uint32_t bstep = (uint32_t)(N * 128) >> 4;          // descriptor units per B K-tile
      const uint32_t d_tmem = tmem_base + (uint32_t)(t * N);
      const uint32_t a_base = tmem_base + acol + (uint32_t)(t * 32 * KT);
      const uint32_t a_step = (uint32_t)(sub * 32 * KT);        // columns per A stage
      // Unrolled over one turn of the B ring (BS stages, a whole number of A-ring turns), so
      // ring slots, parities and descriptor offsets are constants: the issuing thread shares
      // its SM sub-partition with decoder warps, and every instruction it waits to issue
      // delays the tensor pipe.
      bool ok = true;
      for (int i0 = 0; i0 < ns && ok; i0 += BS) {
        const uint32_t ph0 = (uint32_t)(i0 / S) & 1u;
#pragma unroll
        for (int u = 0; u < BS; ++u) {
          const int i = i0 + u;
          if (i >= ns) break;
          if (!mbar_wait(&st_full[u % S], ph0 ^ (uint32_t)((u / S) & 1), err, 2, abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
          for (int kk = 0; kk < KT; ++kk) {
            const uint64_t bd = bdesc0 + (uint64_t)((u * KT + kk) * bstep);
            const uint32_t ad = a_base + (uint32_t)(u % S) * a_step + (uint32_t)(kk * 32);
            mma_bf16_ts(d_tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            mma_bf16_ts(d_tmem, ad + 8, bd + 2, idesc, 1u);
            mma_bf16_ts(d_tmem, ad + 16, bd + 4, idesc, 1u);
            mma_bf16_ts(d_tmem, ad + 24, bd + 6, idesc, 1u);
          }
          mma_commit(&done[u]);   // frees A stage u % S and B stage u once these MMAs complete
        }
      }
      mma_commit(accum);   // arrives once every MMA this thread issued has completed
    }
  } else {
    // ---------------- decoders (one row per thread), then epilogue ----------------
    const int dw = warp - P.dec_warp0();     // decoder warp index
    const int grp = dw / dec_warps;          // group: stages i ≡ grp (mod kNG)
    const int tsub = (dw % dec_warps) >> 2;  // tile 0 … sub−1
    const int lq = warp & 3;                 // TMEM lane quarter = row quarter
    const int r = lq * 32 + lane;            // row within the tile
    for (int i = grp; i < ns; i += kNG) {
      const int q0 = i * KT;                   // first K-tile of stage i
      const int slot = q0 / kPkg, sp = slot % PK, u0 = q0 % kPkg, s = i % S;
      bool got = mbar_wait(&pk_full[sp], (uint32_t)(slot / PK) & 1, err, 4, abort_flag, 64);
      if (!__all_sync(0xffffffffu, got)) break;   // warp-uniform exit
      uint4 pk[KT];
#pragma unroll
      for (int kk = 0; kk < KT; ++kk)
        pk[kk] = *reinterpret_cast<const uint4*>(sPk + (((size_t)sp * sub + tsub) * kPkg + u0 + kk) * kTileBytes + r * 16);
      __syncwarp();
      if (lane == 0) mbar_arrive(&pk_empty[sp]);
      bool ok = true;
#pragma unroll
      for (int kk = 0; kk < KT; ++kk) {
        uint32_t v[32];
        const uint32_t words[4] = {pk[kk].x, pk[kk].y, pk[kk].z, pk[kk].w};
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int q = 0; q < 8; ++q) v[w * 8 + q] = pair_of<F16>(words[w], q);
        if (kk == 0 && i >= S) {   // the stage that last used this A slot has been consumed
          got = mbar_wait(&done[(i - S) % BS], (uint32_t)((i - S) / BS) & 1, err, 64, abort_flag, 64);
          if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        tmem_st32(tmem_base + ((uint32_t)(lq * 32) << 16) + acol + (uint32_t)(((s * sub + tsub) * KT + kk) * 32), v);
      }
      if (!ok) break;
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (SB > 0 && (dw % dec_warps) == 0) {   // this stage's B tile has landed before the stage is full
        got = mbar_wait(&b_full[i % BS], (uint32_t)(i / BS) & 1, err, 32, abort_flag, 64);
        if (!__all_sync(0xffffffffu, got)) break;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&st_full[s]);
    }
    // epilogue (group 0): each warp owns its lane quarter of one tile's accumulator
    if (grp == 0) {
      const bool got = mbar_wait(accum, 0, err, 8, abort_flag, 256);
      const bool ok = __all_sync(0xffffffffu, got && !*abort_flag);   // tcgen05.ld is warp-wide
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (ok) {
        // column c of D = Σ_p accumulator column p·kp + c (the pieces of c): kp columns per split
        float* Dbase = D + ((size_t)split * kp) * M_pad + (mt0 + tsub) * 128 + r;
        const uint32_t tl = tmem_base + ((uint32_t)(lq * 32) << 16) + (uint32_t)(tsub * N);
        for (int c0 = 0; c0 < kp; c0 += 8) {
          float acc[8] = {};
          for (int p = 0; p < pieces; ++p) {
            uint32_t o[8];
            tmem_ld8_nowait(tl + (uint32_t)(p * kp + c0), o);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = __fadd_rn(acc[j], __uint_as_float(o[j]));
          }
          if (nk == 0) {
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = 0.f;
          }
          if constexpr (F16) {   // the FP16 counts were x·2^(2s−24), the operand ·2^−2s
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = __fmul_rn(acc[j], kF16SubUnscale);
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) Dbase[(size_t)(c0 + j) * M_pad] = acc[j];
        }
      }
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) {
    if (*abort_flag && lane == 0) mbar_wait_drain(accum, 0);   // MMAs finished before freeing TMEM
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TM)
                 : "memory");
  }
}

// ---- host side ------------------------------------------------------------------------------
// Test support (slemm_gpu_test_withhold_b_stage): the B stage the next tensor-core launch leaves
// unfilled in its first CTA, or −1.  Read and reset by that launch.
static std::atomic<int> g_withhold_b{-1};

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

int gemm_tc_rows_per_cta(int N, int plan)
{
  if (N <= kNarrowN && plan == 1) return kTileM;
  return (N <= kNarrowN ? plan_tc<6, 3, 0, 2>(N).sub : plan_tc<4, 3, 6, 1>(N).sub) * kTileM;
}

// Sets the kernel's shared-memory limit once per device (the attribute belongs to the device's
// context, so a process that uses several GPUs sets it on each).
template <auto kernel>   // one flag set per kernel instantiation
static void configure_once()
{
  static std::atomic<uint64_t> done{0};
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
  if (bit && (done.load() & bit)) return;
  CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
  done.fetch_or(bit);
}

template <int PK, int S, int SB, int KT, bool F16, int TM = 512>
static void launch_tc(const GemmArgs& a, cudaStream_t st)
{
  const TcPlan<PK, S, SB, KT> P = plan_tc<PK, S, SB, KT, TM>(a.N);
  CHECK_ARG(a.M_pad % (P.sub * kTileM) == 0 && a.K_pad % 128 == 0, "unpadded operand");
  CHECK_ARG(((uintptr_t)a.A % 16) == 0 && ((uintptr_t)a.B % 16) == 0, "misaligned operand");
  CHECK_ARG(P.total <= kSmemBudget && P.acol() + 32 * P.sub * S * KT <= TM, "no TMEM/shared-memory plan for this N");
  const int64_t Mc = a.M_pad / (P.sub * kTileM);
  const int K_tiles = (int)(a.K_pad / kTileK);
  CHECK_ARG(K_tiles % KT == 0, "K tiles not a multiple of the stage");
  const int tps = (int)(ceil_div(ceil_div(K_tiles, a.splits), KT) * KT);   // whole stages per split

  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)a.K_pad, (cuuint64_t)a.N};
  const cuuint64_t strides[1] = {(cuuint64_t)a.K_pad * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)a.N};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = get_encode()(&map, F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                            const_cast<void*>(a.B), dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) SLEMM_THROW(SLEMM_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));

  configure_once<gemm_tc_kernel<PK, S, SB, KT, F16, TM>>();
  CHECK_ARG(a.kp % 8 == 0 && a.pieces >= 1 && a.pieces * a.kp <= a.N, "bad piece layout");
  // Each CTA allocates TM of the SM's 512 TMEM columns: request enough shared memory that at most
  // 512 / TM CTAs are resident per SM, so no allocation ever has to wait for another CTA's release.
  const size_t smem = std::max<size_t>(P.total, TM == 512 ? 120 * 1024 : 80 * 1024);
  dim3 grid((unsigned)Mc, (unsigned)a.splits);
  gemm_tc_kernel<PK, S, SB, KT, F16, TM><<<grid, P.threads(), smem, st>>>(a.A, map, a.D, a.M_pad, K_tiles, tps, a.N,
                                                                       P.sub, a.kp, a.pieces, a.err,
                                                                       g_withhold_b.exchange(-1));
  LAUNCH_CHECK();
}

void gemm_tc(const GemmArgs& a, cudaStream_t st)
{
  CHECK_ARG(a.N >= 16 && a.N <= 256 && a.N % 16 == 0, "TC path needs N in [16,256], N%16==0");
  CHECK_ARG(a.plan == 0 || (a.plan == 1 && a.N <= kNarrowN), "unknown tensor-core plan");
  if (a.f16) {
    if (a.N > kNarrowN) launch_tc<4, 3, 6, 1, true>(a, st);
    else if (a.plan == 1) launch_tc<6, 3, 0, 2, true, 256>(a, st);
    else launch_tc<6, 3, 0, 2, true>(a, st);
  } else {
    if (a.N > kNarrowN) launch_tc<4, 3, 6, 1, false>(a, st);
    else if (a.plan == 1) launch_tc<6, 3, 0, 2, false, 256>(a, st);
    else launch_tc<6, 3, 0, 2, false>(a, st);
  }
}

}  // namespace slemm

extern "C" int slemm_gpu_test_withhold_b_stage(int stage)
{
  slemm::g_withhold_b.store(stage < 0 ? -1 : stage);
  return SLEMM_OK;
}
