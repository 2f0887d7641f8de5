// probes.cu — the reference's Rademacher probe block generated on the GPU, draw for draw.
//
// The reference fills V (n×n_V, column by column) with std::mt19937(seed + 54321) and
// uniform_real_distribution<float>(0, 1) < 0.5 → −1, then divides each column by its norm
// (src/reml.cpp:597-605).  With a 32-bit engine, generate_canonical<float> returns
// float(x)/2^32 for the engine output x (rounded to nearest), so a draw is −1 exactly when
// float(x) < 2^31.  The column norm is √n (Σ(±1)² is exact), so every entry is ±1/√n in FP32.
//
// MT19937 (Matsumoto & Nishimura, 1998) as a word sequence: x_0 … x_623 is the seeded state
// (x_i = 1812433253·(x_{i−1} ⊕ (x_{i−1} ≫ 30)) + i) and
//   x_j = x_{j−227} ⊕ twist(upper bit of x_{j−624} | lower 31 bits of x_{j−623}),   j ≥ 624,
// draw d being temper(x_{624+d}).  The window (x_d … x_{d+623}) is the generator state before
// draw d.
//
// Parallel generation.  The draws are cut into P chunks of L0 = 624·2^e draws; each chunk is
// generated by its own CTA from its starting window.  Starting windows come from jump-ahead
// (Haramoto, Matsumoto, L'Ecuyer et al., "Efficient jump ahead for F2-linear random number
// generators", 2008): the transition is linear over GF(2) with characteristic polynomial χ
// (degree 19937), so the window J steps ahead is p(A)·window_0 = Σ_i p_i·window_i with
// p = z^J mod χ, i.e. word w of the new window is the XOR of x_{i+w} over the nonzero
// coefficients i of p.  The host computes T_s = z^(624·2^s) mod χ once (repeated squaring; χ
// has 135 terms, so each reduction is cheap) and stores each T_s as its list of nonzero
// exponents.  Chunk windows are then built in ⌈log2 P⌉ doubling levels: level l derives the
// windows of chunks 2^l … 2^(l+1)−1 from those of chunks 0 … 2^l−1 with T_(e+l), each jump
// spread over several CTAs that XOR their partial windows into place (XOR is order-free, so the
// result is deterministic).
//
// One generator step, pipelined.  In x_j = x_{j−227} ⊕ f(x_{j−624}, x_{j−623}) the first operand
// comes from the word the same thread produced one phase earlier when 227 threads each produce
// one word per phase; the other two come from at least two phases back.  So 227 threads run the
// recurrence with one register carry and one CTA barrier every two phases (454 words).
#include "internal.h"

#include <map>
#include <mutex>

namespace slemm {

constexpr int kMtN = 624, kMtM = 397, kMtLag = kMtN - kMtM;   // 227
constexpr int kMtDeg = 19937;
// Exponents of the nonzero terms of χ, the characteristic polynomial of the MT19937
// transition (printed by gen_mt_charpoly.py: Berlekamp–Massey on one output bit sequence).
constexpr int kMtCharTerms[135] = {
    0,     1189,  1416,  1585,  1643,  1870,  2493,  2773,  3000,  3227,  3454,  3681,  3908,  4135,
    4362,  4753,  5661,  6337,  6569,  7129,  7477,  7525,  7583,  7752,  7979,  8206,  9505,  9901,
    9969,  10128, 10693, 10761, 10920, 11089, 11147, 11157, 11215, 11321, 11374, 11384, 11485, 11611,
    11712, 11717, 11838, 11881, 11944, 11997, 12277, 12335, 12393, 12504, 12509, 12620, 12673, 12731,
    12736, 12789, 12905, 12958, 12963, 13137, 13185, 13190, 13243, 13301, 13412, 13528, 13533, 13639,
    13697, 13760, 13813, 13866, 14093, 14151, 14209, 14320, 14325, 14436, 14547, 14552, 14605, 14721,
    14774, 14779, 14953, 15001, 15006, 15059, 15117, 15228, 15344, 15349, 15455, 15513, 15576, 15629,
    15682, 15909, 15967, 16025, 16136, 16141, 16252, 16363, 16368, 16421, 16537, 16590, 16595, 16817,
    16822, 16875, 16933, 17044, 17160, 17271, 17329, 17445, 17498, 17725, 17783, 17841, 17952, 18068,
    18179, 18237, 18406, 18633, 18691, 18860, 19087, 19314, 19937};
constexpr int kMtMaxLog = 48;          // T_s for s < 48: jumps up to 624·2^47 draws
constexpr int kMtSeqWords = 20608;     // ≥ 624 + 88·227: x_0 … x_{19936+623} plus one phase
constexpr int kMtSeqPhases = 88;       // phases that produce x_624 … x_20559
constexpr int kMtJumpThreads = 640;
constexpr int kMtChunkThreads = 256;
constexpr int kMtRing = 2048;          // ring of the chunk generator (≥ 624 + 3 phases + reuse gap)

// ---- host: jump polynomials ----------------------------------------------------------------------
namespace {

constexpr int kPolyWords = (kMtDeg + 63) / 64;   // 312 64-bit words

uint64_t spread32(uint32_t v)
{
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}

uint64_t get64(const std::vector<uint64_t>& a, int64_t pos)
{
  const size_t w = (size_t)(pos >> 6);
  const int o = (int)(pos & 63);
  uint64_t v = a[w] >> o;
  if (o && w + 1 < a.size()) v |= a[w + 1] << (64 - o);
  return v;
}

void xor64(std::vector<uint64_t>& a, int64_t pos, uint64_t v)
{
  const size_t w = (size_t)(pos >> 6);
  const int o = (int)(pos & 63);
  a[w] ^= v << o;
  if (o && w + 1 < a.size()) a[w + 1] ^= v >> (64 - o);
}

// a² mod χ for deg a < 19937 (GF(2): squaring interleaves zeros).  The part at or above z^19937
// is folded down 64 bits at a time from the top: z^19937 ≡ Σ_{t<19937} z^t over χ's other
// terms, all at least 623 bits lower, so a folded chunk never lands in itself.
std::vector<uint64_t> sqr_mod(const std::vector<uint64_t>& a)
{
  std::vector<uint64_t> s(2 * kPolyWords + 1, 0);
  for (int w = 0; w < kPolyWords; ++w) {
    s[2 * w] = spread32((uint32_t)a[w]);
    s[2 * w + 1] = spread32((uint32_t)(a[w] >> 32));
  }
  const int chunks = (int)ceil_div(2 * (kMtDeg - 1) - kMtDeg + 1, 64);
  for (int c = chunks - 1; c >= 0; --c) {
    const int64_t p = kMtDeg + 64 * (int64_t)c;
    const uint64_t v = get64(s, p);
    if (!v) continue;
    xor64(s, p, v);
    for (int q = 0; q < 134; ++q) xor64(s, 64 * (int64_t)c + kMtCharTerms[q], v);
  }
  std::vector<uint64_t> r(s.begin(), s.begin() + kPolyWords);
  r[kPolyWords - 1] &= (1ull << (kMtDeg - 64 * (kPolyWords - 1))) - 1;
  return r;
}

struct MtHostTables {
  std::vector<uint16_t> idx;   // nonzero exponents of T_0, T_1, … concatenated
  int off[kMtMaxLog + 1];
};

const MtHostTables& host_tables()
{
  static MtHostTables T;
  static std::once_flag once;
  std::call_once(once, [] {
    std::vector<uint64_t> p(kPolyWords, 0);
    p[kMtN / 64] = 1ull << (kMtN % 64);   // T_0 = z^624
    for (int s = 0; s < kMtMaxLog; ++s) {
      T.off[s] = (int)T.idx.size();
      for (int b = 0; b < kMtDeg; ++b)
        if ((p[b >> 6] >> (b & 63)) & 1) T.idx.push_back((uint16_t)b);
      p = sqr_mod(p);
    }
    T.off[kMtMaxLog] = (int)T.idx.size();
  });
  return T;
}

struct MtDevTables {
  uint16_t* idx = nullptr;
};

// Device copy of the jump tables for the current device (uploaded once per device).
const uint16_t* device_tables(cudaStream_t st)
{
  static std::mutex mu;
  static std::map<int, MtDevTables> per_dev;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = per_dev.find(dev);
  if (it != per_dev.end()) return it->second.idx;
  const MtHostTables& T = host_tables();
  MtDevTables d;
  CUDA_TRY(cudaMalloc(&d.idx, T.idx.size() * sizeof(uint16_t)));
  CUDA_TRY(cudaMemcpyAsync(d.idx, T.idx.data(), T.idx.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaStreamSynchronize(st));   // the host table is static, but keep the upload ordered
  per_dev[dev] = d;
  return d.idx;
}

}  // namespace

// ---- device -------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mt_step(uint32_t lag227, uint32_t a, uint32_t b)
{
  const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  return lag227 ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y)
{
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// Runs the recurrence from the window held in x (positions 0 … 623, indices taken & kMask):
// at phase t thread tid < 227 produces word 624 + 227·t + tid, stores it and passes it to
// emit(t, word).  Two phases run between barriers: their cross-thread operands are at least two
// phases old, so all four are loaded up front.  `phases` must be even.  Every thread of the CTA
// must call this (it contains barriers).
template <uint32_t kMask, class Emit>
__device__ __forceinline__ void mt_pipeline(uint32_t* x, int64_t phases, Emit&& emit)
{
  const int tid = threadIdx.x;
  const bool act = tid < kMtLag;
  uint32_t prev = act ? x[(kMtM + tid) & kMask] : 0u;   // x_{j−227} for j = 624 + tid
  uint32_t j = (uint32_t)(kMtN + tid);                  // wraps harmlessly: only j & kMask is used
  for (int64_t t = 0; t < phases; t += 2) {
    if (act) {
      const uint32_t a0 = x[(j - kMtN) & kMask], b0 = x[(j - kMtN + 1) & kMask];
      const uint32_t a1 = x[(j + kMtLag - kMtN) & kMask], b1 = x[(j + kMtLag - kMtN + 1) & kMask];
      const uint32_t w0 = mt_step(prev, a0, b0);
      const uint32_t w1 = mt_step(w0, a1, b1);
      x[j & kMask] = w0;
      x[(j + kMtLag) & kMask] = w1;
      prev = w1;
      emit(t, w0);
      emit(t + 1, w1);
    }
    j += 2 * kMtLag;
    __syncthreads();
  }
}

// Window 0: the seeded state of std::mt19937(seed).
__global__ void mt_seed_kernel(uint32_t seed, uint32_t* __restrict__ states)
{
  if (threadIdx.x != 0) return;
  uint32_t s = seed;
  states[0] = s;
  for (int i = 1; i < kMtN; ++i) {
    s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)i;
    states[i] = s;
  }
}

// One doubling level: window of chunk dst0 + a ^= slice blockIdx.y of Σ_i x_{i+w} over the
// exponents i of the jump polynomial, x generated from the window of chunk a.
__global__ void __launch_bounds__(kMtJumpThreads)
mt_jump_kernel(uint32_t* __restrict__ states, int dst0, const uint16_t* __restrict__ idx, int nidx, int slices)
{
  extern __shared__ uint32_t x[];
  const int a = blockIdx.x;
  for (int w = threadIdx.x; w < kMtN; w += blockDim.x) x[w] = states[(size_t)a * kMtN + w];
  __syncthreads();
  mt_pipeline<0xffffffffu>(x, kMtSeqPhases, [](int64_t, uint32_t) {});
  const int per = (nidx + slices - 1) / slices;
  const int q0 = blockIdx.y * per, q1 = min(nidx, q0 + per);
  const int w = threadIdx.x;
  if (w < kMtN && q0 < q1) {
    uint32_t acc = 0;
    for (int q = q0; q < q1; ++q) acc ^= x[idx[q] + w];
    atomicXor(&states[(size_t)(dst0 + a) * kMtN + w], acc);
  }
}

// Chunk k: draws k·L0 … min((k+1)·L0, total) − 1 from its window; draw d goes to
// V[(d / n)·ld + d mod n] as −value when float(temper(x)) < 2^31, else +value.
__global__ void __launch_bounds__(kMtChunkThreads)
mt_chunk_kernel(const uint32_t* __restrict__ states, int64_t L0, int64_t total, int64_t n,
                float* __restrict__ V, int64_t ld, float value)
{
  __shared__ uint32_t x[kMtRing];
  const int k = blockIdx.x;
  for (int w = threadIdx.x; w < kMtN; w += blockDim.x) x[w] = states[(size_t)k * kMtN + w];
  __syncthreads();
  const int64_t d0 = (int64_t)k * L0;
  const int64_t len = min64(L0, total - d0);
  const int tid = threadIdx.x;
  int64_t i = 0;
  float* dst = V;
  if (tid < kMtLag) {
    const int64_t c = (d0 + tid) / n;
    i = d0 + tid - c * n;
    dst = V + c * ld + i;
  }
  const int64_t phases = ceil_div(len, kMtLag);
  mt_pipeline<kMtRing - 1>(x, phases + (phases & 1), [&](int64_t t, uint32_t w) {
    if (kMtLag * t + tid < len) {
      const bool neg = __uint2float_rn(mt_temper(w)) < 2147483648.0f;   // float(x)/2^32 < 0.5
      *dst = neg ? -value : value;
    }
    i += kMtLag;
    dst += kMtLag;
    while (i >= n) {
      i -= n;
      dst += ld - n;
    }
  });
}

// Fills the device block V (n×n_V, ld) with the reference's normalised Rademacher probes.
void rademacher_device(int seed, int64_t n, int n_V, float* dV, int64_t ld, cudaStream_t st)
{
  const float value = 1.0f / std::sqrt((float)n);   // ±1 / ‖±1‖, both IEEE-rounded in FP32
  const int64_t total = n * (int64_t)n_V;
  // chunk count ≈ √(total / 1500): the doubling levels cost ∝ P, the chunk pass ∝ total / P
  const int64_t target = std::max<int64_t>(1, std::min<int64_t>(512, (int64_t)std::sqrt((double)total / 1500.0)));
  int e = 0;
  while (((int64_t)kMtN << e) * target < total) ++e;
  const int64_t L0 = (int64_t)kMtN << e;
  const int P = (int)ceil_div(total, L0);
  int levels = 0;
  while ((1 << levels) < P) ++levels;
  CHECK_ARG(e + levels <= kMtMaxLog, "too many probe draws");
  const MtHostTables& T = host_tables();
  const uint16_t* didx = device_tables(st);
  uint32_t* states = nullptr;
  CUDA_TRY(cudaMallocAsync((void**)&states, (size_t)P * kMtN * sizeof(uint32_t), st));
  try {
    if (P > 1) CUDA_TRY(cudaMemsetAsync(states, 0, (size_t)P * kMtN * sizeof(uint32_t), st));
    mt_seed_kernel<<<1, 32, 0, st>>>((uint32_t)(seed + 54321), states);
    LAUNCH_CHECK();
    if (levels > 0) {
      static std::once_flag attr;
      std::call_once(attr, [] {
        cudaFuncSetAttribute(mt_jump_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMtSeqWords * (int)sizeof(uint32_t));
      });
    }
    const int sms = num_sms();
    for (int l = 0; l < levels; ++l) {
      const int J = std::min(1 << l, P - (1 << l));
      const int s = e + l;
      const int nidx = T.off[s + 1] - T.off[s];
      const int slices = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(2 * sms, J), ceil_div(nidx, 256)));
      mt_jump_kernel<<<dim3(J, slices), kMtJumpThreads, kMtSeqWords * sizeof(uint32_t), st>>>(
          states, 1 << l, didx + T.off[s], nidx, slices);
      LAUNCH_CHECK();
    }
    mt_chunk_kernel<<<P, kMtChunkThreads, 0, st>>>(states, L0, total, n, dV, ld, value);
    LAUNCH_CHECK();
  } catch (...) {
    cudaFreeAsync(states, st);
    throw;
  }
  CUDA_TRY(cudaFreeAsync(states, st));
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
