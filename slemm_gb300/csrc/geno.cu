// geno.cu — library state, the packed genotype handle and its bit-exact integer kernels.
//
// Device layout of the counts.  The reference keeps genotypes as m rows of 2n bits
// (std::vector<std::vector<bool>>, src/option.cpp:347) decoded byte by byte from the .bed
// (src/input.cpp:343-386).  Here each allele-2 count x ∈ {0,1,2} is a 2-bit binary field in a
// tiled layout:
//   tile (mt, kt) = 128 rows × 64 K-elements = 2048 contiguous bytes at
//   ((mt·K_tiles + kt)·128 + r)·16; the 16 bytes of row r hold K-elements kt·64 … kt·64+63 as
//   four 32-bit words, word w covering elements 16w … 16w+15 with
//     bits  2q, 2q+1      : the even element 16w+2q
//     bits 16+2q, 17+2q   : the odd element 16w+2q+1
// so that an element pair becomes a BF16 pair with one AND-OR and one BF16 FMA (decode.cuh).
// Two copies are kept: G (rows = SNPs, K = individuals) and GT
// (rows = individuals, K = SNPs), so both products read K-contiguous tiles with one 2048-byte
// bulk copy per tile.  Padding rows/columns hold count 0.
#include "internal.h"

#include <map>

#include <cstring>
#include <mutex>
#include <unistd.h>

namespace slemm {

std::atomic<int64_t> g_launches{0};
static thread_local std::string t_last_error;
void set_error(const std::string& msg) { t_last_error = msg; }

void configure_pool(int device)
{
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lock(mu);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  cudaMemPool_t pool;
  CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t keep = UINT64_MAX;   // this process's pool only: freed blocks stay cached for reuse
  CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  done.push_back(device);
}

cudaMemPool_t own_pool(int device, Pool which)
{
  static std::mutex mu;
  static std::map<std::pair<int, int>, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(device, (int)which);
  auto it = pools.find(key);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool;
  CUDA_TRY(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = UINT64_MAX;   // freed blocks stay cached for the next handle or fit
  CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  pools[key] = pool;
  return pool;
}

int num_sms()
{
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// Picks the split-K factor so that M_tiles·splits CTAs fill whole waves, keeping at least
// 16 K-tiles per split and at least min_splits splits.
int choose_splits(int64_t M_tiles, int64_t K_tiles, int ctas_per_sm, int sms, int min_splits)
{
  const int64_t slots = (int64_t)ctas_per_sm * sms;
  int best = 1;
  double best_eff = -1.0;
  for (int s = 1; s <= std::max(16, min_splits); ++s) {
    if (s > 1 && K_tiles / s < 16) break;
    if (s < min_splits) continue;
    const int64_t ctas = M_tiles * s;
    const double waves = (double)ctas / slots;
    const double eff = waves / std::ceil(waves) - 0.015 * (s - 1);   // partials cost per split
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = s;
    }
  }
  return best;
}

// ---- tiled pack -------------------------------------------------------------------------------------
// One CTA turns a block of 128 SNP rows × 512 analysed individuals into the 8 G tiles and 8 GT
// tiles that cover it.  The raw bytes are read from device memory (the caller's rows, or a
// staging buffer the host rows were copied into): row-contiguously (128 bytes per row) when every
// individual is analysed; with a keep list, each thread gathers the 16 codes of one count word
// from one .bed row through the block's 512 .fam positions (staged in shared memory), loading a
// byte only when the position moves to the next one — sorted lists of a few percent to a few tens
// of percent missing read each byte about once.  The codes become 2-bit counts with four bit
// operations per 16 calls, and both copies are written tile-contiguously through shared memory.
constexpr int kPackThreads = 256;

// 16 PLINK codes (code e at bits 2e) → 16 counts in the same positions: count = bit0 + bit1
// (00 → 0, 10 → 1, 11 → 2, missing 01 → 1).
__device__ __forceinline__ uint32_t counts_of_codes(uint32_t w)
{
  const uint32_t lo = w & 0x55555555u, hi = (w >> 1) & 0x55555555u;
  return (lo ^ hi) | ((lo & hi) << 1);
}

// Natural order (field e at bits 2e) → tile word order (even e = 2q at bits 2q, odd e = 2q+1 at
// bits 16+2q): an inverse perfect shuffle of 2-bit units in three exchange steps.
__device__ __forceinline__ uint32_t unshuffle2(uint32_t x)
{
  uint32_t t = (x ^ (x >> 2)) & 0x0C0C0C0Cu;
  x ^= t ^ (t << 2);
  t = (x ^ (x >> 4)) & 0x00F000F0u;
  x ^= t ^ (t << 4);
  t = (x ^ (x >> 8)) & 0x0000FF00u;
  x ^= t ^ (t << 8);
  return x;
}

// raw row j (global SNP index) is at raw + (j − j0)·row_stride; rows j0 … j0 + rows − 1 are present.
// blockIdx.x: SNP group (G M-tile, GT K-tiles 2·sg, 2·sg+1); blockIdx.y: 512-individual group.
// Also adds the block's per-SNP class counts (fields 01 and 10) into c1/c2 ([m_pad] int32 each,
// zeroed beforehand); integer sums, so the totals do not depend on the order of the blocks.
// keep (KEEP only): .fam position of each of the n analysed individuals, < row_bytes·4.
template <bool KEEP>
__global__ void __launch_bounds__(kPackThreads)
pack_tiles_kernel(const uint8_t* __restrict__ raw, int64_t row_stride, int64_t row_bytes, int64_t j0,
                  int64_t rows, int64_t m, int64_t n, int64_t Kt_G, int64_t Mt_T, int64_t Kt_T, bool aligned4,
                  const int32_t* __restrict__ keep, uint32_t* __restrict__ G, uint32_t* __restrict__ GT,
                  int32_t* __restrict__ c1, int32_t* __restrict__ c2)
{
  __shared__ uint32_t cnt[128][33];    // [SNP row][16-individual word], natural order
  __shared__ uint32_t outT[512][9];    // [individual][GT word 0 … 7 (2 K-tiles × 4)]
  __shared__ int32_t sfam[KEEP ? 512 : 1];   // .fam positions of the block's individuals, −1 past n
  const int tid = threadIdx.x;
  const int64_t sg = (int64_t)blockIdx.x + j0 / 128;
  const int64_t ig = blockIdx.y;
  if constexpr (KEEP) {
    for (int t = tid; t < 512; t += kPackThreads) {
      const int64_t i = ig * 512 + t;
      sfam[t] = i < n ? keep[i] : -1;
    }
    __syncthreads();
    // a warp: one SNP row, 32 consecutive count words (512 individuals) — neighbouring bytes
    for (int idx = tid; idx < 128 * 32; idx += kPackThreads) {
      const int r = idx >> 5, q = idx & 31;
      const int64_t j = sg * 128 + r;
      uint32_t w = 0;   // codes in natural order; 00 (count 0) past n
      if (j < m && j - j0 < rows) {
        const uint8_t* p = raw + (j - j0) * row_stride;
        int64_t at = -1;
        uint32_t byte = 0;
#pragma unroll 4
        for (int e = 0; e < 16; ++e) {
          const int32_t f = sfam[16 * q + e];
          if (f < 0) break;
          const int64_t bi = f >> 2;
          if (bi != at) {
            byte = p[bi];
            at = bi;
          }
          w |= ((byte >> (2 * (f & 3))) & 3u) << (2 * e);
        }
      }
      cnt[r][q] = counts_of_codes(w);
    }
  } else {
    for (int idx = tid; idx < 128 * 32; idx += kPackThreads) {
      const int r = idx >> 5, q = idx & 31;
      const int64_t j = sg * 128 + r;
      const int64_t b0 = ig * 128 + 4 * q;
      uint32_t w = 0;
      if (j < m && j - j0 < rows && b0 < row_bytes) {
        const uint8_t* p = raw + (j - j0) * row_stride + b0;
        if (aligned4 && b0 + 4 <= row_bytes) {
          w = *reinterpret_cast<const uint32_t*>(p);
        } else {
          for (int k = 0; k < 4 && b0 + k < row_bytes; ++k) w |= (uint32_t)p[k] << (8 * k);
        }
      }
      const int64_t i0 = 4 * b0;   // first individual of the word
      const uint32_t valid = (i0 + 16 <= n) ? 0xFFFFFFFFu : (i0 >= n ? 0u : ((1u << (2 * (n - i0))) - 1u));
      cnt[r][q] = counts_of_codes(w) & valid;
    }
  }
  __syncthreads();
  if (tid < 128 && sg * 128 + tid < m) {   // the row's 512 individuals: count-1 and count-2 fields
    int ones = 0, twos = 0;
#pragma unroll 8
    for (int q = 0; q < 32; ++q) {
      const uint32_t w = cnt[tid][q];
      ones += __popc(w & 0x55555555u);
      twos += __popc(w & 0xAAAAAAAAu);
    }
    if (ones) atomicAdd(&c1[sg * 128 + tid], ones);
    if (twos) atomicAdd(&c2[sg * 128 + tid], twos);
  }
  // G: tile (sg, 8·ig + t), row r = SNP, words 0 … 3 = local words 4t … 4t+3 of that row
  for (int idx = tid; idx < 8 * 128; idx += kPackThreads) {
    const int t = idx >> 7, r = idx & 127;
    const int64_t kt = ig * 8 + t;
    if (kt >= Kt_G) continue;
    uint4 o;
    o.x = unshuffle2(cnt[r][4 * t]);
    o.y = unshuffle2(cnt[r][4 * t + 1]);
    o.z = unshuffle2(cnt[r][4 * t + 2]);
    o.w = unshuffle2(cnt[r][4 * t + 3]);
    *reinterpret_cast<uint4*>(G + ((sg * Kt_G + kt) * 128 + r) * 4) = o;
  }
  // GT: individuals in quads (one count byte of a word), SNP rows 16·hw … 16·hw + 15
  for (int idx = tid; idx < 128 * 8; idx += kPackThreads) {
    const int iq = idx & 127, hw = idx >> 7;   // quad, GT word (K-tile hw/4, word hw%4)
    uint32_t o0 = 0, o1 = 0, o2 = 0, o3 = 0;
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const uint32_t b = (cnt[16 * hw + e][iq >> 2] >> (8 * (iq & 3))) & 0xFFu;
      o0 |= (b & 3u) << (2 * e);
      o1 |= ((b >> 2) & 3u) << (2 * e);
      o2 |= ((b >> 4) & 3u) << (2 * e);
      o3 |= ((b >> 6) & 3u) << (2 * e);
    }
    outT[4 * iq][hw] = unshuffle2(o0);
    outT[4 * iq + 1][hw] = unshuffle2(o1);
    outT[4 * iq + 2][hw] = unshuffle2(o2);
    outT[4 * iq + 3][hw] = unshuffle2(o3);
  }
  __syncthreads();
  // GT tiles (4·ig + i/128, 2·sg + h), row i % 128, words 4h … 4h+3
  for (int idx = tid; idx < 512 * 2; idx += kPackThreads) {
    const int i = idx & 511, h = idx >> 9;
    const int64_t mt = ig * 4 + (i >> 7), kt = sg * 2 + h;
    if (mt >= Mt_T || kt >= Kt_T) continue;
    uint4 o;
    o.x = outT[i][4 * h];
    o.y = outT[i][4 * h + 1];
    o.z = outT[i][4 * h + 2];
    o.w = outT[i][4 * h + 3];
    *reinterpret_cast<uint4*>(GT + ((mt * Kt_T + kt) * 128 + (i & 127)) * 4) = o;
  }
}

// Per-row integer counts over the G copy: n1 = fields 01, n2 = fields 10, allele count n1 + 2·n2.
__global__ void row_counts_kernel(const uint32_t* __restrict__ G, int64_t m, int64_t K_tiles,
                                  int64_t* __restrict__ pc, int32_t* __restrict__ c1,
                                  int32_t* __restrict__ c2)
{
  // one warp per SNP row
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= m) return;
  const int64_t mt = warp / 128, r = warp % 128;
  long long ones = 0, twos = 0;
  for (int64_t wi = lane; wi < K_tiles * 4; wi += 32) {
    const int64_t kt = wi / 4, wr = wi % 4;
    const uint32_t w = G[((mt * K_tiles + kt) * 128 + r) * 4 + wr];
    ones += __popc(w & 0x55555555u);   // low bit of a field: count 1
    twos += __popc(w & 0xAAAAAAAAu);   // high bit of a field: count 2
  }
  for (int o = 16; o; o >>= 1) {
    ones += __shfl_xor_sync(0xffffffffu, ones, o);
    twos += __shfl_xor_sync(0xffffffffu, twos, o);
  }
  if (lane == 0) {
    pc[warp] = ones + 2 * twos;
    c1[warp] = (int32_t)ones;
    c2[warp] = (int32_t)twos;
  }
}

// The same counts over the kept positions of a trait view only: kmask holds, per K-tile word, the
// low bit of every kept 2-bit field.
__global__ void masked_row_counts_kernel(const uint32_t* __restrict__ G, int64_t m, int64_t K_tiles,
                                         const uint32_t* __restrict__ kmask, int64_t* __restrict__ pc,
                                         int32_t* __restrict__ c1, int32_t* __restrict__ c2)
{
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= m) return;
  const int64_t mt = warp / 128, r = warp % 128;
  long long ones = 0, twos = 0;
  for (int64_t wi = lane; wi < K_tiles * 4; wi += 32) {
    const int64_t kt = wi / 4, wr = wi % 4;
    const uint32_t w = G[((mt * K_tiles + kt) * 128 + r) * 4 + wr];
    const uint32_t mk = kmask[wi];
    ones += __popc(w & mk);
    twos += __popc(w & (mk << 1));
  }
  for (int o = 16; o; o >>= 1) {
    ones += __shfl_xor_sync(0xffffffffu, ones, o);
    twos += __shfl_xor_sync(0xffffffffu, twos, o);
  }
  if (lane == 0) {
    pc[warp] = ones + 2 * twos;
    c1[warp] = (int32_t)ones;
    c2[warp] = (int32_t)twos;
  }
}

}  // namespace slemm

namespace slemm {
__global__ void counts_from_classes_kernel(const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                                           int64_t m, int64_t* __restrict__ pc, int32_t* __restrict__ c1,
                                           int32_t* __restrict__ c2)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  pc[j] = (int64_t)n1[j] + 2 * (int64_t)n2[j];
  c1[j] = n1[j];
  c2[j] = n2[j];
}

void row_counts_device(slemm_geno* g, int64_t* pc, int32_t* c1, int32_t* c2)
{
  const int th = 256;
  if (g->is_view) {   // the view's own individuals
    masked_row_counts_kernel<<<(unsigned)ceil_div(g->m * 32, th), th, 0, g->stream>>>(
        g->G.as<uint32_t>(), g->m, g->n_pad / kTileK, g->kmask.as<uint32_t>(), pc, c1, c2);
  } else if (g->dcounts_valid) {   // summed by the pack kernel
    const int32_t* n1 = g->dcounts.as<int32_t>();
    counts_from_classes_kernel<<<(unsigned)ceil_div(g->m, th), th, 0, g->stream>>>(n1, n1 + g->m_pad, g->m, pc, c1, c2);
  } else {
    row_counts_kernel<<<(unsigned)ceil_div(g->m * 32, th), th, 0, g->stream>>>(g->G.as<uint32_t>(), g->m,
                                                                               g->n_pad / kTileK, pc, c1, c2);
  }
  LAUNCH_CHECK();
}

// Ends the upload pipeline of genotype_create on every path out: waits for the copy stream
// before the staging buffers (declared earlier, so released later) go back to the pool.
// Reads one byte of every host page of [p, p + bytes) (p: the device view of pinned host memory).
// A DMA from pinned memory whose pages the GPU has not translated recently — after a fit has
// streamed tens of GB through the GPU's translation caches, or at first use — runs at ≈25 GB/s
// while it waits on each page's translation in turn, against ≈210 GB/s warm (measured on GB300
// over its C2C link: 7.5 GB of .bed rows took 0.27–0.50 s after a fit, 0.036 s warm).  Many
// threads reading a byte each have all those translations in flight at once: 16 ms for the
// 117,000 64-KB pages of 7.5 GB, after which the copies run warm (0.05 s in all).
__device__ uint32_t g_touch_sink;
__global__ void touch_host_pages_kernel(const uint8_t* __restrict__ p, int64_t bytes, int64_t page)
{
  uint32_t acc = 0;
  for (int64_t o = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * page; o < bytes;
       o += (int64_t)gridDim.x * blockDim.x * page)
    acc += p[o];
  if (acc == 0xFFFFFFFFu) g_touch_sink = acc;   // keeps the loads (a thread's sum stays below 2^32 − 1
                                                // for fewer than 2^24 pages per thread)
}

// Device view of pinned host memory (cudaHostAlloc / cudaHostRegister), or null for any other
// pointer (pageable host memory is not touched from the device).
static const uint8_t* pinned_device_view(const void* host)
{
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? static_cast<const uint8_t*>(at.devicePointer) : nullptr;
}

struct UploadPipe {
  cudaStream_t cs = nullptr;
  cudaEvent_t copied[2] = {nullptr, nullptr}, packed[2] = {nullptr, nullptr}, ready = nullptr;
  void open()
  {
    CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
      CUDA_TRY(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
      CUDA_TRY(cudaEventCreateWithFlags(&packed[b], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  }
  ~UploadPipe()
  {
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t e : {copied[0], copied[1], packed[0], packed[1], ready})
      if (e) cudaEventDestroy(e);
    if (cs) cudaStreamDestroy(cs);
  }
};
}  // namespace slemm

using namespace slemm;

// =================================================================================================
// C ABI
// =================================================================================================
extern "C" {

const char* slemm_gpu_last_error(void) { return t_last_error.c_str(); }
int slemm_gpu_version(void) { return 100; }   // 0.1.0
int64_t slemm_gpu_launch_count(void) { return g_launches.load(); }

int slemm_gpu_init(int device)
{
  return guarded([&] {
    int cnt = 0;
    CUDA_TRY(cudaGetDeviceCount(&cnt));
    CHECK_ARG(device >= 0 && device < cnt, "device index out of range");
    CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp p;
    CUDA_TRY(cudaGetDeviceProperties(&p, device));
    if (!(p.major == 10 && p.minor == 3))
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "this build targets sm_103a; device is sm_" +
                                             std::to_string(p.major) + std::to_string(p.minor));
    configure_pool(device);
  });
}

int slemm_gpu_genotype_create(const uint8_t* bed_rows, int64_t n_fam, int64_t m,
                              int64_t row_stride, const int64_t* keep_idx, int64_t n, int flags,
                              slemm_geno** out)
{
  return guarded([&] {
    CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    CHECK_ARG(bed_rows != nullptr, "bed_rows is null");
    CHECK_ARG(n_fam > 0 && m > 0 && n > 0, "empty genotype matrix");
    const int64_t row_bytes = ceil_div(n_fam, 4);
    CHECK_ARG(row_stride >= row_bytes, "row_stride < ceil(n_fam/4)");
    if (!keep_idx) CHECK_ARG(n == n_fam, "keep_idx is null but n != n_fam");
    CHECK_ARG(n <= n_fam, "n > n_fam");
    CHECK_ARG(n_fam < (int64_t)INT32_MAX && m < (int64_t)INT32_MAX, "dimension exceeds 2^31");
    if (keep_idx)
      for (int64_t i = 0; i < n; ++i)
        CHECK_ARG(keep_idx[i] >= 0 && keep_idx[i] < n_fam, "keep_idx entry out of range");
    CHECK_ARG((flags & ~SLEMM_ROWS_DEVICE) == 0, "unknown flags");
    const bool rows_on_device = (flags & SLEMM_ROWS_DEVICE) != 0;

    auto* g = new slemm_geno();
    try {
      CUDA_TRY(cudaGetDevice(&g->device));
      configure_pool(g->device);
      CUDA_TRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      g->own_stream = true;
      g->bind_stream();
      g->n = n;
      g->m = m;
      // rows padded to 256 so every tensor-core CTA (two 128-row tiles) is full
      g->n_pad = round_up(n, kPadRows);
      g->m_pad = round_up(m, kPadRows);
      const int64_t Kt_G = g->n_pad / kTileK, Kt_GT = g->m_pad / kTileK;
      const size_t bytes_G = (size_t)(g->m_pad / kTileM) * Kt_G * kTileBytes;
      const size_t bytes_GT = (size_t)(g->n_pad / kTileM) * Kt_GT * kTileBytes;
      g->G.pool = g->GT.pool = own_pool(g->device, Pool::Packed);
      g->G.ensure(bytes_G);
      g->GT.ensure(bytes_GT);
      g->err.ensure(sizeof(int));
      CUDA_TRY(cudaMemsetAsync(g->err.p, 0, sizeof(int), g->stream));
      const int64_t Mt_T = g->n_pad / kTileM;
      // kept individuals as 32-bit .fam positions (checked on the host above)
      DevBuf d_keep(g->stream);
      const int32_t* kp = nullptr;
      if (keep_idx) {
        std::vector<int32_t> k32(n);
        for (int64_t i = 0; i < n; ++i) k32[i] = (int32_t)keep_idx[i];
        d_keep.ensure((size_t)n * sizeof(int32_t));
        CUDA_TRY(cudaMemcpyAsync(d_keep.p, k32.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                 g->stream));   // pageable source: copied out before the call returns
        kp = d_keep.as<int32_t>();
      }
      // tiled pack of both copies, padding included, with the per-SNP class counts on the side
      g->dcounts.ensure((size_t)2 * g->m_pad * sizeof(int32_t));
      CUDA_TRY(cudaMemsetAsync(g->dcounts.p, 0, (size_t)2 * g->m_pad * sizeof(int32_t), g->stream));
      int32_t* d_n1 = g->dcounts.as<int32_t>();
      int32_t* d_n2 = d_n1 + g->m_pad;
      const unsigned gy = (unsigned)ceil_div(g->n_pad, 512);
      auto pack = [&](const uint8_t* raw, int64_t stride, int64_t j0, int64_t rows, unsigned gx, bool al) {
        if (kp)
          pack_tiles_kernel<true><<<dim3(gx, gy), kPackThreads, 0, g->stream>>>(
              raw, stride, row_bytes, j0, rows, m, n, Kt_G, Mt_T, Kt_GT, al, kp, g->G.as<uint32_t>(),
              g->GT.as<uint32_t>(), d_n1, d_n2);
        else
          pack_tiles_kernel<false><<<dim3(gx, gy), kPackThreads, 0, g->stream>>>(
              raw, stride, row_bytes, j0, rows, m, n, Kt_G, Mt_T, Kt_GT, al, nullptr, g->G.as<uint32_t>(),
              g->GT.as<uint32_t>(), d_n1, d_n2);
        LAUNCH_CHECK();
      };
      if (rows_on_device) {
        pack(bed_rows, row_stride, 0, m, (unsigned)(g->m_pad / 128),
             ((uintptr_t)bed_rows % 4 == 0) && (row_stride % 4 == 0));
      } else {
        // Host rows: the host link is the bound (≈210 GB/s on GB300's C2C, whether DMA or the
        // kernel reads host memory itself, and the pack kernel's scattered 128-byte reads got
        // only ≈155 GB/s).  So DMA chunks of 4096 rows into two staging buffers on a copy
        // stream while the handle's stream packs the previous chunk from HBM.
        const int64_t chunk = 4096;
        DevBuf raw0(g->stream), raw1(g->stream);
        raw0.ensure((size_t)chunk * row_bytes);
        raw1.ensure((size_t)chunk * row_bytes);
        uint8_t* raw[2] = {raw0.as<uint8_t>(), raw1.as<uint8_t>()};
        UploadPipe pipe;   // destroyed before raw0/raw1: the copy stream is drained first
        pipe.open();
        if (const uint8_t* dv = pinned_device_view(bed_rows)) {   // warm the translations of every page
          const int64_t bytes = (m - 1) * row_stride + row_bytes;
          const long hp = sysconf(_SC_PAGESIZE);
          const int64_t page = std::min<int64_t>(65536, hp > 0 ? hp : 4096);
          const int64_t pages = ceil_div(bytes, page);
          const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(pages, 256), 8 * num_sms()));
          touch_host_pages_kernel<<<blocks, 256, 0, g->stream>>>(dv, bytes, page);
          CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaEventRecord(pipe.ready, g->stream));   // staging allocations, keep list, count zeroing,
                                                             // page touches
        CUDA_TRY(cudaStreamWaitEvent(pipe.cs, pipe.ready, 0));
        const bool al = (row_bytes % 4 == 0);
        int c = 0;
        for (int64_t j0 = 0; j0 < g->m_pad; j0 += chunk, ++c) {
          const int b = c & 1;
          const int64_t rows = std::max<int64_t>(0, std::min(chunk, m - j0));
          if (rows > 0) {
            if (c >= 2) CUDA_TRY(cudaStreamWaitEvent(pipe.cs, pipe.packed[b], 0));   // buffer b is free
            CUDA_TRY(cudaMemcpy2DAsync(raw[b], row_bytes, bed_rows + j0 * row_stride, row_stride, row_bytes, rows,
                                       cudaMemcpyDefault, pipe.cs));
            CUDA_TRY(cudaEventRecord(pipe.copied[b], pipe.cs));
            CUDA_TRY(cudaStreamWaitEvent(g->stream, pipe.copied[b], 0));
          }
          pack(raw[b], row_bytes, j0, rows, (unsigned)(std::min(chunk, g->m_pad - j0) / 128), al);
          CUDA_TRY(cudaEventRecord(pipe.packed[b], g->stream));
        }
      }
      g->dcounts_valid = true;
      CUDA_TRY(cudaStreamSynchronize(g->stream));   // staging buffers and the keep list are released on return
    } catch (...) {
      g->for_each_buf([](DevBuf& b) { b.release(); });
      if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
      delete g;
      throw;
    }
    *out = g;
  });
}

int slemm_gpu_genotype_destroy(slemm_geno* g)
{
  return guarded([&] {
    if (!g) return;
    g->for_each_buf([](DevBuf& b) { b.release(); });   // stream-ordered frees before the stream goes
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    delete g;
  });
}

int slemm_gpu_genotype_view(slemm_geno* parent, const int64_t* keep_idx, int64_t n, slemm_geno** out)
{
  return guarded([&] {
    CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    CHECK_ARG(parent != nullptr && keep_idx != nullptr, "null argument");
    CHECK_ARG(!parent->is_view, "a view of a view is not supported; take the view of the parent");
    CHECK_ARG(n >= 1 && n <= parent->n, "n out of [1, parent's individuals]");
    for (int64_t r = 0; r < n; ++r)
      CHECK_ARG(keep_idx[r] >= 0 && keep_idx[r] < parent->n && (r == 0 || keep_idx[r] > keep_idx[r - 1]),
                "keep_idx must be increasing indices of the parent's individuals");
    CUDA_TRY(cudaSetDevice(parent->device));
    auto* g = new slemm_geno;
    try {
      g->device = parent->device;
      CUDA_TRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      g->own_stream = true;
      g->bind_stream();
      g->is_view = true;
      g->n = n;
      g->m = parent->m;
      g->n_pad = parent->n_pad;
      g->m_pad = parent->m_pad;
      g->prec = parent->prec;
      g->G.alias(parent->G);
      g->GT.alias(parent->GT);
      // the parent's packed copies are complete once its queued work is
      CUDA_TRY(cudaStreamSynchronize(parent->stream));
      const int64_t K_tiles = g->n_pad / kTileK;
      std::vector<int32_t> map(n), inv(g->n_pad, -1);
      std::vector<uint32_t> mask((size_t)K_tiles * 4, 0u);
      for (int64_t r = 0; r < n; ++r) {
        const int64_t i = keep_idx[r];
        map[r] = (int32_t)i;
        inv[i] = (int32_t)r;
        const int64_t e = i % 64, q = e % 16;
        const int sh = (q & 1) ? 16 + (int)(q & ~1) : (int)q;   // bit of the element's 2-bit field
        mask[(size_t)(i / 64) * 4 + e / 16] |= 1u << sh;
      }
      g->ind_map.ensure((size_t)n * sizeof(int32_t));
      g->ind_inv.ensure((size_t)g->n_pad * sizeof(int32_t));
      g->kmask.ensure(mask.size() * sizeof(uint32_t));
      g->err.ensure(sizeof(int));
      CUDA_TRY(cudaMemsetAsync(g->err.p, 0, sizeof(int), g->stream));
      CUDA_TRY(cudaMemcpyAsync(g->ind_map.p, map.data(), map.size() * sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
      CUDA_TRY(cudaMemcpyAsync(g->ind_inv.p, inv.data(), inv.size() * sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
      CUDA_TRY(cudaMemcpyAsync(g->kmask.p, mask.data(), mask.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               g->stream));
      CUDA_TRY(cudaStreamSynchronize(g->stream));   // the host vectors go out of scope
    } catch (...) {
      g->for_each_buf([](DevBuf& b) { b.release(); });
      if (g->stream) cudaStreamSynchronize(g->stream);
      if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
      delete g;
      throw;
    }
    *out = g;
  });
}

int slemm_gpu_genotype_dims(const slemm_geno* g, int64_t* n, int64_t* m)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    if (n) *n = g->n;
    if (m) *m = g->m;
  });
}

int slemm_gpu_set_stream(slemm_geno* g, void* stream)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    if (g->own_stream) cudaStreamDestroy(g->stream);
    if (stream) {
      g->stream = (cudaStream_t)stream;
      g->own_stream = false;
    } else {
      CUDA_TRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      g->own_stream = true;
    }
    g->bind_stream();   // the old stream was synchronised: later frees may run on the new one
  });
}

int slemm_gpu_get_stream(const slemm_geno* g, void** stream)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && stream != nullptr, "null argument");
    *stream = (void*)g->stream;
  });
}

int slemm_gpu_genotype_counts(slemm_geno* g, int64_t* popcnt, int32_t* n0, int32_t* n1,
                              int32_t* n2)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    // exact integer counts of the immutable packed copy: computed on first use, then kept
    if (g->counts_pc.empty()) {
      DevBuf d_pc(g->stream), d_c1(g->stream), d_c2(g->stream);
      d_pc.ensure(g->m * sizeof(int64_t));
      d_c1.ensure(g->m * sizeof(int32_t));
      d_c2.ensure(g->m * sizeof(int32_t));
      row_counts_device(g, d_pc.as<int64_t>(), d_c1.as<int32_t>(), d_c2.as<int32_t>());
      std::vector<int64_t> hpc(g->m);
      std::vector<int32_t> hc1(g->m), hc2(g->m);
      CUDA_TRY(cudaMemcpyAsync(hpc.data(), d_pc.p, g->m * sizeof(int64_t), cudaMemcpyDeviceToHost, g->stream));
      CUDA_TRY(cudaMemcpyAsync(hc1.data(), d_c1.p, g->m * sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
      CUDA_TRY(cudaMemcpyAsync(hc2.data(), d_c2.p, g->m * sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
      CUDA_TRY(cudaStreamSynchronize(g->stream));
      g->counts_pc = std::move(hpc);
      g->counts_c1 = std::move(hc1);
      g->counts_c2 = std::move(hc2);
    }
    const std::vector<int64_t>& pc = g->counts_pc;
    const std::vector<int32_t>& c1 = g->counts_c1;
    const std::vector<int32_t>& c2 = g->counts_c2;
    for (int64_t j = 0; j < g->m; ++j) {
      if (popcnt) popcnt[j] = pc[j];
      if (n1) n1[j] = c1[j];
      if (n2) n2[j] = c2[j];
      if (n0) n0[j] = (int32_t)(g->n - c1[j] - c2[j]);
    }
  });
}

int slemm_gpu_set_weights(slemm_geno* g, const float* gm, const float* w, const float* rr)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && gm != nullptr && w != nullptr, "null argument");
    std::vector<float> hgm(g->m_pad, 0.f), hw(g->m_pad, 0.f), hrr(g->n_pad, 0.f);
    for (int64_t j = 0; j < g->m; ++j) {
      CHECK_ARG(std::isfinite(gm[j]) && std::isfinite(w[j]), "non-finite gm or w");
      hgm[j] = gm[j];
      hw[j] = w[j];
    }
    for (int64_t i = 0; i < g->n; ++i) {
      hrr[i] = rr ? rr[i] : 1.0f;
      CHECK_ARG(std::isfinite(hrr[i]), "non-finite rr");
    }
    // Z_cᵀ1 = Σ_i (x_ij − gm_j) = pc_j − n·gm_j, from the exact integer popcounts
    std::vector<int64_t> pc(g->m);
    {
      const int st = slemm_gpu_genotype_counts(g, pc.data(), nullptr, nullptr, nullptr);
      if (st != SLEMM_OK) SLEMM_THROW(st, "genotype counts failed");
    }
    std::vector<float> hcorr(g->m_pad, 0.f);
    for (int64_t j = 0; j < g->m; ++j) hcorr[j] = (float)((double)pc[j] - (double)g->n * (double)gm[j]);
    g->gm.ensure(g->m_pad * sizeof(float));
    g->w.ensure(g->m_pad * sizeof(float));
    g->rr.ensure(g->n_pad * sizeof(float));
    g->gcorr.ensure(g->m_pad * sizeof(float));
    CUDA_TRY(cudaMemcpyAsync(g->gcorr.p, hcorr.data(), g->m_pad * sizeof(float), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaMemcpyAsync(g->gm.p, hgm.data(), g->m_pad * sizeof(float), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaMemcpyAsync(g->w.p, hw.data(), g->m_pad * sizeof(float), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaMemcpyAsync(g->rr.p, hrr.data(), g->n_pad * sizeof(float), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    g->weights_set = true;
  });
}

int slemm_gpu_set_projection(slemm_geno* g, const float* Q, int64_t ldq, int c)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    CHECK_ARG(c >= 0 && c <= SLEMM_MAX_COVARIATES, "projection rank must be in [0, SLEMM_MAX_COVARIATES]");
    g->c = c;
    if (c == 0) return;
    CHECK_ARG(Q != nullptr && ldq >= g->n, "bad Q");
    std::vector<float> hq((size_t)g->n_pad * c, 0.f);
    for (int l = 0; l < c; ++l)
      for (int64_t i = 0; i < g->n; ++i) hq[(size_t)l * g->n_pad + i] = Q[(size_t)l * ldq + i];
    g->Q.ensure(hq.size() * sizeof(float));
    CUDA_TRY(cudaMemcpyAsync(g->Q.p, hq.data(), hq.size() * sizeof(float), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
  });
}

int slemm_gpu_set_precision(slemm_geno* g, int prec)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    CHECK_ARG(prec == SLEMM_PREC_FP32 || prec == SLEMM_PREC_BF16X2 || prec == SLEMM_PREC_BF16X3 ||
                  prec == SLEMM_PREC_FP16X2,
              "unknown precision");
    g->prec = prec;
  });
}

int slemm_gpu_set_per_vector(slemm_geno* g, int per_vector)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    g->per_vector = per_vector ? 1 : 0;
  });
}

int slemm_gpu_set_lanczos(slemm_geno* g, int mode)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    CHECK_ARG((mode & ~SLEMM_LANCZOS_REORTH) == 0, "unknown Lanczos mode bits");
    g->lanczos_mode = mode;
  });
}

}  // extern "C"
