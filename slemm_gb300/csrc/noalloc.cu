// noalloc.cu — Z_cᵀ·v for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc while they use this library: a host framework may already
// have reserved nearly all of the GPU's memory for its own pool, or the caller may run a
// latency-critical loop in which cudaMalloc/cudaFree (which can synchronise the whole device) are
// not allowed.  slemm_gpu_rmatvec_noalloc serves them: it computes the same product as
// slemm_gpu_op(SLEMM_OP_RMATVEC) on the FP32 CUDA-core path, but takes its scratch (the padded
// dense operand, the split-K partial products and the column-sum partials) from one file-scope
// device array of fixed size instead of allocating.
//
// Rules for callers:
//   * The array holds SLEMM_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads this library,
//     for as long as the library stays loaded.
//   * A call whose scratch would exceed that size is rejected with SLEMM_ERR_UNSUPPORTED and a
//     message giving the bytes it would need; nothing is launched.
//   * The first call on each device looks up the array's device address (cudaGetSymbolAddress)
//     with that device current; make that first call before any stream capture.  The call makes
//     the handle's device current for its duration (the caller's current device is restored),
//     so a caller with another device current still gets the handle's GPU and its array.  The
//     address is cached for the life of the process: a caller that resets the device
//     (cudaDeviceReset) must not use this entry point afterwards.
//   * All calls on a device share the one array and each call overwrites what it uses (nothing
//     has to be cleared between calls).  Calls whose GPU work overlaps — on different streams or
//     different handles at the same time — race on the array; order them on one stream.
//   * v and out are device pointers; the work is queued on the handle's stream and the call
//     returns without synchronising.
#include "internal.h"
#include "reduce.cuh"

#include <mutex>

namespace slemm {

constexpr size_t kNoAllocBytes = SLEMM_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNaRows = 4096;     // rows per block of the row-wise kernels
constexpr int kMaxDevices = 64;
static void* s_scratch[kMaxDevices] = {};
static std::mutex s_scratch_mu;

// Makes `dev` the calling thread's current device for the scope and restores the caller's after.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev)
  {
    CUDA_TRY(cudaGetDevice(&prev));
    if (prev != dev) CUDA_TRY(cudaSetDevice(dev));
  }
  ~DeviceScope()
  {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Device address of the static scratch array on device `dev`, which must be current (looked up
// once per device; the cache assumes the device's context lives as long as the process).
static void* scratch_on_device(int dev)
{
  if (dev < 0 || dev >= kMaxDevices) SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "device index beyond 64");
  std::lock_guard<std::mutex> lk(s_scratch_mu);
  if (!s_scratch[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      SLEMM_THROW(SLEMM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) -> ") + cudaGetErrorString(e));
    s_scratch[dev] = p;
  }
  return s_scratch[dev];
}

// The column mean the operand has removed: μ_c = (float)(Σ_i v[i,c] / n).
__device__ __forceinline__ float na_mean(const double* __restrict__ mu_sum, int c, int64_t n)
{
  return (float)(mu_sum[c] * (1.0 / (double)n));
}

// B[c][i] = v[i,c] − μ_c for i < n, 0 for n ≤ i < n_pad; red[c][blk] = Σ_i B[c][i] (double-float per thread, FP64 per block).
// With B == nullptr only the sums of v are taken (μ_c's pass); mu_sum == nullptr: μ_c = 0.
__global__ void na_prologue_kernel(const float* __restrict__ v, int64_t ldv, int64_t n, int64_t n_pad,
                                   float* __restrict__ B, double* __restrict__ red, int nblk,
                                   const double* __restrict__ mu_sum)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kNaRows, i1 = min64(n_pad, i0 + kNaRows);
  const float mu = mu_sum ? na_mean(mu_sum, c, n) : 0.f;
  DF sum;   // double-float: FP32 operations per element, FP64 once per thread
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const float x = (i < n) ? __fsub_rn(v[(int64_t)c * ldv + i], mu) : 0.f;
    if (B) B[(int64_t)c * n_pad + i] = x;
    df_add(sum, x);
  }
  double acc = df_value(sum);
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    red[(int64_t)c * nblk + blockIdx.x] = s;
  }
}

// colsum[c] = Σ_blk red[c][blk] in a fixed order.
__global__ void na_colsum_kernel(const double* __restrict__ red, int nblk, int k, double* __restrict__ colsum)
{
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= k) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += red[(int64_t)c * nblk + b];
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) colsum[c] = s;
}

// out[j,c] = Σ_s D[s][c][j] − gm_j·colsum_c + μ_c·(pc_j − n·gm_j)   (j < m): the mean the
// operand removed comes back exactly through Z_cᵀ1 = pc − n·gm (see ops.cu).
__global__ void na_finalize_kernel(const float* __restrict__ D, int splits, int k, int64_t m_pad, int64_t m,
                                   const float* __restrict__ gm, const double* __restrict__ colsum,
                                   const double* __restrict__ mu_sum, const float* __restrict__ gcorr, int64_t n,
                                   float* __restrict__ out, int64_t ldo)
{
  __shared__ float sc[3];   // colsum_c as a hi+lo FP32 pair, μ_c
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (threadIdx.x == 0) {
    split_double(colsum[c], sc[0], sc[1]);
    sc[2] = mu_sum ? na_mean(mu_sum, c, n) : 0.f;
  }
  __syncthreads();
  if (j >= m) return;
  float raw = 0.f;
  for (int s = 0; s < splits; ++s) raw += D[((int64_t)s * k + c) * m_pad + j];
  const float g = gm[j];
  float val = __fmaf_rn(-g, sc[1], __fmaf_rn(-g, sc[0], raw));
  if (mu_sum) val = __fmaf_rn(sc[2], gcorr[j], val);
  out[(int64_t)c * ldo + j] = val;
}

struct NaLayout {
  size_t b_off, d_off, red_off, cs_off, mu_off, total;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static NaLayout na_layout(int64_t n_pad, int64_t m_pad, int k, int splits, int nblk)
{
  NaLayout L;
  L.b_off = 0;
  L.d_off = align256(L.b_off + (size_t)k * n_pad * sizeof(float));
  L.red_off = align256(L.d_off + (size_t)splits * k * m_pad * sizeof(float));
  L.cs_off = align256(L.red_off + (size_t)nblk * k * sizeof(double));
  L.mu_off = align256(L.cs_off + (size_t)k * sizeof(double));
  L.total = L.mu_off + (size_t)k * sizeof(double);
  return L;
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_rmatvec_noalloc(slemm_geno* g, const float* v, int64_t ldv, int k, float* out,
                                         int64_t ldo)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && v != nullptr && out != nullptr, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_rmatvec_noalloc reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    CHECK_ARG(k >= 1, "k must be >= 1");
    CHECK_ARG(ldv >= g->n && ldo >= g->m, "leading dimension too small");
    if (!g->weights_set) SLEMM_THROW(SLEMM_ERR_STATE, "set_weights must be called before operators");
    const int64_t M_tiles = g->m_pad / kTileM, K_tiles = g->n_pad / kTileK;
    const int nblk = (int)ceil_div(g->n_pad, kNaRows);
    int splits = choose_splits(M_tiles, K_tiles, 8, num_sms());
    NaLayout L = na_layout(g->n_pad, g->m_pad, k, splits, nblk);
    while (L.total > kNoAllocBytes && splits > 1) L = na_layout(g->n_pad, g->m_pad, k, --splits, nblk);
    if (L.total > kNoAllocBytes)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED,
                  "rmatvec_noalloc needs " + std::to_string(L.total) + " bytes of scratch for n=" +
                      std::to_string(g->n) + ", m=" + std::to_string(g->m) + ", k=" + std::to_string(k) +
                      "; the static scratch holds " + std::to_string(kNoAllocBytes) + " bytes");
    // The handle's stream belongs to the handle's device: its scratch address and every launch
    // below are taken with that device current, whichever device the caller has current.
    DeviceScope on_device(g->device);
    uint8_t* base = static_cast<uint8_t*>(scratch_on_device(g->device));
    float* B = reinterpret_cast<float*>(base + L.b_off);
    float* D = reinterpret_cast<float*>(base + L.d_off);
    double* red = reinterpret_cast<double*>(base + L.red_off);
    double* colsum = reinterpret_cast<double*>(base + L.cs_off);
    const float* gcorr = g->gcorr.as<float>();
    double* mu_sum = gcorr ? reinterpret_cast<double*>(base + L.mu_off) : nullptr;
    cudaStream_t st = g->stream;
    if (mu_sum) {   // column means first: they are removed from the operand and added back exactly
      na_prologue_kernel<<<dim3(nblk, k), 256, 0, st>>>(v, ldv, g->n, g->n_pad, nullptr, red, nblk, nullptr);
      LAUNCH_CHECK();
      na_colsum_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, st>>>(red, nblk, k, mu_sum);
      LAUNCH_CHECK();
    }
    na_prologue_kernel<<<dim3(nblk, k), 256, 0, st>>>(v, ldv, g->n, g->n_pad, B, red, nblk, mu_sum);
    LAUNCH_CHECK();
    na_colsum_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, st>>>(red, nblk, k, colsum);
    LAUNCH_CHECK();
    GemmArgs a{g->G.as<uint8_t>(), g->m_pad, g->n_pad, B, k, D, splits, nullptr};
    gemm_simt(a, st);
    na_finalize_kernel<<<dim3((unsigned)ceil_div(g->m, 256), k), 256, 0, st>>>(
        D, splits, k, g->m_pad, g->m, g->gm.as<float>(), colsum, mu_sum, gcorr, g->n, out, ldo);
    LAUNCH_CHECK();
  });
}
