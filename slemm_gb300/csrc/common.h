// common.h — shared internals of libslemm_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <atomic>

#include "../../include/slemm_gpu.h"

namespace slemm {

// ---- errors --------------------------------------------------------------------------------
void set_error(const std::string& msg);
struct Error {
  int code;
  std::string msg;
};

#define SLEMM_THROW(code_, msg_)                                      \
  do {                                                                \
    throw ::slemm::Error{(code_), std::string(__func__) + ": " + (msg_)}; \
  } while (0)

#define CUDA_TRY(expr)                                                              \
  do {                                                                              \
    cudaError_t e__ = (expr);                                                       \
    if (e__ != cudaSuccess)                                                         \
      throw ::slemm::Error{SLEMM_ERR_CUDA, std::string(#expr) + " -> " +            \
                                               cudaGetErrorString(e__)};           \
  } while (0)

#define CHECK_ARG(cond, msg_) \
  do {                        \
    if (!(cond)) SLEMM_THROW(SLEMM_ERR_ARG, msg_); \
  } while (0)

// Wraps a C-ABI body: maps exceptions to status codes and the thread-local message.
template <class F>
int guarded(F&& f)
{
  try {
    f();
    return SLEMM_OK;
  } catch (const Error& e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return SLEMM_ERR_NOMEM;
  } catch (const std::exception& e) {
    set_error(e.what());
    return SLEMM_ERR_STATE;
  }
}

// ---- launch accounting -----------------------------------------------------------------------
extern std::atomic<int64_t> g_launches;
inline void count_launch(int k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }
// Checks the launch just issued.
#define LAUNCH_CHECK()                                   \
  do {                                                   \
    ::slemm::count_launch();                             \
    CUDA_TRY(cudaGetLastError());                        \
  } while (0)

// ---- sizes -----------------------------------------------------------------------------------
constexpr int kTileM = 128;          // rows of one packed tile (M of one MMA)
constexpr int kTileK = 64;           // K elements of one packed tile (one 128-B bf16 row)
constexpr int kTileBytes = kTileM * kTileK / 4;   // 2048 packed bytes per tile
constexpr int kPadRows = 256;        // n and m are padded to this (two row tiles per TC CTA)
__host__ __device__ inline int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
__host__ __device__ inline int64_t ceil_div(int64_t x, int64_t a) { return (x + a - 1) / a; }

// ---- device buffer -----------------------------------------------------------------------------
// Plain buffers use cudaMalloc/cudaFree.  A buffer bound to a stream (DevBuf(stream)) is
// allocated and freed stream-ordered from the device's default memory pool, whose release
// threshold configure_pool raises so that freed blocks stay cached for the next fit: such
// allocations cost no device synchronisation.  Buffers that set `pool` draw from that pool
// instead (the packed copies and the Lanczos basis have their own, so that each reuses its own
// freed blocks instead of competing with every other allocation for the default pool's).  A
// stream-bound buffer must be released before its stream is destroyed.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  bool ordered = false;
  bool owned = true;   // false: p aliases another buffer (a trait view's packed copies), never freed here
  cudaMemPool_t pool = nullptr;   // stream-ordered from this pool instead of the default one
  DevBuf() = default;
  explicit DevBuf(cudaStream_t s) : stream(s), ordered(true) {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release()
  {
    if (p && owned) {
      if (ordered) cudaFreeAsync(p, stream);
      else cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    owned = true;
  }
  // Points at `other`'s memory without owning it.
  void alias(const DevBuf& other)
  {
    release();
    p = other.p;
    bytes = other.bytes;
    owned = false;
  }
  // Grows (never shrinks); contents are not preserved.
  void* ensure(size_t nbytes)
  {
    if (nbytes <= bytes) return p;
    release();
    if (nbytes == 0) return nullptr;
    cudaError_t e = !ordered ? cudaMalloc(&p, nbytes)
                    : pool ? cudaMallocFromPoolAsync(&p, nbytes, pool, stream)
                           : cudaMallocAsync(&p, nbytes, stream);
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error{SLEMM_ERR_NOMEM, std::string(ordered ? "cudaMallocAsync(" : "cudaMalloc(") +
                                       std::to_string(nbytes) + ") -> " + cudaGetErrorString(e)};
    }
    bytes = nbytes;
    return p;
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};
// Small page-locked host array mapped into the device address space: kernels write scalars that
// the host reads after a stream synchronisation, without a separate copy.
struct HostScal {
  double* h = nullptr;   // host view
  double* d = nullptr;   // device view
  size_t count = 0;
  HostScal() = default;
  HostScal(const HostScal&) = delete;
  HostScal& operator=(const HostScal&) = delete;
  ~HostScal()
  {
    if (h) cudaFreeHost(h);
  }
  double* ensure(size_t n)
  {
    if (n <= count) return d;
    if (h) cudaFreeHost(h);
    h = d = nullptr;
    count = 0;
    cudaError_t e = cudaHostAlloc((void**)&h, n * sizeof(double), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&d, h, 0);
    if (e != cudaSuccess) {
      if (h) cudaFreeHost(h);
      h = d = nullptr;
      throw Error{SLEMM_ERR_NOMEM, std::string("cudaHostAlloc -> ") + cudaGetErrorString(e)};
    }
    count = n;
    return d;
  }
};

// Keeps freed stream-ordered blocks of the device's default pool cached (idempotent).
void configure_pool(int device);
// The device's pools for the packed genotype copies and for the Lanczos basis (created on first
// use, freed blocks kept cached like the default pool's).
enum class Pool { Packed = 0, Basis = 1 };
cudaMemPool_t own_pool(int device, Pool which);

// ---- packed product plan ------------------------------------------------------------------------
// D[M_pad × N] = Cnt[M_pad × K_pad] · B where the count matrix is a tiled 2-bit packed array
// (tiles of kTileM rows × kTileK K-elements, 2048 contiguous bytes each, see geno.cu) and B is
// either FP32 [k][K_pad] (SIMT) or 16-bit pieces [N][K_pad] (tensor cores: piece p of column c
// in row p·kp + c, kp = k rounded up to 8, BF16 or FP16).  The raw product goes to partials
// [splits][kp][M_pad] (FP32; the tensor-core epilogue adds a column's pieces before the store),
// reduced by the finalize kernels of ops.cu.
struct GemmArgs {
  const uint8_t* A;     // tiled packed counts
  int64_t M_pad;        // rows (multiple of 128)
  int64_t K_pad;        // K elements (multiple of 128)
  const void* B;        // dense side
  int N;                // columns of the product (k for SIMT, padded pieces·kp for TC)
  float* D;             // partials
  int splits;           // split-K factor
  int* err;             // device error word (bounded waits that gave up set bits here)
  int kp = 0;           // columns of D per split (TC: k rounded up to 8; SIMT: N)
  int pieces = 1;       // pieces per column (TC)
  bool f16 = false;     // TC operand type: FP16 (true) or BF16
  int plan = 0;         // TC ring plan: 0 by N (N ≤ 64: two tiles per CTA, one CTA per SM), 1: N ≤ 64,
                        // one tile per CTA and two CTAs per SM (256 TMEM columns each)
};

void gemm_simt(const GemmArgs& a, cudaStream_t st);
// Tensor-core path (tcgen05); N must be a multiple of 16 in [16, 256].
void gemm_tc(const GemmArgs& a, cudaStream_t st);
int choose_splits(int64_t M_tiles, int64_t K_tiles, int ctas_per_sm, int num_sms, int min_splits = 1);
// Rows one tensor-core CTA covers for this N and plan (128 or 256).
int gemm_tc_rows_per_cta(int N, int plan);
int num_sms();

}  // namespace slemm
