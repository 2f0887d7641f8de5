// ops.cu — operator applications built on the packed products (src/reml.cpp:8-233).
//
// Centring is an exact rank-1 correction: with x the allele count and gm_j its mean,
//   Z_cᵀu  = Cntᵀu − gm·(1ᵀu)          (direction 1, K = individuals, M = SNPs)
//   Z_c v  = Cnt v − 1·(gmᵀv)           (direction 2, K = SNPs, M = individuals)
// where Cnt holds the exact integer counts.  The dense side is prepared once per pass by a
// prologue (projection, rr scaling, FP32 → BF16 or FP16 pieces) that also sums exactly what the
// tensor cores multiply, in FP64, for the correction term.  Direction 1 first removes each
// column's mean μ and adds it back exactly: Z_cᵀu = Z_cᵀ(u − μ1) + μ·(pc − n·gm), with pc the
// integer popcounts.  Without it a column with a large mean (the intercept column of a Lanczos
// block) leaves Cntᵀu and gm·(1ᵀu) nearly equal and large, and their FP32 accumulation error
// swamps the true difference: at n = 10⁶ the intercept's Lanczos recurrence never converged.  Finalize kernels reduce the split-K
// partials, apply the correction and the reference's diagonal scalings,
// and either write the result or directly build the next pass's dense operand.
//
// All reductions are two-stage (per-block FP64 partials, then a fixed-order sum), so results
// are bit-reproducible run to run.
#include "internal.h"
#include "reduce.cuh"
#include "decode.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <map>
#include <mutex>

namespace slemm {

constexpr int kRedThreads = 256;
static_assert(SLEMM_MAX_COVARIATES <= kRedThreads, "load_qt gives one covariate per thread");
constexpr int kRowsPerBlock = 4096;   // rows handled by one block of the row-wise kernels

// 4-wide accesses need rows % 4 == 0 (a vector never straddles the end), ld % 4 == 0 and a
// 16-byte aligned base.
static bool vec4_ok(int64_t rows, int64_t ld, const void* p)
{
  return rows % 4 == 0 && ld % 4 == 0 && ((uintptr_t)p & 15u) == 0;
}

// out[q] = Σ_b red[q][b] in block order
__global__ void reduce_partials_kernel(const double* __restrict__ red, int nblk, int nq,
                                       double* __restrict__ out)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) out[q] = sum_partials(red + (int64_t)q * nblk, nblk);
}

static void reduce_partials(const double* red, int nblk, int nq, double* out, cudaStream_t st)
{
  reduce_partials_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, st>>>(red, nblk, nq, out);
  LAUNCH_CHECK();
}

// ---- projections ---------------------------------------------------------------------------------
// red[(l*k + c)][blk] = Σ_{i in block} Q[i,l]·X[i,c]; grid (c·k, row blocks): c·k reaches
// 256 × 269 for the largest covariate count, beyond the 65,535 of a grid's y dimension.
template <int V>
__global__ void __launch_bounds__(kRedThreads)
proj_partial_kernel(const float* __restrict__ Q, int64_t ldq, const float* __restrict__ X, int64_t ldx,
                    int64_t n, int k, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.x % k, l = blockIdx.x / k;
  const int64_t i0 = (int64_t)blockIdx.y * kRowsPerBlock, i1 = min64(n, i0 + kRowsPerBlock);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kRedThreads * V) {
    float q[V], x[V];
    ldv<V>(Q + (int64_t)l * ldq + i, q);
    ldv<V>(X + (int64_t)c * ldx + i, x);
#pragma unroll
    for (int u = 0; u < V; ++u) df_fma(acc, q[u], x[u]);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)(l * k + c) * nblk + blockIdx.y] = s;
}

// qt[l] = QᵀX[l, c] from its partials (nblk = 1: final values), l < cq ≤ SLEMM_MAX_COVARIATES,
// as hi+lo FP32 pairs; warp w of the block reduces the covariates l ≡ w (mod warps).
__device__ __forceinline__ void load_qt(const double* __restrict__ parts, int nblk, int cq, int k, int c, float2* qt)
{
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int l = warp; l < cq; l += nw) {
    const double v = warp_sum_partials(parts + (int64_t)(l * k + c) * nblk, nblk);
    if ((threadIdx.x & 31) == 0) {
      float h, lo;
      split_double(v, h, lo);
      qt[l] = make_float2(h, lo);
    }
  }
  __syncthreads();
}

// Σ_l Q[i,l]·qt_l rounded once to FP32.  The products (TwoProd by FMA, plus the low coefficient
// word) and their sum are carried as a double-float pair, so the value is the FP64 one to about
// 2⁻⁴⁴ before the final rounding, at FP32 rates: GB300's FP64 pipe would otherwise bound the
// row-wise kernels that project every element.
__device__ __forceinline__ float proj_dot(const float* __restrict__ Q, int64_t ldq, int cq, int64_t i,
                                          const float2* qt)
{
  DF a;
  for (int l = 0; l < cq; ++l) {
    const float q = Q[(int64_t)l * ldq + i];
    df_fma(a, q, qt[l].x);
    a.lo = __fmaf_rn(q, qt[l].y, a.lo);
  }
  return __fadd_rn(a.hi, a.lo);
}

// X[i,c] −= Σ_l Q[i,l]·QtX[l,c] (+ tau0·Vin[i,c] when Vin != nullptr)
template <int V>
__global__ void __launch_bounds__(kRedThreads)
proj_apply_kernel(const float* __restrict__ Q, int64_t ldq, int cq, float* __restrict__ X, int64_t ldx,
                  int64_t n, int k, const double* __restrict__ qparts, int nblkq,
                  const float* __restrict__ Vin, int64_t ld_v, float tau0)
{
  __shared__ float2 qt[SLEMM_MAX_COVARIATES];
  const int c = blockIdx.y;
  load_qt(qparts, nblkq, cq, k, c, qt);
  const int64_t i = ((int64_t)blockIdx.x * kRedThreads + threadIdx.x) * V;
  if (i >= n) return;
  float x[V];
  ldv<V>(X + (int64_t)c * ldx + i, x);
#pragma unroll
  for (int u = 0; u < V; ++u) {
    x[u] = __fsub_rn(x[u], proj_dot(Q, ldq, cq, i + u, qt));
    if (Vin) x[u] = __fmaf_rn(tau0, Vin[(int64_t)c * ld_v + i + u], x[u]);
  }
  stv<V>(X + (int64_t)c * ldx + i, x);
}

template <int V>
static void launch_proj_partial(slemm_geno* g, const float* X, int64_t ldx, int k, double* red, int nblk)
{
  proj_partial_kernel<V><<<dim3(g->c * k, nblk), kRedThreads, 0, g->stream>>>(g->Q.as<float>(), g->n_pad, X, ldx,
                                                                               g->n, k, red, nblk);
  LAUNCH_CHECK();
}

static void proj_partials(slemm_geno* g, const float* X, int64_t ldx, int k, double* red, int nblk)
{
  if (vec4_ok(g->n, ldx, X)) launch_proj_partial<4>(g, X, ldx, k, red, nblk);
  else launch_proj_partial<1>(g, X, ldx, k, red, nblk);
}

static void proj_apply_parts(slemm_geno* g, float* X, int64_t ldx, int k, const double* qparts, int nblkq,
                             const float* Vin, int64_t ld_v, float tau0)
{
  const bool v4 = vec4_ok(g->n, ldx, X) && (!Vin || vec4_ok(g->n, ld_v, Vin));
  if (v4) {
    dim3 grid((unsigned)ceil_div(g->n, 4 * kRedThreads), k);
    proj_apply_kernel<4><<<grid, kRedThreads, 0, g->stream>>>(g->Q.as<float>(), g->n_pad, g->c, X, ldx, g->n, k,
                                                              qparts, nblkq, Vin, ld_v, tau0);
  } else {
    dim3 grid((unsigned)ceil_div(g->n, kRedThreads), k);
    proj_apply_kernel<1><<<grid, kRedThreads, 0, g->stream>>>(g->Q.as<float>(), g->n_pad, g->c, X, ldx, g->n, k,
                                                              qparts, nblkq, Vin, ld_v, tau0);
  }
  LAUNCH_CHECK();
}

void proj_coeffs(slemm_geno* g, const float* X, int64_t ldx, int k, double* d_QtX)
{
  if (g->c == 0) return;
  CHECK_ARG(g->c <= SLEMM_MAX_COVARIATES, "too many covariates");
  const int nblk = (int)ceil_div(g->n, kRowsPerBlock);
  double* red = (double*)g->ws_red.ensure((size_t)nblk * g->c * k * sizeof(double));
  proj_partials(g, X, ldx, k, red, nblk);
  reduce_partials(red, nblk, g->c * k, d_QtX, g->stream);
}

void proj_apply(slemm_geno* g, float* X, int64_t ldx, int k, const double* d_QtX)
{
  if (g->c == 0) return;
  proj_apply_parts(g, X, ldx, k, d_QtX, 1, nullptr, 0, 0.f);
}

// ---- column dots ------------------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__(kRedThreads)
col_dots_partial_kernel(const float* __restrict__ a, int64_t lda, const float* __restrict__ b, int64_t ldb,
                        int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kRowsPerBlock, i1 = min64(n, i0 + kRowsPerBlock);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kRedThreads * V) {
    float x[V], y[V];
    ldv<V>(a + (int64_t)c * lda + i, x);
    if (b) ldv<V>(b + (int64_t)c * ldb + i, y);
#pragma unroll
    for (int u = 0; u < V; ++u) df_fma(acc, x[u], b ? y[u] : x[u]);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

void col_dots(slemm_geno* g, const float* a, int64_t lda, const float* b, int64_t ldb, int64_t n,
              int k, double* d_out)
{
  const int nblk = (int)ceil_div(n, kRowsPerBlock);
  double* red = (double*)g->ws_red.ensure((size_t)nblk * k * sizeof(double));
  dim3 grid(nblk, k);
  if (vec4_ok(n, lda, a) && (!b || vec4_ok(n, ldb, b)))
    col_dots_partial_kernel<4><<<grid, kRedThreads, 0, g->stream>>>(a, lda, b, ldb, n, red, nblk);
  else
    col_dots_partial_kernel<1><<<grid, kRedThreads, 0, g->stream>>>(a, lda, b, ldb, n, red, nblk);
  LAUNCH_CHECK();
  reduce_partials(red, nblk, k, d_out, g->stream);
}

// ---- dense-operand builders ------------------------------------------------------------------------
// FP16 pieces (SLEMM_PREC_FP16X2) are a fixed-point split: the operand column is scaled by a power
// of two 2^e, chosen from a bound on |x| so that the largest value lies in [2^10, 2^11); the hi
// piece is rint(x·2^e), an integer of at most 11 bits (exact in FP16), and the lo piece is the
// FP16 rounding of the remainder (|lo| ≤ 1/2).  Products count·hi are integers below 2^12, so the
// tensor cores' FP32 accumulation of the hi pieces is exact while a partial sum stays below 2^24
// (a random-sign sum over 10^6 individuals reaches ~2^18), and the lo pieces carry 2^−11 of the
// magnitude: the accumulation error that bounds the BF16 and CUDA-core FP32 paths at long K
// (≈4e-6 relative over 500,000 individuals) falls away and what remains is the lo piece's
// rounding, ≤ 2^−23 of the column's largest value.  The products are scaled back by 2^−e
// (exact).  BF16 shares FP32's exponent range and needs no scale.
__device__ __forceinline__ int f16_exp(double bound)
{
  if (!(bound > 0.0) || !isfinite(bound)) return 0;
  int E;
  frexp(bound, &E);                       // bound = f·2^E, f ∈ [0.5, 1)
  return max(-120, min(120, 11 - E));     // bound·2^e ∈ [2^10, 2^11)
}

// max_b parts[c·nblk + b] by the 32 lanes of the calling warp (0 for no partials)
__device__ __forceinline__ double max_partials(const double* __restrict__ parts, int nblk, int c)
{
  return warp_max_partials(parts + (int64_t)c * nblk, nblk);
}

// Block maximum of one float per thread (valid in thread 0; −∞ when every thread holds −∞);
// sh holds ≥ 32 floats.
__device__ __forceinline__ float block_max_f(float v, float* sh)
{
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  float r = -INFINITY;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmaxf(r, sh[i]);
  return r;
}

// Scale exponent of individual-side operand column c whose stored values are x − μ: from the
// measure pass's signed block extremes range[(c·nblk + b)·2 + {0, 1}] = {max x, max −x} over the
// valid rows, the bound max(max x − μ, μ − min x) ≥ |x − μ|.  A column with a large mean keeps
// the resolution of its spread.  The prologue and the finalize take the same e from this.
__device__ __forceinline__ int f16_col_exp(const double* __restrict__ range, int nblk, int c, float mu)
{
  // by the 32 lanes of the calling warp
  const double hi = warp_max_partials(range + (int64_t)c * nblk * 2, nblk, 2, -INFINITY);
  const double nlo = warp_max_partials(range + (int64_t)c * nblk * 2 + 1, nblk, 2, -INFINITY);
  return f16_exp(fmax(hi - (double)mu, nlo + (double)mu));
}

// Row of piece p of column c in a tensor-core operand whose pieces are kp rows apart.
__device__ __forceinline__ int64_t piece_row(int p, int kp, int c) { return (int64_t)p * kp + c; }

// Row of padding row q (q < N − pieces·k) of such an operand: first the kp − k spare rows after
// each piece's k columns, then the rows from pieces·kp to N.
__device__ __forceinline__ int pad_row(int q, int k, int kp, int pieces)
{
  const int per = kp - k;
  if (q < pieces * per) return (q / per) * kp + k + (q % per);
  return pieces * kp + (q - pieces * per);
}

// Writes x[0 … V−1] (rows kidx …) into the dense operand — FP32 row c (npieces == 0) or 16-bit
// pieces in rows p·kp + c (BF16, or the FP16 fixed-point split of x·scale when F16) — and adds
// exactly what the products will see, in the units of x, to acc (weighted by wt when kWeighted).
template <int V, bool kWeighted, bool F16 = false>
__device__ __forceinline__ void store_operand(const float (&x)[V], int npieces, void* Bv, int64_t K_pad, int kp,
                                              int c, int64_t kidx, DF& acc, const float (&wt)[V],
                                              float scale = 1.f, float inv_scale = 1.f)
{
  if (npieces == 0) {
    stv<V>(static_cast<float*>(Bv) + (int64_t)c * K_pad + kidx, x);
#pragma unroll
    for (int u = 0; u < V; ++u) {
      if (kWeighted) df_fma(acc, wt[u], x[u]);
      else df_add(acc, x[u]);
    }
    return;
  }
  uint16_t* B = static_cast<uint16_t*>(Bv);
  float r[V];
#pragma unroll
  for (int u = 0; u < V; ++u) r[u] = F16 ? __fmul_rn(x[u], scale) : x[u];   // exact: scale is 2^e
  for (int p = 0; p < npieces; ++p) {
    uint16_t h[V];
#pragma unroll
    for (int u = 0; u < V; ++u) {
      float hf;
      if constexpr (F16) {
        // Stored times the K position's 2^−2s (the decoded counts carry 2^2s, f16sub_pair_of).
        // piece 0: the integer part (|r| ≤ 2^11: exact in FP16 after the ≥ 2^−8 factor); later
        // pieces: FP16 rounding of the scaled residual, subnormal below 2^−14 (absolute step
        // 2^−24·2^2s ≤ 2^−16 in units of r, against pieces of up to 2^11)
        const __half hh = __float2half_rn(__fmul_rn(p == 0 ? rintf(r[u]) : r[u], f16sub_kscale(kidx + u)));
        hf = __fmul_rn(__half2float(hh), f16sub_kunscale(kidx + u));   // exact
        h[u] = __half_as_ushort(hh);
      } else {
        const __nv_bfloat16 hb = __float2bfloat16_rn(r[u]);
        hf = __bfloat162float(hb);
        h[u] = __bfloat16_as_ushort(hb);
      }
      r[u] = __fsub_rn(r[u], hf);   // exact in FP32
      const float hv = F16 ? __fmul_rn(hf, inv_scale) : hf;
      if (kWeighted) df_fma(acc, wt[u], hv);
      else df_add(acc, hv);
    }
    uint16_t* dst = B + piece_row(p, kp, c) * K_pad + kidx;
    if constexpr (V == 4) {
      uint2 pk;
      pk.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
      pk.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
      *reinterpret_cast<uint2*>(dst) = pk;
    } else {
      dst[0] = h[0];
    }
  }
}

// Zeroes 16-bit padding row `row` of the operand over K-range [k0, k1).
__device__ __forceinline__ void zero_pad_row(void* Bv, int64_t K_pad, int row, int64_t k0, int64_t k1)
{
  uint2* dst = reinterpret_cast<uint2*>(static_cast<uint16_t*>(Bv) + (int64_t)row * K_pad);
  for (int64_t q = k0 / 4 + threadIdx.x; q < k1 / 4; q += blockDim.x) dst[q] = make_uint2(0u, 0u);
}

// Direction-1 operand (K = individuals): x = in[i,c]; for the first nq columns
// x −= Σ_l Q[i,l]·QtV[l,c] (QtV from its partials); optionally x *= rr[i]; rows i ≥ n are 0.
// red[c][blk] = Σ_i stored(x).  Blocks with c ≥ k zero the operand's padding rows (pad_row).
// MEASURE: only red[c][blk] = Σ_i x (the column sums that give the means), nothing stored.
// Otherwise, with mparts (those sums), x − μ_c is stored, μ_c = (float)(Σ/n) as in column_mean.
__device__ __forceinline__ float column_mean(const double* __restrict__ mparts, int nblk, int c, double inv_n)
{
  return (float)(warp_sum_partials(mparts + (int64_t)c * nblk, nblk) * inv_n);   // by a whole warp
}

// F16: the operand is stored as FP16 pieces of (x − μ)·2^e, e from the MEASURE pass's signed
// extremes (f16_col_exp).  MEASURE also writes xmax[c][blk][2] = {max x, max −x} over the valid
// rows when xmax != nullptr.
template <int V, bool MEASURE, bool F16 = false>
__global__ void __launch_bounds__(kRedThreads)
prologue_indiv_kernel(const float* __restrict__ in, int64_t ld, int64_t n, int64_t n_pad, int k, int kp,
                      const float* __restrict__ Q, int64_t ldq, int cq, const double* __restrict__ qparts,
                      int nblkq, int nq, const float* __restrict__ rr, int npieces, void* B,
                      double* __restrict__ red, int nblk, const double* __restrict__ mparts,
                      double* __restrict__ xmax, const int32_t* __restrict__ inv)
{
  __shared__ double sh[32];
  __shared__ float shf[32];
  __shared__ float2 qt[SLEMM_MAX_COVARIATES];
  __shared__ float smu, ssc[2];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kRowsPerBlock, i1 = min64(n_pad, i0 + kRowsPerBlock);
  if (c >= k) {
    if (!MEASURE) zero_pad_row(B, n_pad, pad_row(c - k, k, kp, npieces), i0, i1);
    return;
  }
  const bool proj = qparts != nullptr && c < nq;
  if (proj) load_qt(qparts, nblkq, cq, nq, c, qt);
  if (!MEASURE && (mparts != nullptr || F16)) {
    if (threadIdx.x < 32) {   // warp 0 reduces the column's partials
      const float mu_ = mparts != nullptr ? column_mean(mparts, nblk, c, 1.0 / (double)n) : 0.f;
      const int e = F16 ? f16_col_exp(xmax, nblk, c, mu_) : 0;
      if (threadIdx.x == 0) {
        smu = mu_;
        ssc[0] = ldexpf(1.f, e);
        ssc[1] = ldexpf(1.f, -e);
      }
    }
    __syncthreads();
  }
  const float mu = (!MEASURE && mparts != nullptr) ? smu : 0.f;
  const float sc = (!MEASURE && F16) ? ssc[0] : 1.f, isc = (!MEASURE && F16) ? ssc[1] : 1.f;
  DF acc;
  float xhi = -INFINITY, nxlo = -INFINITY;   // MEASURE: max x and max −x over the valid rows
  const float one[V] = {};
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kRedThreads * V) {
    float x[V] = {};
    bool ok[V];
    if (inv != nullptr) {
      // trait view: packed position i + u holds view row inv[i + u], or no individual of the view
#pragma unroll
      for (int u = 0; u < V; ++u) {
        const int64_t rv = inv[i + u];
        ok[u] = rv >= 0;
        if (ok[u]) {
          x[u] = in[(int64_t)c * ld + rv];
          if (proj) x[u] = __fsub_rn(x[u], proj_dot(Q, ldq, cq, rv, qt));
          if (rr) x[u] = __fmul_rn(x[u], rr[rv]);
          if (!MEASURE) x[u] = __fsub_rn(x[u], mu);
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < V; ++u) ok[u] = i + u < n;
      if (i < n) {
        ldv<V>(in + (int64_t)c * ld + i, x);
        if (proj) {
#pragma unroll
          for (int u = 0; u < V; ++u) x[u] = __fsub_rn(x[u], proj_dot(Q, ldq, cq, i + u, qt));
        }
        if (rr) {
          float r[V];
          ldv<V>(rr + i, r);
#pragma unroll
          for (int u = 0; u < V; ++u) x[u] = __fmul_rn(x[u], r[u]);
        }
        if (!MEASURE) {
#pragma unroll
          for (int u = 0; u < V; ++u)
            if (ok[u]) x[u] = __fsub_rn(x[u], mu);
        }
      }
    }
    if (MEASURE) {
#pragma unroll
      for (int u = 0; u < V; ++u) {
        df_add(acc, x[u]);
        if (ok[u]) {
          xhi = fmaxf(xhi, x[u]);
          nxlo = fmaxf(nxlo, -x[u]);
        }
      }
    } else {
      store_operand<V, false, F16>(x, npieces, B, n_pad, kp, c, i, acc, one, sc, isc);
    }
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0 && red != nullptr) red[(int64_t)c * nblk + blockIdx.x] = s;
  if (MEASURE && xmax != nullptr) {   // signed extremes [c][blk][2] (f16_col_exp)
    const float mx = block_max_f(xhi, shf);
    const float mn = block_max_f(nxlo, shf);
    if (threadIdx.x == 0) {
      xmax[((int64_t)c * nblk + blockIdx.x) * 2] = (double)mx;
      xmax[((int64_t)c * nblk + blockIdx.x) * 2 + 1] = (double)mn;
    }
  }
}

// Sum over the split-K partials ([splits][kp][M_pad]) of column c, rows r … r+V−1, times isc
// (2^−e of an FP16 operand column, else 1).
template <int V>
__device__ __forceinline__ void gather_D(const float* __restrict__ D, int splits, int kp, int64_t M_pad,
                                         int c, int64_t r, float isc, float (&acc)[V])
{
#pragma unroll
  for (int u = 0; u < V; ++u) acc[u] = 0.f;
  for (int s = 0; s < splits; ++s) {
    float t[V];
    ldv<V>(D + ((int64_t)s * kp + c) * M_pad + r, t);
#pragma unroll
    for (int u = 0; u < V; ++u) acc[u] = __fadd_rn(acc[u], t[u]);
  }
#pragma unroll
  for (int u = 0; u < V; ++u) acc[u] = __fmul_rn(acc[u], isc);
}

// Direction-1 finalize (rows = SNPs): val = raw·2^−e1 − gm_j·colsum_c (colsum from the prologue's
// partials; e1 the FP16 scale of operand column c when xmax1 != nullptr), plus μ·gcorr_j for the
// mean the prologue removed, times w_j when w != nullptr.  mode 0: out[j,c] = val (j < m).
// mode 1: val becomes the direction-2 operand (K = SNPs) and red[c][blk] = Σ_j gm_j·stored(val);
// with V2 != nullptr (FP16 operand) val goes to V2[c][j] in FP32 with its block maxima in xmax2,
// for convert_snp_kernel to scale and split.  Blocks with c ≥ k zero the operand's padding rows.
template <int V>
__global__ void __launch_bounds__(kRedThreads)
finalize_snp_kernel(const float* __restrict__ D, int splits, int kp1, int64_t m_pad, int k, int64_t m,
                    const float* __restrict__ gm, const float* __restrict__ w, const double* __restrict__ cparts,
                    int nblkc, int mode, float* __restrict__ out, int64_t ldo, int npieces2, int kp2, void* B2,
                    double* __restrict__ red, int nblk, const double* __restrict__ mparts,
                    const float* __restrict__ gcorr, int64_t n_rows, const double* __restrict__ xmax1,
                    float* __restrict__ V2, double* __restrict__ xmax2)
{
  __shared__ double sh[32];
  __shared__ float shf[32];
  __shared__ float sb[2];
  __shared__ float smu, sisc;
  const int c = blockIdx.y;
  const int64_t j0 = (int64_t)blockIdx.x * kRowsPerBlock, j1 = min64(m_pad, j0 + kRowsPerBlock);
  if (c >= k) {
    zero_pad_row(B2, m_pad, pad_row(c - k, k, kp2, npieces2), j0, j1);
    return;
  }
  float ch, cl;
  block_scalar([&] { return warp_sum_partials(cparts + (int64_t)c * nblkc, nblkc); }, sb, ch, cl);
  if (threadIdx.x < 32) {   // the mean the prologue removed, added back as μ·(pc_j − n·gm_j)
    const float mu_ = mparts != nullptr ? column_mean(mparts, nblkc, c, 1.0 / (double)n_rows) : 0.f;
    const float isc_ = xmax1 != nullptr ? ldexpf(1.f, -f16_col_exp(xmax1, nblkc, c, mu_)) : 1.f;
    if (threadIdx.x == 0) {
      smu = mu_;
      sisc = isc_;
    }
  }
  __syncthreads();
  const float mu = mparts != nullptr ? smu : 0.f;
  const float isc = sisc;
  DF acc;
  float amax = 0.f;
  for (int64_t j = j0 + threadIdx.x * V; j < j1; j += kRedThreads * V) {
    float val[V] = {}, g[V], e[V] = {};
    ldv<V>(gm + j, g);   // gm is zero-padded to m_pad
    if (mparts != nullptr) ldv<V>(gcorr + j, e);
    if (j < m) {
      gather_D<V>(D, splits, kp1, m_pad, c, j, isc, val);
      float ws[V];
      if (w) ldv<V>(w + j, ws);
#pragma unroll
      for (int u = 0; u < V; ++u) {
        float v = __fmaf_rn(-g[u], cl, __fmaf_rn(-g[u], ch, val[u]));
        if (mparts != nullptr) v = __fmaf_rn(mu, e[u], v);
        if (w) v = __fmul_rn(v, ws[u]);
        val[u] = v;
      }
    }
    if (mode == 0) {
      if (j < m) stv<V>(out + (int64_t)c * ldo + j, val);
    } else if (V2 != nullptr) {
      stv<V>(V2 + (int64_t)c * m_pad + j, val);
#pragma unroll
      for (int u = 0; u < V; ++u) amax = fmaxf(amax, fabsf(val[u]));
    } else {
      store_operand<V, true>(val, npieces2, B2, m_pad, kp2, c, j, acc, g);
    }
  }
  if (mode == 1) {
    if (V2 != nullptr) {
      const float mx = block_max_f(amax, shf);
      if (threadIdx.x == 0) xmax2[(int64_t)c * nblk + blockIdx.x] = (double)mx;
    } else {
      const double s = block_sum_d(df_value(acc), sh);
      if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
    }
  }
}

// FP16 direction-2 operand from the FP32 values V2[c][j] (finalize_snp_kernel, mode 1): pieces of
// V2·2^e2, e2 from the block maxima xmax2, and red[c][blk] = Σ_j gm_j·stored(val).
template <int V>
__global__ void __launch_bounds__(kRedThreads)
convert_snp_kernel(const float* __restrict__ V2, int64_t m_pad, int k, int kp2, const float* __restrict__ gm,
                   int npieces, void* B, double* __restrict__ red, int nblk, const double* __restrict__ xmax2)
{
  __shared__ double sh[32];
  __shared__ float ssc[2];
  const int c = blockIdx.y;
  const int64_t j0 = (int64_t)blockIdx.x * kRowsPerBlock, j1 = min64(m_pad, j0 + kRowsPerBlock);
  if (threadIdx.x < 32) {
    const int e = f16_exp(max_partials(xmax2, nblk, c));
    if (threadIdx.x == 0) {
      ssc[0] = ldexpf(1.f, e);
      ssc[1] = ldexpf(1.f, -e);
    }
  }
  __syncthreads();
  DF acc;
  for (int64_t j = j0 + threadIdx.x * V; j < j1; j += kRedThreads * V) {
    float x[V], g[V];
    ldv<V>(V2 + (int64_t)c * m_pad + j, x);
    ldv<V>(gm + j, g);
    store_operand<V, true, true>(x, npieces, B, m_pad, kp2, c, j, acc, g, ssc[0], ssc[1]);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// Direction-2 operand straight from an m×k input (matvec): stored(in) and red = Σ gm·stored;
// blocks with c ≥ k zero the padding rows.  F16: MEASURE writes the block maxima of |in| to
// xmax, and the store pass scales each column by 2^e from them.
template <int V, bool MEASURE = false, bool F16 = false>
__global__ void __launch_bounds__(kRedThreads)
prologue_snp_kernel(const float* __restrict__ in, int64_t ld, int64_t m, int64_t m_pad, int k, int kp,
                    const float* __restrict__ gm, int npieces, void* B, double* __restrict__ red, int nblk,
                    double* __restrict__ xmax)
{
  __shared__ double sh[32];
  __shared__ float shf[32];
  __shared__ float ssc[2];
  const int c = blockIdx.y;
  const int64_t j0 = (int64_t)blockIdx.x * kRowsPerBlock, j1 = min64(m_pad, j0 + kRowsPerBlock);
  if (c >= k) {
    if (!MEASURE) zero_pad_row(B, m_pad, pad_row(c - k, k, kp, npieces), j0, j1);
    return;
  }
  if (F16 && !MEASURE) {
    if (threadIdx.x < 32) {
      const int e = f16_exp(max_partials(xmax, nblk, c));
      if (threadIdx.x == 0) {
        ssc[0] = ldexpf(1.f, e);
        ssc[1] = ldexpf(1.f, -e);
      }
    }
    __syncthreads();
  }
  DF acc;
  float amax = 0.f;
  for (int64_t j = j0 + threadIdx.x * V; j < j1; j += kRedThreads * V) {
    float x[V] = {}, g[V];
    if (j < m) ldv<V>(in + (int64_t)c * ld + j, x);
    if (MEASURE) {
#pragma unroll
      for (int u = 0; u < V; ++u) amax = fmaxf(amax, fabsf(x[u]));
      continue;
    }
    ldv<V>(gm + j, g);
    if (F16) store_operand<V, true, true>(x, npieces, B, m_pad, kp, c, j, acc, g, ssc[0], ssc[1]);
    else store_operand<V, true>(x, npieces, B, m_pad, kp, c, j, acc, g);
  }
  if (MEASURE) {
    const float mx = block_max_f(amax, shf);
    if (threadIdx.x == 0) xmax[(int64_t)c * nblk + blockIdx.x] = (double)mx;
    return;
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// Direction-2 finalize (rows = individuals): val = raw·2^−e2 − t_c (t from the direction-1
// partials; e2 the FP16 scale of operand column c when xmax2 != nullptr), times rr_i when
// rr != nullptr, plus tau0·Vin for columns c ≥ nq when Vin != nullptr.
template <int V>
__global__ void __launch_bounds__(kRedThreads)
finalize_indiv_kernel(const float* __restrict__ D, int splits, int kp2, int64_t n_pad, int k,
                      int64_t n, const double* __restrict__ tparts, int nblkt, const float* __restrict__ rr,
                      const float* __restrict__ Vin, int64_t ld_v, float tau0, int nq, float* __restrict__ out,
                      int64_t ldo, const double* __restrict__ xmax2, const int32_t* __restrict__ map)
{
  __shared__ float sb[2];
  __shared__ float sisc;
  const int c = blockIdx.y;
  float th, tl;
  block_scalar([&] { return warp_sum_partials(tparts + (int64_t)c * nblkt, nblkt); }, sb, th, tl);
  if (threadIdx.x < 32) {
    const float isc_ = xmax2 != nullptr ? ldexpf(1.f, -f16_exp(max_partials(xmax2, nblkt, c))) : 1.f;
    if (threadIdx.x == 0) sisc = isc_;
  }
  __syncthreads();
  const float isc = sisc;
  const int64_t i = ((int64_t)blockIdx.x * kRedThreads + threadIdx.x) * V;
  if (i >= n) return;
  float val[V];
  if (map != nullptr) {   // trait view: view row i + u is packed row map[i + u]
#pragma unroll
    for (int u = 0; u < V; ++u) {
      float t[1];
      gather_D<1>(D, splits, kp2, n_pad, c, map[i + u], isc, t);
      val[u] = t[0];
    }
  } else {
    gather_D<V>(D, splits, kp2, n_pad, c, i, isc, val);
  }
  float r[V], v[V];
  if (rr) ldv<V>(rr + i, r);
  const bool addv = Vin != nullptr && c >= nq;
  if (addv) ldv<V>(Vin + (int64_t)c * ld_v + i, v);
#pragma unroll
  for (int u = 0; u < V; ++u) {
    float x = __fsub_rn(__fsub_rn(val[u], th), tl);
    if (rr) x = __fmul_rn(x, r[u]);
    if (addv) x = __fmaf_rn(tau0, v[u], x);
    val[u] = x;
  }
  stv<V>(out + (int64_t)c * ldo + i, val);
}

// ---- one packed pass ---------------------------------------------------------------------------------
struct PassPlan {
  bool tc;
  bool f16;     // FP16 pieces with per-column scales (tc)
  int pieces;   // 16-bit pieces per column (tc) or 1 (simt)
  int kp;       // rows between a column's pieces (k rounded up to 8) and columns of D per split
  int N;        // columns of the product
  int splits;
  int plan = 0; // tensor-core ring plan (GemmArgs::plan)
};

// Fewest splits of a tensor-core pass.  Once the dense operand (K_pad·N BF16) is larger than half
// the L2, CTAs with long K ranges run slower per K-tile — co-running CTAs drift apart along K and
// miss on the dense tiles they share.  Measured for Zᵀ over n = 950,000 individuals at N = 144:
// 4,948 K-tiles per CTA 0.417 µs per K-tile, 1,485 0.356 (8.25 → 6.87 ms per launch), and 0.331
// at n = 100,000 where the operand stays in L2.  So such passes keep ≤ 1,536 K-tiles per CTA.
static int tc_min_splits(int64_t K_tiles, int N)
{
  const double dense_bytes = (double)K_tiles * kTileK * N * 2.0;
  return dense_bytes > 64.0 * 1024 * 1024 ? (int)ceil_div(K_tiles, 1536) : 1;
}

static cudaEvent_t take_event(slemm_geno* g);

// ---- split-K autotuner ------------------------------------------------------------------------------
// With a handle's autotune on, the first tensor-core pass of each shape (device, N, pieces, K-tiles,
// padded rows) times a handful of (plan, split-K) choices with CUDA events on the handle's stream —
// the fixed rule's count, and counts near it whose CTAs fill the last wave to ≥ 80 %; for N ≤ 64
// also the two-CTAs-per-SM plan at its own rule's count and counts near it — each launched once to
// warm up and twice timed over the real packed copy, and keeps the fastest if it beats the rule's by
// ≥ 3 % (else the rule's, so close calls do not flip between processes).  Decisions are cached for
// the life of the process; no tuning happens while the stream is being captured.
struct TuneKey {
  int dev, N, pieces;
  int64_t K_tiles, M_pad;
  bool operator<(const TuneKey& o) const
  {
    return std::tie(dev, N, pieces, K_tiles, M_pad) < std::tie(o.dev, o.N, o.pieces, o.K_tiles, o.M_pad);
  }
};
struct TuneEntry {
  int rule, best, plan, candidates;
  double ms_rule, ms_best;
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tune;

// Up to `most` split counts near `rule` (rule first) whose CTAs fill the last wave to ≥ 80 %.
static void near_splits(int rule, int64_t ctas, int per_sm, int64_t K_tiles, int plan, size_t most,
                        std::vector<std::pair<int, int>>& cand)
{
  const int sms = num_sms() * per_sm;
  cand.push_back({plan, rule});
  std::vector<std::pair<int, int>> near;   // (distance, s)
  const int smax = (int)std::min<int64_t>(std::max(3 * rule + 2, 8), std::max<int64_t>(1, K_tiles / 16));
  for (int s = std::max(1, rule / 3); s <= smax; ++s) {
    if (s == rule) continue;
    const double waves = (double)(ctas * s) / sms;
    if (waves / std::ceil(waves) >= 0.8) near.push_back({std::abs(s - rule), s});
  }
  std::sort(near.begin(), near.end());
  for (size_t i = 0; i < near.size() && i + 1 < most; ++i) cand.push_back({plan, near[i].second});
}

// Tunes p.splits and p.plan in place.
static void tune_pass(slemm_geno* g, PassPlan& p, const uint8_t* A, int64_t M_pad, int64_t K_pad)
{
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CUDA_TRY(cudaStreamIsCapturing(g->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return;
  const int64_t K_tiles = K_pad / kTileK;
  const TuneKey key{g->device, p.N, p.pieces, K_tiles, M_pad};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      p.splits = it->second.best;
      p.plan = it->second.plan;
      return;
    }
  }
  // candidates: the rule's count, then counts near it with a well-filled last wave; for N ≤ 64 the
  // same around the two-CTAs-per-SM plan's rule
  std::vector<std::pair<int, int>> cand;   // (plan, splits)
  near_splits(p.splits, M_pad / gemm_tc_rows_per_cta(p.N, 0), 1, K_tiles, 0, 6, cand);
  if (p.N <= 64) {
    const int64_t ctas1 = M_pad / gemm_tc_rows_per_cta(p.N, 1);
    const int rule1 = choose_splits(ctas1, K_tiles, 2, num_sms(), tc_min_splits(K_tiles, p.N));
    near_splits(rule1, ctas1, 2, K_tiles, 1, 3, cand);
  }
  int smost = 1;
  for (const auto& c : cand) smost = std::max(smost, c.second);
  DevBuf dD(g->stream);
  float* D = (float*)dD.ensure((size_t)smost * p.kp * M_pad * sizeof(float));
  const void* B = g->ws_B.ensure((size_t)p.N * K_pad * 2);   // timing only: the operand's values do not matter
  cudaEvent_t e0 = take_event(g), e1 = take_event(g);
  std::vector<double> ms(cand.size());
  for (size_t i = 0; i < cand.size(); ++i) {
    GemmArgs a{A, M_pad, K_pad, B, p.N, D, cand[i].second, g->err.as<int>(), p.kp, p.pieces, p.f16, cand[i].first};
    gemm_tc(a, g->stream);
    CUDA_TRY(cudaEventRecord(e0, g->stream));
    gemm_tc(a, g->stream);
    gemm_tc(a, g->stream);
    CUDA_TRY(cudaEventRecord(e1, g->stream));
    CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
    ms[i] = t / 2.0;
  }
  g->event_pool.push_back(e0);
  g->event_pool.push_back(e1);
  CUDA_TRY(cudaMemsetAsync(g->err.p, 0, sizeof(int), g->stream));   // the timing launches' waits are not the caller's
  size_t b = 0;
  for (size_t i = 1; i < cand.size(); ++i)
    if (ms[i] < ms[b]) b = i;
  if (ms[b] > 0.97 * ms[0]) b = 0;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = {p.splits, cand[b].second, cand[b].first, (int)cand.size(), ms[0], ms[b]};
  p.plan = cand[b].first;
  p.splits = cand[b].second;
}

static PassPlan plan_pass(slemm_geno* g, int k, int64_t M_pad, int64_t K_pad, const uint8_t* A)
{
  PassPlan p;
  p.tc = g->prec != SLEMM_PREC_FP32;
  p.f16 = g->prec == SLEMM_PREC_FP16X2;
  p.pieces = g->prec == SLEMM_PREC_BF16X3 ? 3 : (p.tc ? 2 : 1);
  p.kp = p.tc ? (int)round_up(k, 8) : k;
  p.N = p.tc ? (int)round_up((int64_t)p.pieces * p.kp, 16) : k;
  const int64_t M_tiles = M_pad / kTileM, K_tiles = K_pad / kTileK;
  p.splits = p.tc ? choose_splits(M_pad / gemm_tc_rows_per_cta(p.N, 0), K_tiles, 1, num_sms(),
                                  tc_min_splits(K_tiles, p.N))
                  : choose_splits(M_tiles, K_tiles, 8, num_sms());
  if (p.tc && g->autotune == 2 && p.N <= 64) {
    p.plan = 1;
    p.splits = choose_splits(M_pad / gemm_tc_rows_per_cta(p.N, 1), K_tiles, 2, num_sms(),
                             tc_min_splits(K_tiles, p.N));
  }
  if (p.tc && g->autotune == 1 && A) tune_pass(g, p, A, M_pad, K_pad);
  return p;
}

static int max_group(const slemm_geno* g)
{
  if (g->per_vector) return 1;
  if (g->prec == SLEMM_PREC_BF16X2 || g->prec == SLEMM_PREC_FP16X2) return 128;
  if (g->prec == SLEMM_PREC_BF16X3) return 80;
  return 64;
}

static cudaEvent_t take_event(slemm_geno* g)
{
  if (!g->event_pool.empty()) {
    cudaEvent_t e = g->event_pool.back();
    g->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CUDA_TRY(cudaEventCreate(&e));
  return e;
}

// Folds completed launch records into the per-shape statistics (synchronises on the events).
void profile_collect(slemm_geno* g)
{
  for (auto& r : g->prof_pending) {
    CUDA_TRY(cudaEventSynchronize(r.stop));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, r.start, r.stop));
    bool found = false;
    for (auto& s : g->prof_stats)
      if (s.tc == r.tc && s.N == r.N && s.k == r.k && s.dir == r.dir && s.pieces == r.pieces &&
          s.splits == r.splits && s.plan == r.plan) {
        s.launches += 1;
        s.ms += ms;
        found = true;
        break;
      }
    if (!found) g->prof_stats.push_back({r.tc, r.N, r.k, r.pieces, r.dir, r.splits, r.plan, 1, (double)ms});
    g->event_pool.push_back(r.start);
    g->event_pool.push_back(r.stop);
  }
  g->prof_pending.clear();
}

static void run_gemm(slemm_geno* g, const PassPlan& p, const uint8_t* A, int64_t M_pad,
                     int64_t K_pad, const void* B, float* D, int* err, int k, int dir)
{
  GemmArgs a{A, M_pad, K_pad, B, p.N, D, p.splits, err, p.kp, p.pieces, p.f16, p.plan};
  slemm_geno::GemmRecord rec{};
  if (g->profiling) {
    if (g->prof_pending.size() >= 512) profile_collect(g);
    rec = {take_event(g), take_event(g), p.tc ? 1 : 0, p.N, k, p.pieces, p.splits, dir, p.plan};
    CUDA_TRY(cudaEventRecord(rec.start, g->stream));
  }
  if (p.tc) gemm_tc(a, g->stream);
  else gemm_simt(a, g->stream);
  if (g->profiling) {
    CUDA_TRY(cudaEventRecord(rec.stop, g->stream));
    g->prof_pending.push_back(rec);
  }
}

// One operator application on a column group (k ≤ max_group).  For the H0 operators (kind
// LDET, or QUADFORM) the first nq columns get the projections of H0_quadform_mv and the others
// are plain H0_ldet_mv columns, so one block can carry both kinds of seed systems.
//
// Launches: [QᵀV partials] → prologue (operand 1 + its column sums) → packed pass 1 → finalize 1
// (operand 2 + its centring sums) → packed pass 2 → finalize 2 → [QᵀT partials → projection].
// Each kernel sums the partials it needs itself, in a fixed order.
static void op_group(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
                     float* out, int64_t ld_out, int nq)
{
  if (kind == SLEMM_OP_QUADFORM) kind = SLEMM_OP_LDET;   // nq carries the projected columns
  cudaStream_t st = g->stream;
  const bool dir1 = kind != SLEMM_OP_MATVEC;                          // needs Zᵀ pass
  const bool dir2 = kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET || kind == SLEMM_OP_MATVEC;
  // (the tuner times only the directions this operator runs)
  const PassPlan p1 = plan_pass(g, k, g->m_pad, g->n_pad, dir1 ? g->G.as<uint8_t>() : nullptr);    // M = SNPs, K = indiv
  const PassPlan p2 = plan_pass(g, k, g->n_pad, g->m_pad, dir2 ? g->GT.as<uint8_t>() : nullptr);   // M = indiv, K = SNPs
  const int np1 = p1.tc ? p1.pieces : 0, np2 = p2.tc ? p2.pieces : 0;
  const int pad1 = p1.tc ? p1.N - p1.pieces * k : 0;                   // padding rows of the operands
  const int pad2 = p2.tc ? p2.N - p2.pieces * k : 0;
  const bool f16 = p1.f16;
  const size_t b1 = dir1 ? (p1.tc ? (size_t)p1.N * g->n_pad * 2 : (size_t)k * g->n_pad * 4) : 0;
  const size_t b2 = dir2 ? (p2.tc ? (size_t)p2.N * g->m_pad * 2 : (size_t)k * g->m_pad * 4) : 0;
  // FP16: the direction-2 values in FP32 before they are scaled and split
  const size_t bv2 = (dir1 && dir2 && f16) ? (size_t)k * g->m_pad * 4 : 0;
  uint8_t* Bbuf = (uint8_t*)g->ws_B.ensure(b1 + b2 + bv2);
  void* B1 = Bbuf;
  void* B2 = Bbuf + b1;
  float* V2 = bv2 ? (float*)(Bbuf + b1 + b2) : nullptr;
  const size_t d1 = dir1 ? (size_t)p1.splits * p1.kp * g->m_pad : 0;
  const size_t d2 = dir2 ? (size_t)p2.splits * p2.kp * g->n_pad : 0;
  float* D = (float*)g->ws_D.ensure(std::max(d1, d2) * sizeof(float));
  const int nblk_n = (int)ceil_div(g->n_pad, kRowsPerBlock);
  const int nblk_m = (int)ceil_div(g->m_pad, kRowsPerBlock);
  const int nblk_q = (int)ceil_div(g->n, kRowsPerBlock);
  // partials: colsum [k][nblk_n] | tsum [k][nblk_m] | QᵀV [c·nq][nblk_q] | QᵀT [c·nq][nblk_q] |
  // column sums for the means [k][nblk_n] | FP16 ranges: operand 1 signed extremes [k][nblk_n][2],
  // operand 2 maxima of |x| [k][nblk_m]
  const int cq = g->c;
  CHECK_ARG(cq <= SLEMM_MAX_COVARIATES, "too many covariates");
  const size_t nred = 2 * (size_t)k * nblk_n + (size_t)k * nblk_m + 2 * (size_t)std::max(cq, 1) * k * nblk_q +
                      (f16 ? (size_t)k * (2 * nblk_n + nblk_m) : 0);
  double* r_col = (double*)g->ws_red.ensure(nred * sizeof(double));
  double* r_t = r_col + (size_t)k * nblk_n;
  double* r_qv = r_t + (size_t)k * nblk_m;
  double* r_qt = r_qv + (size_t)std::max(cq, 1) * k * nblk_q;
  double* r_mu = r_qt + (size_t)std::max(cq, 1) * k * nblk_q;   // column sums for the means [k][nblk_n]
  double* x_max1 = f16 ? r_mu + (size_t)k * nblk_n : nullptr;        // [k][nblk_n][2]
  double* x_max2 = f16 ? x_max1 + 2 * (size_t)k * nblk_n : nullptr;  // [k][nblk_m]
  int* err = g->err.as<int>();

  // H0 operators: the first nq columns are projected (H0_quadform_mv), the rest are not (H0_ldet_mv)
  const bool h0 = kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET;
  const bool vin = vec4_ok(g->n, ld_in, in);
  // a trait view reads its inputs and writes its outputs through its individual map
  const int32_t* inv_ind = g->is_view ? g->ind_inv.as<int32_t>() : nullptr;
  const int32_t* map_ind = g->is_view ? g->ind_map.as<int32_t>() : nullptr;

  if (dir1) {
    // ---- prologue 1: v_adj = rr∘(v − QQᵀv) (quadform), rr∘v (ldet), v (rmatvec) ----
    const bool proj = h0 && nq > 0 && cq > 0;
    if (proj) proj_partials(g, in, ld_in, nq, r_qv, nblk_q);
    dim3 grid(nblk_n, k + pad1);
    const float* rr = h0 ? g->rr.as<float>() : nullptr;
    const float* Qp = g->Q.as<float>();
    const double* qp = proj ? r_qv : nullptr;
    double* const mu = g->gcorr.p ? r_mu : nullptr;   // mean removal needs Z_cᵀ1 (set with the weights)
    if (mu || f16) {
      // measure pass: column sums (for the means) and, for FP16 operands, the column maxima
      if (vin)
        prologue_indiv_kernel<4, true><<<dim3(nblk_n, k), kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, mu, nblk_n, nullptr,
            x_max1, inv_ind);
      else
        prologue_indiv_kernel<1, true><<<dim3(nblk_n, k), kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, mu, nblk_n, nullptr,
            x_max1, inv_ind);
      LAUNCH_CHECK();
    }
    if (f16) {
      if (vin)
        prologue_indiv_kernel<4, false, true><<<grid, kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, r_col, nblk_n, mu,
            x_max1, inv_ind);
      else
        prologue_indiv_kernel<1, false, true><<<grid, kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, r_col, nblk_n, mu,
            x_max1, inv_ind);
    } else {
      if (vin)
        prologue_indiv_kernel<4, false><<<grid, kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, r_col, nblk_n, mu,
            nullptr, inv_ind);
      else
        prologue_indiv_kernel<1, false><<<grid, kRedThreads, 0, st>>>(
            in, ld_in, g->n, g->n_pad, k, p1.kp, Qp, g->n_pad, cq, qp, nblk_q, nq, rr, np1, B1, r_col, nblk_n, mu,
            nullptr, inv_ind);
    }
    LAUNCH_CHECK();
    // ---- pass 1: Cntᵀ over individuals ----
    run_gemm(g, p1, g->G.as<uint8_t>(), g->m_pad, g->n_pad, B1, D, err, k, 1);
    // ---- finalize 1 ----
    const float* wsc = (kind == SLEMM_OP_RMATVEC) ? nullptr : g->w.as<float>();
    if (h0) {
      finalize_snp_kernel<4><<<dim3(nblk_m, k + pad2), kRedThreads, 0, st>>>(
          D, p1.splits, p1.kp, g->m_pad, k, g->m, g->gm.as<float>(), wsc, r_col, nblk_n, 1, nullptr, 0, np2, p2.kp,
          B2, r_t, nblk_m, mu, g->gcorr.as<float>(), g->n, x_max1, V2, x_max2);
      LAUNCH_CHECK();
      if (f16) {
        convert_snp_kernel<4><<<dim3(nblk_m, k), kRedThreads, 0, st>>>(V2, g->m_pad, k, p2.kp, g->gm.as<float>(),
                                                                        np2, B2, r_t, nblk_m, x_max2);
        LAUNCH_CHECK();
      }
    } else {
      if (vec4_ok(g->m, ld_out, out))
        finalize_snp_kernel<4><<<dim3(nblk_m, k), kRedThreads, 0, st>>>(
            D, p1.splits, p1.kp, g->m_pad, k, g->m, g->gm.as<float>(), wsc, r_col, nblk_n, 0, out, ld_out, 0, 8,
            nullptr, nullptr, 0, mu, g->gcorr.as<float>(), g->n, x_max1, nullptr, nullptr);
      else
        finalize_snp_kernel<1><<<dim3(nblk_m, k), kRedThreads, 0, st>>>(
            D, p1.splits, p1.kp, g->m_pad, k, g->m, g->gm.as<float>(), wsc, r_col, nblk_n, 0, out, ld_out, 0, 8,
            nullptr, nullptr, 0, mu, g->gcorr.as<float>(), g->n, x_max1, nullptr, nullptr);
      LAUNCH_CHECK();
      return;
    }
  } else {
    // matvec: operand straight from the m×k input
    dim3 gridm(nblk_m, k + pad2);
    const bool v4 = vec4_ok(g->m, ld_in, in);
    if (f16) {
      if (v4) {
        prologue_snp_kernel<4, true, true><<<dim3(nblk_m, k), kRedThreads, 0, st>>>(
            in, ld_in, g->m, g->m_pad, k, p2.kp, g->gm.as<float>(), np2, B2, r_t, nblk_m, x_max2);
        LAUNCH_CHECK();
        prologue_snp_kernel<4, false, true><<<gridm, kRedThreads, 0, st>>>(in, ld_in, g->m, g->m_pad, k, p2.kp,
                                                                           g->gm.as<float>(), np2, B2, r_t, nblk_m,
                                                                           x_max2);
      } else {
        prologue_snp_kernel<1, true, true><<<dim3(nblk_m, k), kRedThreads, 0, st>>>(
            in, ld_in, g->m, g->m_pad, k, p2.kp, g->gm.as<float>(), np2, B2, r_t, nblk_m, x_max2);
        LAUNCH_CHECK();
        prologue_snp_kernel<1, false, true><<<gridm, kRedThreads, 0, st>>>(in, ld_in, g->m, g->m_pad, k, p2.kp,
                                                                           g->gm.as<float>(), np2, B2, r_t, nblk_m,
                                                                           x_max2);
      }
    } else {
      if (v4)
        prologue_snp_kernel<4><<<gridm, kRedThreads, 0, st>>>(in, ld_in, g->m, g->m_pad, k, p2.kp, g->gm.as<float>(),
                                                              np2, B2, r_t, nblk_m, nullptr);
      else
        prologue_snp_kernel<1><<<gridm, kRedThreads, 0, st>>>(in, ld_in, g->m, g->m_pad, k, p2.kp, g->gm.as<float>(),
                                                              np2, B2, r_t, nblk_m, nullptr);
    }
    LAUNCH_CHECK();
  }
  // ---- pass 2: Cnt over SNPs ----
  run_gemm(g, p2, g->GT.as<uint8_t>(), g->n_pad, g->m_pad, B2, D, err, k, 2);
  // ---- finalize 2 ----
  // matvec: out = raw − t.  H0: out = rr∘(raw − t) (+ τ0·v for the ldet columns nq … k−1)
  const float* rr2 = (kind == SLEMM_OP_MATVEC) ? nullptr : g->rr.as<float>();
  const float* v2 = (kind == SLEMM_OP_MATVEC) ? nullptr : in;
  const int nq2 = (kind == SLEMM_OP_MATVEC) ? 0 : nq;
  if (vec4_ok(g->n, ld_out, out) && (!v2 || vin)) {
    dim3 grid((unsigned)ceil_div(g->n, 4 * kRedThreads), k);
    finalize_indiv_kernel<4><<<grid, kRedThreads, 0, st>>>(D, p2.splits, p2.kp, g->n_pad, k, g->n, r_t, nblk_m, rr2,
                                                           v2, ld_in, tau0, nq2, out, ld_out, x_max2, map_ind);
  } else {
    dim3 grid((unsigned)ceil_div(g->n, kRedThreads), k);
    finalize_indiv_kernel<1><<<grid, kRedThreads, 0, st>>>(D, p2.splits, p2.kp, g->n_pad, k, g->n, r_t, nblk_m, rr2,
                                                           v2, ld_in, tau0, nq2, out, ld_out, x_max2, map_ind);
  }
  LAUNCH_CHECK();
  // quadform columns 0 … nq−1: out = T + τ0 v − QQᵀT
  if (kind != SLEMM_OP_MATVEC && nq > 0) {
    if (cq > 0) {
      proj_partials(g, out, ld_out, nq, r_qt, nblk_q);
      proj_apply_parts(g, out, ld_out, nq, r_qt, nblk_q, in, ld_in, tau0);
    } else {
      proj_apply_parts(g, out, ld_out, nq, nullptr, 1, in, ld_in, tau0);
    }
  }
}

// out[j, c] = Σ_i (count_ij − gm_j)·U[i, c] for SNP rows j ∈ [r0, r0 + rows) of the G copy (the
// centred Z_cᵀU of a window of SNPs) on the tensor cores at precision prec: SLEMM_PREC_FP16X2
// (column-scaled FP16 hi+lo, the most accurate at two pieces), SLEMM_PREC_BF16X3 or BF16X2.
// r0 and rows must be multiples of 256; U is n×k (ld ldu), out rows×k (ld ldo).
void rows_product(slemm_geno* g, int64_t r0, int64_t rows, const float* U, int64_t ldu, int k, float* out,
                  int64_t ldo, int prec)
{
  CHECK_ARG(r0 % kPadRows == 0 && rows % kPadRows == 0 && r0 + rows <= g->m_pad, "row range not aligned");
  CHECK_ARG(prec == SLEMM_PREC_FP16X2 || prec == SLEMM_PREC_BF16X2 || prec == SLEMM_PREC_BF16X3,
            "rows_product runs on the tensor cores");
  const bool f16 = prec == SLEMM_PREC_FP16X2;
  const int pieces = prec == SLEMM_PREC_BF16X3 ? 3 : 2;
  cudaStream_t st = g->stream;
  const int grp = pieces == 3 ? 80 : 128;
  const int64_t K_pad = g->n_pad, K_tiles = K_pad / kTileK;
  const uint8_t* A = g->G.as<uint8_t>() + (size_t)(r0 / kTileM) * K_tiles * kTileBytes;
  const int nblk_n = (int)ceil_div(g->n_pad, kRowsPerBlock);
  const int nblk_m = (int)ceil_div(rows, kRowsPerBlock);
  const int64_t m_valid = std::max<int64_t>(0, std::min<int64_t>(rows, g->m - r0));
  for (int c0 = 0; c0 < k; c0 += grp) {
    const int kc = std::min(grp, k - c0);
    PassPlan p;
    p.tc = true;
    p.f16 = f16;
    p.pieces = pieces;
    p.kp = (int)round_up(kc, 8);
    p.N = (int)round_up((int64_t)pieces * p.kp, 16);
    p.splits = choose_splits(rows / gemm_tc_rows_per_cta(p.N, 0), K_tiles, 1, num_sms(), tc_min_splits(K_tiles, p.N));
    const int pad = p.N - pieces * kc;
    void* B1 = g->ws_B.ensure((size_t)p.N * K_pad * 2);
    float* D = (float*)g->ws_D.ensure((size_t)p.splits * p.kp * rows * sizeof(float));
    // partials: column sums [kc][nblk_n] | sums for the means [kc][nblk_n] | FP16 signed extremes [kc][nblk_n][2]
    double* r_col = (double*)g->ws_red.ensure((size_t)kc * nblk_n * (f16 ? 4 : 2) * sizeof(double));
    double* r_mu = r_col + (size_t)kc * nblk_n;
    double* const mu = g->gcorr.p ? r_mu : nullptr;
    double* const x_rng = f16 ? r_mu + (size_t)kc * nblk_n : nullptr;
    const float* in = U + (int64_t)c0 * ldu;
    const bool v4 = vec4_ok(g->n, ldu, in);
    if (mu || f16) {   // measure pass: sums for the means, signed extremes for the FP16 scales
      if (v4)
        prologue_indiv_kernel<4, true><<<dim3(nblk_n, kc), kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, mu, nblk_n,
            nullptr, x_rng, nullptr);
      else
        prologue_indiv_kernel<1, true><<<dim3(nblk_n, kc), kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, mu, nblk_n,
            nullptr, x_rng, nullptr);
      LAUNCH_CHECK();
    }
    const dim3 grid(nblk_n, kc + pad);
    if (f16) {
      if (v4)
        prologue_indiv_kernel<4, false, true><<<grid, kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, r_col, nblk_n, mu,
            x_rng, nullptr);
      else
        prologue_indiv_kernel<1, false, true><<<grid, kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, r_col, nblk_n, mu,
            x_rng, nullptr);
    } else {
      if (v4)
        prologue_indiv_kernel<4, false><<<grid, kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, r_col, nblk_n, mu,
            nullptr, nullptr);
      else
        prologue_indiv_kernel<1, false><<<grid, kRedThreads, 0, st>>>(
            in, ldu, g->n, g->n_pad, kc, p.kp, nullptr, 0, 0, nullptr, 1, 0, nullptr, pieces, B1, r_col, nblk_n, mu,
            nullptr, nullptr);
    }
    LAUNCH_CHECK();
    run_gemm(g, p, A, rows, K_pad, B1, D, g->err.as<int>(), kc, 1);
    float* o = out + (int64_t)c0 * ldo;
    if (vec4_ok(m_valid, ldo, o))
      finalize_snp_kernel<4><<<dim3(nblk_m, kc), kRedThreads, 0, st>>>(
          D, p.splits, p.kp, rows, kc, m_valid, g->gm.as<float>() + r0, nullptr, r_col, nblk_n, 0, o, ldo, 0, 8,
          nullptr, nullptr, 0, mu, mu ? g->gcorr.as<float>() + r0 : nullptr, g->n, x_rng, nullptr, nullptr);
    else
      finalize_snp_kernel<1><<<dim3(nblk_m, kc), kRedThreads, 0, st>>>(
          D, p.splits, p.kp, rows, kc, m_valid, g->gm.as<float>() + r0, nullptr, r_col, nblk_n, 0, o, ldo, 0, 8,
          nullptr, nullptr, 0, mu, mu ? g->gcorr.as<float>() + r0 : nullptr, g->n, x_rng, nullptr, nullptr);
    LAUNCH_CHECK();
  }
}

void op_device_mixed(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
                     float* out, int64_t ld_out, int nq)
{
  if (!g->weights_set) SLEMM_THROW(SLEMM_ERR_STATE, "set_weights must be called before operators");
  CHECK_ARG(kind >= SLEMM_OP_QUADFORM && kind <= SLEMM_OP_WRMATVEC, "unknown operator kind");
  CHECK_ARG(k >= 1, "k must be >= 1");
  if (kind == SLEMM_OP_QUADFORM) nq = k;
  const bool h0 = kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET;
  if (!h0) nq = 0;
  CHECK_ARG(nq >= 0 && nq <= k, "bad number of projected columns");
  const int grp = max_group(g);
  for (int c0 = 0; c0 < k; c0 += grp) {
    const int kc = std::min(grp, k - c0);
    const int nqg = std::max(0, std::min(kc, nq - c0));
    op_group(g, kind, tau0, in + (int64_t)c0 * ld_in, ld_in, kc, out + (int64_t)c0 * ld_out, ld_out, nqg);
  }
}

void op_device(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
               float* out, int64_t ld_out)
{
  op_device_mixed(g, kind, tau0, in, ld_in, k, out, ld_out, kind == SLEMM_OP_QUADFORM ? k : 0);
}

int64_t workspace_bytes(const slemm_geno* g)
{
  return (int64_t)(g->ws_B.bytes + g->ws_D.bytes + g->ws_red.bytes + g->ws_small.bytes +
                   g->ws_T.bytes + g->ws_in.bytes + g->ws_out.bytes);
}

// Checks the device error word of the kernels' bounded waits (synchronises the stream).
void check_device_error(slemm_geno* g)
{
  int h = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, g->err.p, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
  CUDA_TRY(cudaStreamSynchronize(g->stream));
  if (h) {
    CUDA_TRY(cudaMemsetAsync(g->err.p, 0, sizeof(int), g->stream));
    SLEMM_THROW(SLEMM_ERR_CUDA, "a tensor-core kernel gave up a bounded wait (code " +
                                    std::to_string(h) + ")");
  }
}

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_set_autotune(slemm_geno* g, int on)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    CHECK_ARG(on >= 0 && on <= 2, "on must be 0, 1 or 2");
    g->autotune = on;
  });
}

extern "C" int slemm_gpu_autotune_table(int max_rows, int* rows, int32_t* info, int64_t* shape, double* ms)
{
  return guarded([&] {
    CHECK_ARG(rows != nullptr && max_rows >= 0, "bad arguments");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    *rows = (int)g_tune.size();
    int r = 0;
    for (const auto& kv : g_tune) {
      if (r >= max_rows) break;
      if (info) {
        const int32_t v[7] = {kv.first.dev, kv.first.N, kv.first.pieces, kv.second.rule, kv.second.best,
                              kv.second.plan, kv.second.candidates};
        std::copy(v, v + 7, info + 7 * r);
      }
      if (shape) {
        shape[2 * r] = kv.first.K_tiles;
        shape[2 * r + 1] = kv.first.M_pad;
      }
      if (ms) {
        ms[2 * r] = kv.second.ms_rule;
        ms[2 * r + 1] = kv.second.ms_best;
      }
      ++r;
    }
  });
}

extern "C" int slemm_gpu_op(slemm_geno* g, int op_kind, float tau0, const float* in, int64_t ld_in,
                            int k, float* out, int64_t ld_out, int mem)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && in != nullptr && out != nullptr, "null argument");
    CHECK_ARG(k >= 1 && k <= 4096, "k out of range");
    const int64_t rows_in = (op_kind == SLEMM_OP_MATVEC) ? g->m : g->n;
    const int64_t rows_out = (op_kind == SLEMM_OP_RMATVEC || op_kind == SLEMM_OP_WRMATVEC) ? g->m : g->n;
    CHECK_ARG(ld_in >= rows_in && ld_out >= rows_out, "leading dimension too small");
    if (mem == SLEMM_MEM_DEVICE) {
      op_device(g, op_kind, tau0, in, ld_in, k, out, ld_out);
      check_device_error(g);
      return;
    }
    CHECK_ARG(mem == SLEMM_MEM_HOST, "mem must be SLEMM_MEM_HOST or SLEMM_MEM_DEVICE");
    float* din = (float*)g->ws_in.ensure((size_t)rows_in * k * sizeof(float));
    float* dout = (float*)g->ws_out.ensure((size_t)rows_out * k * sizeof(float));
    CUDA_TRY(cudaMemcpy2DAsync(din, rows_in * sizeof(float), in, ld_in * sizeof(float),
                               rows_in * sizeof(float), k, cudaMemcpyHostToDevice, g->stream));
    op_device(g, op_kind, tau0, din, rows_in, k, dout, rows_out);
    CUDA_TRY(cudaMemcpy2DAsync(out, ld_out * sizeof(float), dout, rows_out * sizeof(float),
                               rows_out * sizeof(float), k, cudaMemcpyDeviceToHost, g->stream));
    check_device_error(g);
  });
}

extern "C" int slemm_gpu_profile(slemm_geno* g, int enable, int max_rows, int* rows, int32_t* info,
                                 int64_t* launches, double* ms)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr, "null handle");
    profile_collect(g);
    int r = 0;
    for (const auto& s : g->prof_stats) {
      if (r < max_rows && info && launches && ms) {
        const int32_t v[7] = {s.tc, s.N, s.k, s.pieces, s.dir, s.splits, s.plan};
        std::copy(v, v + 7, info + 7 * r);
        launches[r] = s.launches;
        ms[r] = s.ms;
      }
      ++r;
    }
    if (rows) *rows = r;
    if (enable >= 0) {
      g->prof_stats.clear();
      g->profiling = enable != 0;
    }
  });
}
