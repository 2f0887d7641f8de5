// ops.cu — operator applications built on the packed products (src/reml.cpp:8-233).
//
// Centring is an exact rank-1 correction: with x the allele count and gm_j its mean,
//   Z_cᵀu  = Cntᵀu − gm·(1ᵀu)          (direction 1, K = individuals, M = SNPs)
//   Z_c v  = Cnt v − 1·(gmᵀv)           (direction 2, K = SNPs, M = individuals)
// where Cnt holds the exact integer counts.  The dense side is prepared once per pass by a
// prologue (projection, rr scaling, FP32 → BF16 pieces) that also sums exactly what the
// tensor cores multiply, in FP64, for the correction term.  Finalize kernels reduce the split-K
// partials and the BF16 pieces, apply the correction and the reference's diagonal scalings,
// and either write the result or directly build the next pass's dense operand.
//
// All reductions are two-stage (per-block FP64 partials, then a fixed-order sum), so results
// are bit-reproducible run to run.
#include "internal.h"

#include <cuda_bf16.h>

namespace slemm {

constexpr int kRedThreads = 256;
constexpr int kRowsPerBlock = 4096;   // rows handled by one block of the row-wise kernels

__device__ __forceinline__ double block_sum(double v, double* sh)
{
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  }
  return r;   // valid in thread 0
}

// red[q][nblk] → out[q] (fixed order)
__global__ void reduce_partials_kernel(const double* __restrict__ red, int nblk, int nq,
                                       double* __restrict__ out)
{
  const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += red[(int64_t)q * nblk + b];
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[q] = s;
}

static void reduce_partials(const double* red, int nblk, int nq, double* out, cudaStream_t st)
{
  const int per_block = 8;
  reduce_partials_kernel<<<(unsigned)ceil_div(nq, per_block), 32 * per_block, 0, st>>>(red, nblk, nq, out);
  LAUNCH_CHECK();
}

// ---- projections ---------------------------------------------------------------------------------
// red[(l*k + c)][blk] = Σ_{i in block} Q[i,l]·X[i,c]
__global__ void proj_partial_kernel(const float* __restrict__ Q, int64_t ldq, int cq,
                                    const float* __restrict__ X, int64_t ldx, int64_t n, int k,
                                    double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y % k, l = blockIdx.y / k;
  const int64_t i0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int64_t i1 = min64(n, i0 + kRowsPerBlock);
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x)
    acc += (double)Q[(int64_t)l * ldq + i] * (double)X[(int64_t)c * ldx + i];
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) red[(int64_t)(l * k + c) * nblk + blockIdx.x] = s;
  (void)cq;
}

// X[i,c] += −Σ_l Q[i,l]·QtX[l,c] (+ tau0·V[i,c] when V != nullptr)
__global__ void proj_apply_kernel(const float* __restrict__ Q, int64_t ldq, int cq,
                                  float* __restrict__ X, int64_t ldx, int64_t n, int k,
                                  const double* __restrict__ QtX, const float* __restrict__ V,
                                  int64_t ldv, float tau0)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  double acc = 0.0;
  for (int l = 0; l < cq; ++l) acc += (double)Q[(int64_t)l * ldq + i] * QtX[l * k + c];
  float x = X[(int64_t)c * ldx + i];
  x = x - (float)acc;
  if (V) x += tau0 * V[(int64_t)c * ldv + i];
  X[(int64_t)c * ldx + i] = x;
}

void proj_coeffs(slemm_geno* g, const float* X, int64_t ldx, int k, double* d_QtX)
{
  if (g->c == 0) return;
  const int nblk = (int)ceil_div(g->n, kRowsPerBlock);
  double* red = (double*)g->ws_red.ensure((size_t)nblk * g->c * k * sizeof(double));
  dim3 grid(nblk, g->c * k);
  proj_partial_kernel<<<grid, kRedThreads, 0, g->stream>>>(g->Q.as<float>(), g->n_pad, g->c, X, ldx,
                                                           g->n, k, red, nblk);
  LAUNCH_CHECK();
  reduce_partials(red, nblk, g->c * k, d_QtX, g->stream);
}

void proj_apply(slemm_geno* g, float* X, int64_t ldx, int k, const double* d_QtX)
{
  if (g->c == 0) return;
  dim3 grid((unsigned)ceil_div(g->n, 256), k);
  proj_apply_kernel<<<grid, 256, 0, g->stream>>>(g->Q.as<float>(), g->n_pad, g->c, X, ldx, g->n, k,
                                                 d_QtX, nullptr, 0, 0.f);
  LAUNCH_CHECK();
}

// ---- column dots ------------------------------------------------------------------------------------
__global__ void col_dots_partial_kernel(const float* __restrict__ a, int64_t lda,
                                        const float* __restrict__ b, int64_t ldb, int64_t n,
                                        double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int64_t i1 = min64(n, i0 + kRowsPerBlock);
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double x = a[(int64_t)c * lda + i];
    const double y = b ? (double)b[(int64_t)c * ldb + i] : x;
    acc += x * y;
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

void col_dots(slemm_geno* g, const float* a, int64_t lda, const float* b, int64_t ldb, int64_t n,
              int k, double* d_out)
{
  const int nblk = (int)ceil_div(n, kRowsPerBlock);
  double* red = (double*)g->ws_red.ensure((size_t)nblk * k * sizeof(double));
  dim3 grid(nblk, k);
  col_dots_partial_kernel<<<grid, kRedThreads, 0, g->stream>>>(a, lda, b, ldb, n, red, nblk);
  LAUNCH_CHECK();
  reduce_partials(red, nblk, k, d_out, g->stream);
}

// ---- dense-operand builders ------------------------------------------------------------------------
// Writes x into the dense operand: FP32 row c (npieces == 0) or BF16 pieces p·k + c, and returns
// the exact value the products will see.
__device__ __forceinline__ double store_operand(float x, int npieces, void* Bv, int64_t K_pad,
                                                int k, int c, int64_t kidx)
{
  if (npieces == 0) {
    static_cast<float*>(Bv)[(int64_t)c * K_pad + kidx] = x;
    return (double)x;
  }
  __nv_bfloat16* B = static_cast<__nv_bfloat16*>(Bv);
  double sum = 0.0;
  float r = x;
  for (int p = 0; p < npieces; ++p) {
    const __nv_bfloat16 h = __float2bfloat16_rn(r);
    const float hf = __bfloat162float(h);
    B[(int64_t)(p * k + c) * K_pad + kidx] = h;
    sum += (double)hf;
    r = r - hf;   // exact in FP32
  }
  return sum;
}

// Direction-1 operand (K = individuals): x = in[i,c]; for the first nq columns
// x −= Σ_l Q[i,l]·QtV[l,c]; optionally x *= rr[i]; rows i ≥ n are 0.
// red[c][blk] = Σ_i stored(x).
__global__ void prologue_indiv_kernel(const float* __restrict__ in, int64_t ld, int64_t n,
                                      int64_t n_pad, int k, const float* __restrict__ Q,
                                      int64_t ldq, int cq, const double* __restrict__ QtV, int nq,
                                      const float* __restrict__ rr, int npieces, void* B,
                                      double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int64_t i1 = min64(n_pad, i0 + kRowsPerBlock);
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    float x = 0.f;
    if (i < n) {
      x = in[(int64_t)c * ld + i];
      if (QtV && c < nq) {
        double p = 0.0;
        for (int l = 0; l < cq; ++l) p += (double)Q[(int64_t)l * ldq + i] * QtV[l * nq + c];
        x = x - (float)p;
      }
      if (rr) x *= rr[i];
    }
    acc += store_operand(x, npieces, B, n_pad, k, c, i);
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// Sum over split-K partials and BF16 pieces of column c, row r.
__device__ __forceinline__ float gather_D(const float* __restrict__ D, int splits, int N,
                                          int64_t M_pad, int pieces, int k, int c, int64_t r)
{
  float acc = 0.f;
  for (int s = 0; s < splits; ++s)
    for (int p = 0; p < pieces; ++p) acc += D[((int64_t)s * N + p * k + c) * M_pad + r];
  return acc;
}

// Direction-1 finalize (rows = SNPs): val = raw − gm_j·colsum_c, times w_j when use_w.
// mode 0: out[j,c] = val (j < m).  mode 1: val becomes the direction-2 operand (K = SNPs) and
// red[c][blk] = Σ_j gm_j·stored(val).
__global__ void finalize_snp_kernel(const float* __restrict__ D, int splits, int N, int64_t m_pad,
                                    int pieces, int k, int64_t m, const float* __restrict__ gm,
                                    const float* __restrict__ w, const double* __restrict__ colsum,
                                    int mode, float* __restrict__ out, int64_t ldo, int npieces2,
                                    void* B2, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t j0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int64_t j1 = min64(m_pad, j0 + kRowsPerBlock);
  const double cs = colsum[c];
  double acc = 0.0;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    float val = 0.f;
    if (j < m) {
      const float raw = gather_D(D, splits, N, m_pad, pieces, k, c, j);
      val = (float)((double)raw - (double)gm[j] * cs);
      if (w) val *= w[j];
    }
    if (mode == 0) {
      if (j < m) out[(int64_t)c * ldo + j] = val;
    } else {
      const double st = store_operand(val, npieces2, B2, m_pad, k, c, j);
      acc += (double)gm[j] * st;
    }
  }
  if (mode == 1) {
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
  }
}

// Direction-2 operand straight from an m×k input (matvec): stored(in) and red = Σ gm·stored.
__global__ void prologue_snp_kernel(const float* __restrict__ in, int64_t ld, int64_t m,
                                    int64_t m_pad, int k, const float* __restrict__ gm,
                                    int npieces, void* B, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t j0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int64_t j1 = min64(m_pad, j0 + kRowsPerBlock);
  double acc = 0.0;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const float x = (j < m) ? in[(int64_t)c * ld + j] : 0.f;
    const double st = store_operand(x, npieces, B, m_pad, k, c, j);
    acc += (double)gm[j] * st;
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// Direction-2 finalize (rows = individuals) of columns c0 + blockIdx.y: val = raw − t_c, times
// rr_i when rr != nullptr, plus tau0·v when V != nullptr.  out[i,c] = val for i < n.
__global__ void finalize_indiv_kernel(const float* __restrict__ D, int splits, int N,
                                      int64_t n_pad, int pieces, int k, int64_t n,
                                      const double* __restrict__ tsum, const float* __restrict__ rr,
                                      const float* __restrict__ V, int64_t ldv, float tau0,
                                      float* __restrict__ out, int64_t ldo, int c0)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = c0 + blockIdx.y;
  if (i >= n) return;
  const float raw = gather_D(D, splits, N, n_pad, pieces, k, c, i);
  float val = (float)((double)raw - tsum[c]);
  if (rr) val *= rr[i];
  if (V) val += tau0 * V[(int64_t)c * ldv + i];
  out[(int64_t)c * ldo + i] = val;
}

// ---- one packed pass ---------------------------------------------------------------------------------
struct PassPlan {
  bool tc;
  int pieces;   // BF16 pieces (tc) or 1 (simt)
  int N;        // columns of D
  int splits;
};

static PassPlan plan_pass(const slemm_geno* g, int k, int64_t M_pad, int64_t K_pad)
{
  PassPlan p;
  p.tc = g->prec != SLEMM_PREC_FP32;
  p.pieces = g->prec == SLEMM_PREC_BF16X3 ? 3 : (g->prec == SLEMM_PREC_BF16X2 ? 2 : 1);
  p.N = p.tc ? (int)round_up((int64_t)p.pieces * k, 16) : k;
  const int64_t M_tiles = M_pad / kTileM, K_tiles = K_pad / kTileK;
  p.splits = p.tc ? choose_splits(M_pad / gemm_tc_rows_per_cta(p.N), K_tiles, 1, num_sms())
                  : choose_splits(M_tiles, K_tiles, 8, num_sms());
  return p;
}

static int max_group(const slemm_geno* g)
{
  if (g->per_vector) return 1;
  if (g->prec == SLEMM_PREC_BF16X2) return 128;
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
      if (s.tc == r.tc && s.N == r.N && s.k == r.k && s.dir == r.dir && s.pieces == r.pieces) {
        s.launches += 1;
        s.ms += ms;
        found = true;
        break;
      }
    if (!found) g->prof_stats.push_back({r.tc, r.N, r.k, r.pieces, r.dir, 1, (double)ms});
    g->event_pool.push_back(r.start);
    g->event_pool.push_back(r.stop);
  }
  g->prof_pending.clear();
}

static void run_gemm(slemm_geno* g, const PassPlan& p, const uint8_t* A, int64_t M_pad,
                     int64_t K_pad, const void* B, float* D, int* err, int k, int dir)
{
  GemmArgs a{A, M_pad, K_pad, B, p.N, D, p.splits, err};
  slemm_geno::GemmRecord rec{};
  if (g->profiling) {
    if (g->prof_pending.size() >= 512) profile_collect(g);
    rec = {take_event(g), take_event(g), p.tc ? 1 : 0, p.N, k, p.pieces, p.splits, dir};
    CUDA_TRY(cudaEventRecord(rec.start, g->stream));
  }
  if (p.tc) gemm_tc(a, g->stream);
  else gemm_simt(a, g->stream);
  if (g->profiling) {
    CUDA_TRY(cudaEventRecord(rec.stop, g->stream));
    g->prof_pending.push_back(rec);
  }
}

// Device scratch: small FP64 vectors + error word.
struct Small {
  double* colsum;   // k
  double* tsum;     // k
  double* QtV;      // 64·k
  double* QtT;      // 64·k
  int* err;         // the handle's error word
};

static Small small_ws(slemm_geno* g, int k)
{
  const size_t nd = (size_t)k * 2 + (size_t)64 * k * 2;
  uint8_t* base = (uint8_t*)g->ws_small.ensure(nd * sizeof(double));
  Small s;
  s.colsum = (double*)base;
  s.tsum = s.colsum + k;
  s.QtV = s.tsum + k;
  s.QtT = s.QtV + (size_t)64 * k;
  s.err = g->err.as<int>();
  return s;
}

// One operator application on a column group (k ≤ max_group).  For the H0 operators (kind
// LDET, or QUADFORM) the first nq columns get the projections of H0_quadform_mv and the others
// are plain H0_ldet_mv columns, so one block can carry both kinds of seed systems.
static void op_group(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
                     float* out, int64_t ld_out, int nq)
{
  if (kind == SLEMM_OP_QUADFORM) kind = SLEMM_OP_LDET;   // nq carries the projected columns
  cudaStream_t st = g->stream;
  Small sm = small_ws(g, k);
  const bool dir1 = kind != SLEMM_OP_MATVEC;                          // needs Zᵀ pass
  const bool dir2 = kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET || kind == SLEMM_OP_MATVEC;
  const PassPlan p1 = plan_pass(g, k, g->m_pad, g->n_pad);             // M = SNPs, K = indiv
  const PassPlan p2 = plan_pass(g, k, g->n_pad, g->m_pad);             // M = indiv, K = SNPs
  const int np1 = p1.tc ? p1.pieces : 0, np2 = p2.tc ? p2.pieces : 0;
  const size_t b1 = dir1 ? (p1.tc ? (size_t)p1.N * g->n_pad * 2 : (size_t)k * g->n_pad * 4) : 0;
  const size_t b2 = dir2 ? (p2.tc ? (size_t)p2.N * g->m_pad * 2 : (size_t)k * g->m_pad * 4) : 0;
  uint8_t* Bbuf = (uint8_t*)g->ws_B.ensure(b1 + b2);
  void* B1 = Bbuf;
  void* B2 = Bbuf + b1;
  const size_t d1 = dir1 ? (size_t)p1.splits * p1.N * g->m_pad : 0;
  const size_t d2 = dir2 ? (size_t)p2.splits * p2.N * g->n_pad : 0;
  float* D = (float*)g->ws_D.ensure(std::max(d1, d2) * sizeof(float));
  const int nblk_n = (int)ceil_div(g->n_pad, kRowsPerBlock);
  const int nblk_m = (int)ceil_div(g->m_pad, kRowsPerBlock);
  double* red = (double*)g->ws_red.ensure((size_t)std::max(nblk_n, nblk_m) * k * sizeof(double) +
                                          (size_t)ceil_div(g->n, kRowsPerBlock) * 64 * k * sizeof(double));
  // zero the BF16 padding rows (pieces·k … N) of both operands
  if (p1.tc && dir1 && p1.N > p1.pieces * k)
    CUDA_TRY(cudaMemsetAsync((uint16_t*)B1 + (size_t)p1.pieces * k * g->n_pad, 0,
                             (size_t)(p1.N - p1.pieces * k) * g->n_pad * 2, st));
  if (p2.tc && dir2 && p2.N > p2.pieces * k)
    CUDA_TRY(cudaMemsetAsync((uint16_t*)B2 + (size_t)p2.pieces * k * g->m_pad, 0,
                             (size_t)(p2.N - p2.pieces * k) * g->m_pad * 2, st));

  // H0 operators: the first nq columns are projected (H0_quadform_mv), the rest are not (H0_ldet_mv)
  const bool h0 = kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET;

  if (dir1) {
    // ---- prologue 1: v_adj = rr∘(v − QQᵀv) (quadform), rr∘v (ldet), v (rmatvec) ----
    const double* QtV = nullptr;
    if (h0 && nq > 0 && g->c > 0) {
      proj_coeffs(g, in, ld_in, nq, sm.QtV);
      QtV = sm.QtV;
    }
    dim3 grid(nblk_n, k);
    prologue_indiv_kernel<<<grid, kRedThreads, 0, st>>>(
        in, ld_in, g->n, g->n_pad, k, g->Q.as<float>(), g->n_pad, g->c, QtV, nq,
        h0 ? g->rr.as<float>() : nullptr, np1, B1, red, nblk_n);
    LAUNCH_CHECK();
    reduce_partials(red, nblk_n, k, sm.colsum, st);
    // ---- pass 1: Cntᵀ over individuals ----
    run_gemm(g, p1, g->G.as<uint8_t>(), g->m_pad, g->n_pad, B1, D, sm.err, k, 1);
    // ---- finalize 1 ----
    dim3 gridm(nblk_m, k);
    const float* wsc = (kind == SLEMM_OP_RMATVEC) ? nullptr : g->w.as<float>();
    if (h0) {
      finalize_snp_kernel<<<gridm, kRedThreads, 0, st>>>(
          D, p1.splits, p1.N, g->m_pad, p1.pieces, k, g->m, g->gm.as<float>(), wsc, sm.colsum, 1,
          nullptr, 0, np2, B2, red, nblk_m);
      LAUNCH_CHECK();
      reduce_partials(red, nblk_m, k, sm.tsum, st);
    } else {
      finalize_snp_kernel<<<gridm, kRedThreads, 0, st>>>(
          D, p1.splits, p1.N, g->m_pad, p1.pieces, k, g->m, g->gm.as<float>(), wsc, sm.colsum, 0,
          out, ld_out, 0, nullptr, nullptr, 0);
      LAUNCH_CHECK();
      return;
    }
  } else {
    // matvec: operand straight from the m×k input
    dim3 gridm(nblk_m, k);
    prologue_snp_kernel<<<gridm, kRedThreads, 0, st>>>(in, ld_in, g->m, g->m_pad, k,
                                                       g->gm.as<float>(), np2, B2, red, nblk_m);
    LAUNCH_CHECK();
    reduce_partials(red, nblk_m, k, sm.tsum, st);
  }
  // ---- pass 2: Cnt over SNPs ----
  run_gemm(g, p2, g->GT.as<uint8_t>(), g->n_pad, g->m_pad, B2, D, sm.err, k, 2);
  // ---- finalize 2 ----
  const unsigned gx = (unsigned)ceil_div(g->n, 256);
  if (kind == SLEMM_OP_MATVEC) {
    finalize_indiv_kernel<<<dim3(gx, k), 256, 0, st>>>(D, p2.splits, p2.N, g->n_pad, p2.pieces, k, g->n,
                                                       sm.tsum, nullptr, nullptr, 0, 0.f, out, ld_out, 0);
    LAUNCH_CHECK();
    return;
  }
  // ldet columns nq … k−1: out = rr∘(Z_c W Z_cᵀ rr∘v) + τ0 v
  if (nq < k) {
    finalize_indiv_kernel<<<dim3(gx, k - nq), 256, 0, st>>>(D, p2.splits, p2.N, g->n_pad, p2.pieces, k,
                                                            g->n, sm.tsum, g->rr.as<float>(), in, ld_in,
                                                            tau0, out, ld_out, nq);
    LAUNCH_CHECK();
  }
  // quadform columns 0 … nq−1: T = rr∘(Z_c W Z_cᵀ v_adj); out = T + τ0 v − QQᵀT
  if (nq > 0) {
    finalize_indiv_kernel<<<dim3(gx, nq), 256, 0, st>>>(D, p2.splits, p2.N, g->n_pad, p2.pieces, k,
                                                        g->n, sm.tsum, g->rr.as<float>(), nullptr, 0, 0.f,
                                                        out, ld_out, 0);
    LAUNCH_CHECK();
    if (g->c > 0) proj_coeffs(g, out, ld_out, nq, sm.QtT);
    proj_apply_kernel<<<dim3(gx, nq), 256, 0, st>>>(g->Q.as<float>(), g->n_pad, g->c, out, ld_out, g->n,
                                                    nq, sm.QtT, in, ld_in, tau0);
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
        info[5 * r + 0] = s.tc;
        info[5 * r + 1] = s.N;
        info[5 * r + 2] = s.k;
        info[5 * r + 3] = s.pieces;
        info[5 * r + 4] = s.dir;
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
