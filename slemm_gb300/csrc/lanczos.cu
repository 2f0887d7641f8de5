// lanczos.cu — Lanczos seed systems, shifted solves and the batched tridiagonal eigensolve.
//
// L_Seed (src/reml.cpp:246-339): per-column Lanczos on a block B (n×t) with the operator of
// ops.cu.  The basis vectors are FP32 in HBM like the reference's std::vector<MatrixXf>; the
// vector updates run in FP32 (with the FP64 scalars applied as double-float pairs) and every
// scalar of the three-term recurrence (δ = uᵀAu, β = ‖·‖, the CG coefficients γ, ω, ρ and the
// residual test) is accumulated to FP64 accuracy (reduce.cuh) and kept in FP64.  One step is
// three vector kernels whose block partials the next kernel sums itself in a fixed order, and one
// small kernel that writes the step's scalars into mapped host memory: one synchronisation per
// step, no copies.
//
// L_Solve (src/reml.cpp:369-431): the reference rebuilds CG on (A + σI) from the stored basis
// step by step.  Unrolling its recurrences (P_0 = B, P_j = ρ_j U_j + ω_{j−1} P_{j−1},
// X = Σ_j γ_j P_j) gives X = S_0·B + Σ_{i≥1} ρ_i S_i U_i with S_i = γ_i + ω_i S_{i+1}; the
// host evaluates those FP64 coefficients with the reference's stopping rule and one kernel
// forms the weighted sum over the stored basis — one pass instead of one pass per step.
//
// Tridiagonal eigensolve (src/reml.cpp:638-646): per probe, implicit QL with Wilkinson shifts in
// FP64 on the host (a few hundred flops per probe), tracking only the first row of the
// eigenvector matrix (all the quadrature needs).
#include "internal.h"
#include "reduce.cuh"

#include <chrono>
#include <thread>

struct slemm_lseed {
  slemm_geno* g = nullptr;
  int kind = 0;
  float tau0 = 0.f;
  int t = 0;
  int iters = 0;   // j: basis holds U_0 … U_j
  int64_t n = 0;
  cudaStream_t st = nullptr;                 // the handle's stream: buffers are stream-ordered on it
  static constexpr int kChunk = 16;          // basis blocks per allocation
  std::vector<slemm::DevBuf*> chunks;        // each holds kChunk blocks of n×t FP32
  slemm::DevBuf B;                           // right-hand side block (n×t)
  std::vector<double> beta;                  // (iters+1) × t, row j = step j
  std::vector<double> delta;                 // iters × t
  std::vector<double> unorm;                 // (iters+1) × t, ‖U_j‖ of the stored FP32 vectors
  std::vector<double> bnorm;                 // t
  // Column groups that share one stopping rule (the reference runs each group as its own
  // L_Seed call); group_iters[g] is the step at which group g met the tolerance.
  std::vector<int> group_start, group_iters;
  slemm::DevBuf solve_coef, solve_blk;       // reused by every shifted solve
  // SLEMM_LANCZOS_* bits of the handle when the seed was run (REORTH: every new vector is made
  // orthogonal to the whole stored basis of its column).
  int mode = 0;
  slemm::DevBuf ro_ptr, ro_red, ro_coef;     // reorthogonalisation: block pointers, dot partials, coefficients
  std::vector<const float*> ro_host;         // host copy of the block pointers uploaded so far
  ~slemm_lseed()
  {
    for (auto* c : chunks) delete c;
  }
  float* block(int j)
  {
    const int c = j / kChunk;
    while ((int)chunks.size() <= c) {
      auto* b = new slemm::DevBuf(st);
      b->pool = slemm::own_pool(g->device, slemm::Pool::Basis);
      b->ensure((size_t)kChunk * n * t * sizeof(float));
      chunks.push_back(b);
    }
    return chunks[c]->as<float>() + (size_t)(j % kChunk) * n * t;
  }
};

namespace slemm {

constexpr int kLzRows = 4096;     // rows of one block of the vector kernels
constexpr int kLzThreads = 256;

// red[c][blk] = Σ src²  (norm partials of the right-hand side)
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_norm_kernel(const float* __restrict__ src, int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int c = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kLzRows, i1 = min64(n, i0 + kLzRows);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kLzThreads * V) {
    float x[V];
    ldv<V>(src + (int64_t)c * n + i, x);
#pragma unroll
    for (int q = 0; q < V; ++q) df_fma(acc, x[q], x[q]);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// tmp ← tmp − β·U_prev with β = √(Σ nrm_prev partials) (skipped at step 0);
// red_dot[c][blk] = Σ U_cur·tmp
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_dot_kernel(float* __restrict__ tmp, const float* __restrict__ Ucur, const float* __restrict__ Uprev,
              const double* __restrict__ nrm_prev, int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  __shared__ float sb[2];
  const int c = blockIdx.y;
  float bh = 0.f, bl = 0.f;
  if (Uprev) block_scalar([&] { return sqrt(warp_sum_partials(nrm_prev + (int64_t)c * nblk, nblk)); }, sb, bh, bl);
  const int64_t i0 = (int64_t)blockIdx.x * kLzRows, i1 = min64(n, i0 + kLzRows);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kLzThreads * V) {
    const int64_t o = (int64_t)c * n + i;
    float x[V], u[V];
    ldv<V>(tmp + o, x);
    ldv<V>(Ucur + o, u);
    if (Uprev) {
      float p[V];
      ldv<V>(Uprev + o, p);
#pragma unroll
      for (int q = 0; q < V; ++q) x[q] = __fmaf_rn(-bl, p[q], __fmaf_rn(-bh, p[q], x[q]));
      stv<V>(tmp + o, x);
    }
#pragma unroll
    for (int q = 0; q < V; ++q) df_fma(acc, u[q], x[q]);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// tmp ← tmp − δ·U_cur with δ = Σ dot partials; red_nrm[c][blk] = Σ tmp²
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_orth_kernel(float* __restrict__ tmp, const float* __restrict__ Ucur, const double* __restrict__ dot,
               int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  __shared__ float sb[2];
  const int c = blockIdx.y;
  float dh, dlo;
  block_scalar([&] { return warp_sum_partials(dot + (int64_t)c * nblk, nblk); }, sb, dh, dlo);
  const int64_t i0 = (int64_t)blockIdx.x * kLzRows, i1 = min64(n, i0 + kLzRows);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kLzThreads * V) {
    const int64_t o = (int64_t)c * n + i;
    float x[V], u[V];
    ldv<V>(tmp + o, x);
    ldv<V>(Ucur + o, u);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      x[q] = __fmaf_rn(-dlo, u[q], __fmaf_rn(-dh, u[q], x[q]));
      df_fma(acc, x[q], x[q]);
    }
    stv<V>(tmp + o, x);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// U_next ← src / √(Σ nrm partials); red_un[c][blk] = Σ U_next²
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_scale_kernel(float* __restrict__ Unext, const float* __restrict__ src, const double* __restrict__ nrm,
                int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  __shared__ float sb[2];
  const int c = blockIdx.y;
  float ih, il;
  block_scalar([&] { return 1.0 / sqrt(warp_sum_partials(nrm + (int64_t)c * nblk, nblk)); }, sb, ih, il);
  const int64_t i0 = (int64_t)blockIdx.x * kLzRows, i1 = min64(n, i0 + kLzRows);
  DF acc;
  for (int64_t i = i0 + threadIdx.x * V; i < i1; i += kLzThreads * V) {
    const int64_t o = (int64_t)c * n + i;
    float x[V];
    ldv<V>(src + o, x);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      x[q] = __fmaf_rn(x[q], ih, __fmul_rn(x[q], il));
      df_fma(acc, x[q], x[q]);
    }
    stv<V>(Unext + o, x);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// ---- reorthogonalisation (opt-in, SLEMM_LANCZOS_REORTH) ----------------------------------------
// The reference runs the plain three-term recurrence (src/reml.cpp:293-322).  In finite precision
// its vectors lose orthogonality once Ritz values converge, which on ill-conditioned systems
// (window-weighted GREML) adds steps and makes the stopping step depend on rounding.  The opt-in
// mode removes from each new vector w (column c, after the recurrence) its components along every
// stored vector of that column by classical Gram–Schmidt with FP64-accurate coefficients:
//   d_i = U_i[:,c]·w (double-float sums), w ← w − Σ_i d_i·U_i[:,c] (double-float sum, rounded once).
// Two streaming passes over the stored basis per step: the dots, then the update.
constexpr int kRoRows = 8192;     // rows of one block of the dot pass
constexpr int kRoGroup = 8;       // stored vectors whose block sums share one barrier

// red[(i·t + c)·nblk + blk] = Σ_{rows of blk} U_i[r,c]·w[r,c] for i = 0 … J
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_reorth_dot_kernel(const float* __restrict__ w, const float* const* __restrict__ blocks, int J, int t,
                     int64_t n, double* __restrict__ red, int nblk)
{
  constexpr int P = kRoRows / (kLzThreads * V);
  __shared__ double sh[kRoGroup][kLzThreads / 32];
  const int c = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = (int64_t)blockIdx.x * kRoRows;
  float x[P][V];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    const int64_t r = r0 + ((int64_t)p * kLzThreads + threadIdx.x) * V;
    if (r < n) ldv<V>(w + (int64_t)c * n + r, x[p]);
    else
#pragma unroll
      for (int q = 0; q < V; ++q) x[p][q] = 0.f;
  }
  for (int i0 = 0; i0 <= J; i0 += kRoGroup) {
    const int ni = min(kRoGroup, J + 1 - i0);
    for (int q = 0; q < ni; ++q) {
      const float* U = blocks[i0 + q] + (int64_t)c * n;
      DF acc;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const int64_t r = r0 + ((int64_t)p * kLzThreads + threadIdx.x) * V;
        if (r < n) {
          float u[V];
          ldv<V>(U + r, u);
#pragma unroll
          for (int e = 0; e < V; ++e) df_fma(acc, u[e], x[p][e]);
        }
      }
      double s = df_value(acc);
      for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) sh[q][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x < ni) {
      double s = 0.0;
      for (int k = 0; k < kLzThreads / 32; ++k) s += sh[threadIdx.x][k];
      red[((int64_t)(i0 + threadIdx.x) * t + c) * nblk + blockIdx.x] = s;
    }
    __syncthreads();
  }
}

// coef2[2q], coef2[2q+1] = hi, lo of Σ_b red[q·nblk + b] for q < nq (block order)
__global__ void lz_reorth_coef_kernel(const double* __restrict__ red, int nblk, int nq, float* __restrict__ coef2)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) split_double(sum_partials(red + (int64_t)q * nblk, nblk), coef2[2 * q], coef2[2 * q + 1]);
}

// w[r,c] ← w[r,c] − Σ_{i ≤ J} d_{i,c}·U_i[r,c] (double-float sum rounded once);
// red_nrm[c][blk] = Σ w² of the result (partials over blocks of kLzRows rows, as lz_orth writes them)
template <int V>
__global__ void __launch_bounds__(kLzThreads)
lz_reorth_update_kernel(float* __restrict__ w, const float* const* __restrict__ blocks, int J, int t,
                        const float* __restrict__ coef2, int64_t n, double* __restrict__ red, int nblk)
{
  extern __shared__ float sco[];   // (J+1) hi/lo pairs of this column
  __shared__ double sh[32];
  const int c = blockIdx.y;
  for (int i = threadIdx.x; i <= J; i += kLzThreads) {
    sco[2 * i] = coef2[2 * ((int64_t)i * t + c)];
    sco[2 * i + 1] = coef2[2 * ((int64_t)i * t + c) + 1];
  }
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * kLzRows, i1 = min64(n, i0 + kLzRows);
  DF acc;
  for (int64_t r = i0 + threadIdx.x * V; r < i1; r += kLzThreads * V) {
    const int64_t o = (int64_t)c * n + r;
    DF a[V];
#pragma unroll 4
    for (int i = 0; i <= J; ++i) {
      float u[V];
      ldv<V>(blocks[i] + o, u);
      const float ch = sco[2 * i], cl = sco[2 * i + 1];
#pragma unroll
      for (int e = 0; e < V; ++e) {
        df_fma(a[e], ch, u[e]);
        a[e].lo = __fmaf_rn(cl, u[e], a[e].lo);
      }
    }
    float x[V];
    ldv<V>(w + o, x);
#pragma unroll
    for (int e = 0; e < V; ++e) {
      x[e] = __fsub_rn(__fsub_rn(x[e], a[e].hi), a[e].lo);
      df_fma(acc, x[e], x[e]);
    }
    stv<V>(w + o, x);
  }
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[(int64_t)c * nblk + blockIdx.x] = s;
}

// out[c] = Σ dot, out[t+c] = Σ nrm, out[2t+c] = Σ un (the consumers' order); out[3t] = error word.
// One block per column, one warp per quantity (dot, norm, unscaled norm), each summed over the
// blocks' partials in warp_sum_partials' fixed order (the bits sum_partials gives in one thread);
// a thread per column summing all three serially over strided partials took ≈57 µs per step.
// out[w·stride + c] for block c; err_out[0] = the kernels' error word.
__global__ void __launch_bounds__(96) lz_final_kernel(const double* __restrict__ dot, const double* __restrict__ nrm,
                                                      const double* __restrict__ un, int stride, int nblk,
                                                      const int* __restrict__ err, double* __restrict__ out,
                                                      double* __restrict__ err_out)
{
  const int c = blockIdx.x;
  const int w = threadIdx.x >> 5;   // warp-uniform
  const double* src = w == 0 ? dot : (w == 1 ? nrm : un);
  const double s = src ? warp_sum_partials(src + (int64_t)c * nblk, nblk) : 0.0;
  if ((threadIdx.x & 31) == 0) out[(int64_t)w * stride + c] = s;
  if (c == 0 && threadIdx.x == 0) err_out[0] = (double)*err;
}

// X[i,c] = coefB[c]·B[i,c] + Σ_{j=1..J} coef[j·t + c]·U_j[i,c]
// (columns c0 … c0+tc−1 of the block; coef is steps × tc FP64 values held as hi+lo FP32 pairs,
// coef2[2q] + coef2[2q+1]).  The sum is carried as a double-float pair — each product by
// TwoProd, the low coefficient word by one more FMA — so X is the FP64 combination rounded once,
// at FP32 rates (a per-element FP64 FMA chain would bound this kernel by GB300's FP64 pipe, not
// by the stored basis it streams).
__global__ void lz_combine_kernel(float* __restrict__ X, int64_t ldx, const float* __restrict__ B,
                                  const float* const* __restrict__ blocks, int J,
                                  const float* __restrict__ coef2, int64_t n, int c0, int tc)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  const int64_t o = (int64_t)(c0 + c) * n + i;
  DF acc;
  {
    const float b = B[o];
    df_fma(acc, coef2[2 * c], b);
    acc.lo = __fmaf_rn(coef2[2 * c + 1], b, acc.lo);
  }
  for (int j = 1; j <= J; ++j) {
    const float u = blocks[j][o];
    const int64_t q = (int64_t)j * tc + c;
    df_fma(acc, coef2[2 * q], u);
    acc.lo = __fmaf_rn(coef2[2 * q + 1], u, acc.lo);
  }
  X[(int64_t)c * ldx + i] = __fadd_rn(acc.hi, acc.lo);
}

}  // namespace slemm

using namespace slemm;

namespace slemm {

// Runs L_Seed on a device RHS block B (n×t, ld = n).  Returns the seed object.
slemm_lseed* lanczos_seed_device(slemm_geno* g, int kind, float tau0, const float* dB, int t,
                                 float tol, int maxit, bool verbose, std::vector<int> groups,
                                 int p_freq, int nq)
{
  // projected (H0_quadform_mv) leading columns; QUADFORM projects all of them
  const int nq_eff = (kind == SLEMM_OP_QUADFORM) ? t : std::max(0, std::min(nq, t));
  if (groups.empty()) groups.push_back(t);
  {
    int tot = 0;
    for (int x : groups) {
      CHECK_ARG(x >= 1, "empty column group");
      tot += x;
    }
    CHECK_ARG(tot == t, "column groups do not add up to t");
  }
  CHECK_ARG(kind == SLEMM_OP_QUADFORM || kind == SLEMM_OP_LDET, "seed operator must be QUADFORM or LDET");
  CHECK_ARG(t >= 1 && maxit >= 2, "bad t or maxit");
  const int64_t n = g->n;
  cudaStream_t st = g->stream;
  auto* S = new slemm_lseed();
  try {
    S->g = g;
    S->st = st;
    for (slemm::DevBuf* b : {&S->B, &S->solve_coef, &S->solve_blk}) {
      b->stream = st;
      b->ordered = true;
    }
    S->kind = kind;
    S->tau0 = tau0;
    S->t = t;
    S->n = n;
    {
      int c0 = 0;
      for (int x : groups) {
        S->group_start.push_back(c0);
        c0 += x;
      }
      S->group_start.push_back(c0);
      S->group_iters.assign(groups.size(), -1);
    }
    S->B.ensure((size_t)n * t * sizeof(float));
    CUDA_TRY(cudaMemcpyAsync(S->B.p, dB, (size_t)n * t * sizeof(float), cudaMemcpyDeviceToDevice, st));
    const int nblk = (int)ceil_div(n, kLzRows);
    // partials [t][nblk] of δ (dot), ‖·‖² after orthogonalisation (nrm) and ‖U_{j+1}‖² (un);
    // nrm stays valid until the next step's lz_dot has taken β_{j+1} from it
    DevBuf red(st), tmpb(st);
    red.ensure((size_t)3 * nblk * t * sizeof(double));
    tmpb.ensure((size_t)n * t * sizeof(float));
    double* r_dot = red.as<double>();
    double* r_nrm = r_dot + (size_t)nblk * t;
    double* r_un = r_nrm + (size_t)nblk * t;
    float* tmp = tmpb.as<float>();
    double* d_out = g->scal.ensure((size_t)3 * t + 1);
    const double* h = g->scal.h;
    const bool v4 = (n % 4) == 0;
    const dim3 gr(nblk, t);
    const int* err = g->err.as<int>();
    // Waits for the step's scalars of columns lo … t−1 in the mapped buffer (h[c], h[t + c],
    // h[2t + c]) and checks the kernels' error word (h[3t]).
    auto fetch = [&](const double* dot, int lo) {
      const size_t offr = (size_t)lo * nblk;
      lz_final_kernel<<<(unsigned)(t - lo), 96, 0, st>>>(dot ? dot + offr : nullptr, r_nrm + offr, r_un + offr, t,
                                                        nblk, err, d_out + lo, d_out + 3 * t);
      LAUNCH_CHECK();
      CUDA_TRY(cudaStreamSynchronize(st));
      if (h[3 * t] != 0.0) {
        CUDA_TRY(cudaMemsetAsync(g->err.p, 0, sizeof(int), st));
        SLEMM_THROW(SLEMM_ERR_CUDA, "a tensor-core kernel gave up a bounded wait (code " +
                                        std::to_string((int)h[3 * t]) + ")");
      }
    };

    S->mode = g->lanczos_mode;
    const bool reorth = (S->mode & SLEMM_LANCZOS_REORTH) != 0;
    const int nblkR = (int)ceil_div(n, kRoRows);
    if (reorth) {
      S->ro_ptr.stream = S->ro_red.stream = S->ro_coef.stream = st;
      S->ro_ptr.ordered = S->ro_red.ordered = S->ro_coef.ordered = true;
      S->ro_ptr.ensure((size_t)maxit * sizeof(float*));
      S->ro_red.ensure((size_t)maxit * t * nblkR * sizeof(double));
      S->ro_coef.ensure((size_t)maxit * t * 2 * sizeof(float));
      S->ro_host.reserve(maxit);   // never reallocated while an upload from it is queued
    }
    // w (the new vector of step J, in tmp) ← w minus its components along U_0 … U_J, and the norm
    // partials of the result in r_nrm (what lz_scale and the step's β read).
    auto reorthogonalise = [&](int J) {
      const int have = (int)S->ro_host.size();
      if (have < J + 1) {
        for (int i = have; i <= J; ++i) S->ro_host.push_back(S->block(i));
        CUDA_TRY(cudaMemcpyAsync(S->ro_ptr.as<const float*>() + have, S->ro_host.data() + have,
                                 (size_t)(J + 1 - have) * sizeof(float*), cudaMemcpyHostToDevice, st));
      }
      const float* const* blk = S->ro_ptr.as<const float*>();
      double* rred = S->ro_red.as<double>();
      float* coef = S->ro_coef.as<float>();
      const dim3 grd(nblkR, t);
      if (v4) lz_reorth_dot_kernel<4><<<grd, kLzThreads, 0, st>>>(tmp, blk, J, t, n, rred, nblkR);
      else lz_reorth_dot_kernel<1><<<grd, kLzThreads, 0, st>>>(tmp, blk, J, t, n, rred, nblkR);
      LAUNCH_CHECK();
      const int nq = (J + 1) * t;
      lz_reorth_coef_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, st>>>(rred, nblkR, nq, coef);
      LAUNCH_CHECK();
      const size_t smem = (size_t)2 * (J + 1) * sizeof(float);
      if (v4) lz_reorth_update_kernel<4><<<gr, kLzThreads, smem, st>>>(tmp, blk, J, t, coef, n, r_nrm, nblk);
      else lz_reorth_update_kernel<1><<<gr, kLzThreads, smem, st>>>(tmp, blk, J, t, coef, n, r_nrm, nblk);
      LAUNCH_CHECK();
    };

    // B_norm, U_0 = B / β_0
    if (v4) lz_norm_kernel<4><<<gr, kLzThreads, 0, st>>>(S->B.as<float>(), n, r_nrm, nblk);
    else lz_norm_kernel<1><<<gr, kLzThreads, 0, st>>>(S->B.as<float>(), n, r_nrm, nblk);
    LAUNCH_CHECK();
    if (v4) lz_scale_kernel<4><<<gr, kLzThreads, 0, st>>>(S->block(0), S->B.as<float>(), r_nrm, n, r_un, nblk);
    else lz_scale_kernel<1><<<gr, kLzThreads, 0, st>>>(S->block(0), S->B.as<float>(), r_nrm, n, r_un, nblk);
    LAUNCH_CHECK();
    fetch(nullptr, 0);
    S->bnorm.resize(t);
    S->beta.assign(t, 0.0);
    S->unorm.assign(t, 0.0);
    for (int c = 0; c < t; ++c) {
      S->bnorm[c] = std::sqrt(h[t + c]);
      S->beta[c] = S->bnorm[c];
      S->unorm[c] = std::sqrt(h[2 * t + c]);
      if (!(S->bnorm[c] > 0.0) || !std::isfinite(S->bnorm[c]))
        SLEMM_THROW(SLEMM_ERR_NUMERIC, "right-hand side column " + std::to_string(c) + " has zero or non-finite norm");
    }
    std::vector<double> rho(t), gamma(t, 1.0), omega(t, 0.0);
    for (int c = 0; c < t; ++c) rho[c] = S->bnorm[c];
    int j = 0;
    bool cnvg = false;
    const int ngroups = (int)groups.size();
    std::vector<double> col_res(t, 0.0);
    while (j < maxit - 1) {
      // Leading column groups that have all met the tolerance leave the block: the remaining
      // steps run on the columns from the first unconverged group on (a group's basis past its
      // own step count is never read: solves and moments stop there).  Not with
      // reorthogonalisation, whose passes run over every stored column.
      int lo = 0;
      if (!reorth)
        for (int q = 0; q < ngroups && S->group_iters[q] >= 0; ++q) lo = S->group_start[q + 1];
      const int ta = t - lo;   // ≥ 1: some group is still running
      const size_t off = (size_t)lo * n, offr = (size_t)lo * nblk;
      float* Uj = S->block(j) + off;
      float* Uprev = j > 0 ? S->block(j - 1) + off : nullptr;
      float* Un = S->block(j + 1) + off;
      float* tmpa = tmp + off;
      const dim3 gra(nblk, ta);
      op_device_mixed(g, kind, tau0, Uj, n, ta, tmpa, n, std::max(0, nq_eff - lo));
      if (v4) {
        lz_dot_kernel<4><<<gra, kLzThreads, 0, st>>>(tmpa, Uj, Uprev, r_nrm + offr, n, r_dot + offr, nblk);
        LAUNCH_CHECK();
        lz_orth_kernel<4><<<gra, kLzThreads, 0, st>>>(tmpa, Uj, r_dot + offr, n, r_nrm + offr, nblk);
        LAUNCH_CHECK();
        if (reorth) reorthogonalise(j);
        lz_scale_kernel<4><<<gra, kLzThreads, 0, st>>>(Un, tmpa, r_nrm + offr, n, r_un + offr, nblk);
        LAUNCH_CHECK();
      } else {
        lz_dot_kernel<1><<<gra, kLzThreads, 0, st>>>(tmpa, Uj, Uprev, r_nrm + offr, n, r_dot + offr, nblk);
        LAUNCH_CHECK();
        lz_orth_kernel<1><<<gra, kLzThreads, 0, st>>>(tmpa, Uj, r_dot + offr, n, r_nrm + offr, nblk);
        LAUNCH_CHECK();
        if (reorth) reorthogonalise(j);
        lz_scale_kernel<1><<<gra, kLzThreads, 0, st>>>(Un, tmpa, r_nrm + offr, n, r_un + offr, nblk);
        LAUNCH_CHECK();
      }
      fetch(r_dot, lo);
      double res = 0.0;
      for (int c = 0; c < t; ++c) {
        if (c < lo) {   // a finished group: placeholders, never read
          S->delta.push_back(0.0);
          S->beta.push_back(0.0);
          S->unorm.push_back(0.0);
          continue;
        }
        const double dl = h[c], bt = std::sqrt(h[t + c]), un = std::sqrt(h[2 * t + c]);
        S->delta.push_back(dl);
        S->beta.push_back(bt);
        S->unorm.push_back(un);
        // CG coefficients (src/reml.cpp:304-307)
        const double gm = (j == 0) ? 1.0 / dl : 1.0 / (dl - omega[c] / gamma[c]);
        const double om = (bt * gm) * (bt * gm);
        rho[c] = -bt * gm * rho[c];
        gamma[c] = gm;
        omega[c] = om;
        col_res[c] = std::fabs(rho[c]) * un / S->bnorm[c];
        if (!std::isfinite(dl) || !std::isfinite(bt))
          SLEMM_THROW(SLEMM_ERR_NUMERIC, "non-finite Lanczos coefficient at step " + std::to_string(j));
      }
      ++j;
      bool all = true;
      for (int q = 0; q < ngroups; ++q) {
        if (S->group_iters[q] >= 0) continue;
        double rg = 0.0;
        for (int c = S->group_start[q]; c < S->group_start[q + 1]; ++c) rg = std::max(rg, col_res[c]);
        if (rg <= tol) S->group_iters[q] = j;
        else all = false;
        res = std::max(res, rg);
      }
      if (verbose && j % p_freq == 0) printf("Relative error at step %d is %g\n", j, res);
      if (all) {
        cnvg = true;
        break;
      }
    }
    for (int q = 0; q < ngroups; ++q)
      if (S->group_iters[q] < 0) S->group_iters[q] = j;
    if (verbose) {
      if (cnvg) printf("Converged after %d iterations.\n", j);
      else printf("Failed to converge after %d iterations.\n", maxit);
      fflush(stdout);
    }
    S->iters = j;
  } catch (...) {
    delete S;
    throw;
  }
  return S;
}

// Coefficients of L_Solve for group `grp` at shift σ: X = Σ_i coef[i·tc + c]·V_i[:,c] with
// V_0 = B and V_i = U_i (i ≥ 1), i < steps.  Returns steps.
int solve_coeffs(const slemm_lseed* S, double sigma, double tol, int grp, std::vector<double>& coef)
{
  const int t = S->t;
  const int c0 = S->group_start[grp], tc = S->group_start[grp + 1] - c0;
  const int J = S->group_iters[grp];
  // forward pass: γ, ω, ρ with the reference's stopping rule (src/reml.cpp:404-426)
  std::vector<double> gam((size_t)(J + 1) * tc, 0.0), om((size_t)(J + 1) * tc, 0.0), rho((size_t)(J + 1) * tc, 0.0);
  for (int c = 0; c < tc; ++c) rho[c] = S->bnorm[c0 + c];
  int steps = 0;
  for (int j = 0; j < J; ++j) {
    double res = 0.0;
    for (int c = 0; c < tc; ++c) {
      const int cc = c0 + c;
      const double dl = S->delta[(size_t)j * t + cc] + sigma;
      const double bt = S->beta[(size_t)(j + 1) * t + cc];
      const double g = (j == 0) ? 1.0 / dl : 1.0 / (dl - om[(size_t)(j - 1) * tc + c] / gam[(size_t)(j - 1) * tc + c]);
      gam[(size_t)j * tc + c] = g;
      om[(size_t)j * tc + c] = (bt * g) * (bt * g);
      rho[(size_t)(j + 1) * tc + c] = -bt * g * rho[(size_t)j * tc + c];
      res = std::max(res, std::fabs(rho[(size_t)(j + 1) * tc + c]) * S->unorm[(size_t)(j + 1) * t + cc] / S->bnorm[cc]);
    }
    steps = j + 1;
    if (res <= tol) break;
  }
  // backward pass: S_i = γ_i + ω_i S_{i+1}; X = S_0 B + Σ_{i=1}^{steps-1} ρ_i S_i U_i
  // (the R and P of the last step are not folded into X: X is updated before R).
  coef.assign((size_t)steps * tc, 0.0);
  std::vector<double> Sacc(tc, 0.0);
  for (int i = steps - 1; i >= 0; --i) {
    for (int c = 0; c < tc; ++c) {
      Sacc[c] = gam[(size_t)i * tc + c] + om[(size_t)i * tc + c] * Sacc[c];
      coef[(size_t)i * tc + c] = (i == 0) ? Sacc[c] : rho[(size_t)i * tc + c] * Sacc[c];
    }
  }
  return steps;
}

// mom[i·npairs + p] = Σ_r B[r, a_p]·V_i[r, b_p] for i = 0 … J (V_0 = B, V_i = U_i); double-float
// sums of the stored FP32 vectors, one pass over the basis.  Grid (pairs, row blocks, J + 1): the
// pairs (1 + c² for c covariates) exceed the 65,535 of a grid's y dimension at c = 256.
__global__ void __launch_bounds__(kLzThreads)
lz_moments_kernel(const float* __restrict__ B, const float* const* __restrict__ blocks, int i0,
                  const int2* __restrict__ pairs, int npairs, int64_t n, double* __restrict__ red, int nblk)
{
  __shared__ double sh[32];
  const int p = blockIdx.x, i = i0 + blockIdx.z;   // red holds the steps i0 … of this launch
  const int2 ab = pairs[p];
  const float* Vi = (i == 0) ? B : blocks[i];
  const int64_t r0 = (int64_t)blockIdx.y * kLzRows, r1 = min64(n, r0 + kLzRows);
  DF acc;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += kLzThreads)
    df_fma(acc, B[(int64_t)ab.x * n + r], Vi[(int64_t)ab.y * n + r]);
  const double s = block_sum_d(df_value(acc), sh);
  if (threadIdx.x == 0) red[((int64_t)blockIdx.z * npairs + p) * nblk + blockIdx.y] = s;
}

// out[q] = Σ_b red[q][b] in block order, q < nq
__global__ void lz_sum_kernel(const double* __restrict__ red, int nblk, int nq, double* __restrict__ out)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) out[q] = sum_partials(red + (int64_t)q * nblk, nblk);
}

void lanczos_moments(slemm_lseed* S, const std::vector<std::pair<int, int>>& pairs, int J, std::vector<double>& mom)
{
  const int npairs = (int)pairs.size();
  CHECK_ARG(J >= 0 && J <= S->iters && npairs >= 1, "bad moments request");
  cudaStream_t st = S->g->stream;
  const int nblk = (int)ceil_div(S->n, kLzRows);
  std::vector<const float*> hb(J + 1, nullptr);
  for (int i = 1; i <= J; ++i) hb[i] = S->block(i);
  std::vector<int2> hp(npairs);
  for (int q = 0; q < npairs; ++q) hp[q] = make_int2(pairs[q].first, pairs[q].second);
  DevBuf dblk(st), dpairs(st), dred(st);
  dblk.ensure(hb.size() * sizeof(float*));
  dpairs.ensure(hp.size() * sizeof(int2));
  const int nq = (J + 1) * npairs;
  // the block partials of at most 256 MB of steps at a time (c² pairs for c covariates)
  const size_t per_step = (size_t)npairs * nblk * sizeof(double);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)J + 1, ((size_t)256 << 20) / per_step));
  dred.ensure(per_step * chunk);
  double* out = S->g->scal.ensure((size_t)nq);
  CUDA_TRY(cudaMemcpyAsync(dblk.p, hb.data(), hb.size() * sizeof(float*), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(dpairs.p, hp.data(), hp.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
  for (int i0 = 0; i0 <= J; i0 += chunk) {
    const int ni = std::min(chunk, J + 1 - i0);
    lz_moments_kernel<<<dim3(npairs, nblk, ni), kLzThreads, 0, st>>>(
        S->B.as<float>(), dblk.as<const float*>(), i0, dpairs.as<int2>(), npairs, S->n, dred.as<double>(), nblk);
    LAUNCH_CHECK();
    const int nqc = ni * npairs;
    lz_sum_kernel<<<(unsigned)ceil_div(nqc, 128), 128, 0, st>>>(dred.as<double>(), nblk, nqc,
                                                                 out + (size_t)i0 * npairs);
    LAUNCH_CHECK();
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  mom.assign(S->g->scal.h, S->g->scal.h + nq);
}

// X = (A + σI)^{-1}B for the columns of group `grp` (all columns when the seed has one group),
// using at most that group's basis; X on device (tc columns, ld = ldx).  Returns the CG steps.
int lanczos_solve_device(slemm_lseed* S, double sigma, double tol, float* dX, int64_t ldx, int grp)
{
  const int c0 = S->group_start[grp], tc = S->group_start[grp + 1] - c0;
  cudaStream_t st = S->g->stream;
  std::vector<double> coef;
  const int steps = solve_coeffs(S, sigma, tol, grp, coef);
  std::vector<const float*> hblocks(std::max(steps, 1));
  for (int i = 0; i < steps; ++i) hblocks[i] = (i == 0) ? nullptr : S->block(i);
  DevBuf& dcoef = S->solve_coef;
  DevBuf& dblk = S->solve_blk;
  std::vector<float> coef2(2 * coef.size());
  for (size_t q = 0; q < coef.size(); ++q) {
    coef2[2 * q] = (float)coef[q];
    coef2[2 * q + 1] = (float)(coef[q] - (double)coef2[2 * q]);
  }
  dcoef.ensure(coef2.size() * sizeof(float));
  dblk.ensure(hblocks.size() * sizeof(float*));
  CUDA_TRY(cudaMemcpyAsync(dcoef.p, coef2.data(), coef2.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(dblk.p, hblocks.data(), hblocks.size() * sizeof(float*), cudaMemcpyHostToDevice, st));
  dim3 gr((unsigned)ceil_div(S->n, 256), tc);
  lz_combine_kernel<<<gr, 256, 0, st>>>(dX, ldx, S->B.as<float>(), dblk.as<const float*>(), steps - 1,
                                        dcoef.as<float>(), S->n, c0, tc);
  LAUNCH_CHECK();
  CUDA_TRY(cudaStreamSynchronize(st));   // the host coefficient vectors go out of scope on return
  return steps;
}

// Eigenvalues and squared first eigenvector components of one symmetric tridiagonal matrix
// (diagonal d[0 … nld−1], off-diagonal e[0 … nld−2], both overwritten): implicit QL with
// Wilkinson shifts in FP64, tracking only the first row z of the eigenvector matrix (all the
// Gauss quadrature needs).  Returns false if a sweep limit is hit.
//
// It runs on the Grace host: the QL is a serial chain of FP64 rotations (a square root and a
// division each), and GB300 executes FP64 at a small fraction of its FP32 rate — one thread per
// probe on the GPU took 330 ms for 64 probes of 330 steps (9 % of the window-weighted fit in the
// launch list), the host threads a few milliseconds.
// √(a² + b²) without hypot's overflow handling (a tenth of its cost), falling back to it when the
// squares leave the FP64 range.
static inline double fast_hypot(double a, double b)
{
  const double r = std::sqrt(a * a + b * b);
  return (std::isfinite(r) && (r > 0.0 || (a == 0.0 && b == 0.0))) ? r : std::hypot(a, b);
}

static bool tridiag_ql(double* d, double* e, double* z, int nld)
{
  for (int i = 0; i < nld; ++i) z[i] = (i == 0) ? 1.0 : 0.0;
  if (nld > 0) e[nld - 1] = 0.0;
  const double eps = 2.220446049250313e-16;
  for (int l = 0; l < nld; ++l) {
    for (int iter = 0;; ++iter) {
      int mm = l;
      for (; mm < nld - 1; ++mm) {
        const double dd = std::fabs(d[mm]) + std::fabs(d[mm + 1]);
        if (std::fabs(e[mm]) <= eps * dd) break;
      }
      if (mm == l) break;
      if (iter >= 64) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = fast_hypot(g, 1.0);
      g = d[mm] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      double s = 1.0, c = 1.0, pp = 0.0;
      bool deflated = false;
      for (int i = mm - 1; i >= l; --i) {
        const double f = s * e[i], b = c * e[i];
        r = fast_hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= pp;
          e[mm] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - pp;
        r = (d[i] - g) * s + 2.0 * c * b;
        pp = s * r;
        d[i + 1] = g + pp;
        g = c * r - b;
        const double zf = z[i + 1];
        z[i + 1] = s * z[i] + c * zf;
        z[i] = c * z[i] - s * zf;
      }
      if (deflated) continue;
      d[l] -= pp;
      e[l] = g;
      e[mm] = 0.0;
    }
  }
  return true;
}

// Batched tridiagonal eigensolve (host in/out, FP64).  delta is nld×t (row i = step i), beta
// (nld+1)×t; D and W2 are nld×t with eigenvalues ascending per probe.  The probes are independent
// and are spread over the host's hardware threads; each probe's result does not depend on which
// thread solves it.
void tridiag_eig_host(const double* delta, const double* beta, int t, int nld, double* D, double* W2)
{
  if (t <= 0 || nld <= 0) return;
  std::atomic<int> next{0}, failed{0};
  auto worker = [&] {
    std::vector<double> d(nld), e(nld), z(nld);
    std::vector<int> idx(nld);
    for (int p = next.fetch_add(1); p < t; p = next.fetch_add(1)) {
      for (int i = 0; i < nld; ++i) {
        d[i] = delta[(size_t)i * t + p];
        e[i] = (i + 1 < nld) ? beta[(size_t)(i + 1) * t + p] : 0.0;
      }
      if (!tridiag_ql(d.data(), e.data(), z.data(), nld)) {
        failed = 1;
        continue;
      }
      for (int i = 0; i < nld; ++i) idx[i] = i;
      std::sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
      for (int i = 0; i < nld; ++i) {
        D[(size_t)i * t + p] = d[idx[i]];
        W2[(size_t)i * t + p] = z[idx[i]] * z[idx[i]];
      }
    }
  };
  // a few hundred thousand rotations per probe at a few hundred steps: threads pay off there
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nth = (nld >= 64) ? std::min(t, hw) : 1;
  std::vector<std::thread> pool;
  for (int q = 1; q < nth; ++q) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  if (failed) SLEMM_THROW(SLEMM_ERR_NUMERIC, "tridiagonal QL did not converge in 64 sweeps");
}


}  // namespace slemm

extern "C" {

int slemm_gpu_lanczos_seed(slemm_geno* g, int op_kind, float tau0, const float* B, int64_t ldb, int t,
                           float tol, int maxit, int mem, slemm_lseed** out, int* iters)
{
  return guarded([&] {
    CHECK_ARG(g && B && out, "null argument");
    *out = nullptr;
    CHECK_ARG(ldb >= g->n, "ldb < n");
    CHECK_ARG(t >= 1 && t <= 4096, "t out of [1, 4096]");
    CHECK_ARG(mem == SLEMM_MEM_HOST || mem == SLEMM_MEM_DEVICE, "mem must be SLEMM_MEM_HOST or SLEMM_MEM_DEVICE");
    DevBuf dB;
    const float* src = B;
    if (mem == SLEMM_MEM_HOST || ldb != g->n) {
      dB.ensure((size_t)g->n * t * sizeof(float));
      CUDA_TRY(cudaMemcpy2DAsync(dB.p, g->n * sizeof(float), B, ldb * sizeof(float), g->n * sizeof(float), t,
                                 mem == SLEMM_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                 g->stream));
      src = dB.as<float>();
    }
    slemm_lseed* S = lanczos_seed_device(g, op_kind, tau0, src, t, tol, maxit, false, {}, 5, 0);
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    *out = S;
    if (iters) *iters = S->iters;
  });
}

int slemm_gpu_lseed_destroy(slemm_lseed* s)
{
  return guarded([&] {
    if (s && s->g) cudaStreamSynchronize(s->g->stream);
    delete s;
  });
}

int slemm_gpu_lseed_coeffs(const slemm_lseed* s, double* beta, double* delta)
{
  return guarded([&] {
    CHECK_ARG(s != nullptr, "null seed");
    const int t = s->t, J = s->iters;
    for (int j = 0; j <= J; ++j)
      for (int c = 0; c < t; ++c) {
        if (beta) beta[(size_t)j * t + c] = s->beta[(size_t)j * t + c];
        if (delta && j < J) delta[(size_t)j * t + c] = s->delta[(size_t)j * t + c];
      }
  });
}

int slemm_gpu_lanczos_solve(slemm_lseed* s, float sigma, float tol, float* X, int64_t ldx, int mem)
{
  return guarded([&] {
    CHECK_ARG(s && X, "null argument");
    CHECK_ARG(ldx >= s->n, "ldx < n");
    CHECK_ARG(mem == SLEMM_MEM_HOST || mem == SLEMM_MEM_DEVICE, "mem must be SLEMM_MEM_HOST or SLEMM_MEM_DEVICE");
    if (mem == SLEMM_MEM_DEVICE) {
      lanczos_solve_device(s, sigma, tol, X, ldx, 0);
      return;
    }
    DevBuf dX;
    dX.ensure((size_t)s->n * s->t * sizeof(float));
    lanczos_solve_device(s, sigma, tol, dX.as<float>(), s->n, 0);
    CUDA_TRY(cudaMemcpy2D(X, ldx * sizeof(float), dX.p, s->n * sizeof(float), s->n * sizeof(float), s->t,
                          cudaMemcpyDeviceToHost));
  });
}

int slemm_gpu_tridiag_eig(const double* delta, const double* beta, int t, int nld, double* D, double* W2)
{
  return guarded([&] {
    CHECK_ARG(delta && beta && D && W2, "null argument");
    CHECK_ARG(t >= 1 && nld >= 1, "empty problem");
    tridiag_eig_host(delta, beta, t, nld, D, W2);
  });
}

}  // extern "C"

namespace slemm {
int lseed_iters(const slemm_lseed* S, int grp) { return S->group_iters[grp]; }
const double* lseed_delta(const slemm_lseed* S) { return S->delta.data(); }
const double* lseed_beta(const slemm_lseed* S) { return S->beta.data(); }
int lseed_t(const slemm_lseed* S) { return S->t; }
void lseed_free(slemm_lseed* S) { delete S; }
}  // namespace slemm
