// gwa.cu — windowed MLMA of slemm_gwa.py (bin/slemm_gwa.py:259-431) on the packed genotypes.
//
// The model SNPs of a chromosome are cut into overlapping blocks of block_size (step
// block_size/2, the last block flush with the end; :322-335); block i serves the tested variants
// from the previous block's bound to model SNP [block_size − block_size/4] of its own (:337-344).
// Per block, with B the block's centred (per-SNP mean), rr-scaled, projected genotypes:
//   H = BBᵀ + model_snp_ct·τ·diag(rvar),  rvar = (2 − mean)·mean/2            (:376-408)
// and per tested variant x (centred, MAC filter on allele-1 counts):
//   xy = xᵀy (before scaling; y is the Py column of .reml.py.txt),
//   xx = ‖x̃‖² − (Bx̃)ᵀH⁻¹(Bx̃) with x̃ = (I − QQᵀ)(rr∘x)                          (:409-428)
// then xx /= τ, β = xy/xx·cf, se = √(snp_var·cf/xx), χ² = (β/se)², p = P(χ²₁ > χ²)  (:430-434).
// Allele-1 counts are 2 − the .bed's allele-2 counts: centring flips the sign of x, which leaves
// xx unchanged and flips xy — computed here with allele-2 counts and xy negated at the end.
//
// GB300 mapping: the model SNPs are gathered into their own packed copy (16-byte rows of the
// tiles), so every block is a contiguous row range; BBᵀ and Bx̃ for all the block's tested
// variants are packed tensor-core products Cc_blockᵀ·U (column-scaled FP16 hi+lo, ≈ FP32 like the
// script's float32 BLAS) with U = rr∘(I − QQᵀ)(rr∘Cc) or rr∘X̃ — no dense B is ever formed.  The
// blocks' systems are factored together (blocked FP32 Cholesky, one CTA per block), and the
// quadratic forms come from one batched multi-right-hand-side triangular solve in shared memory.
#include "internal.h"
#include "reduce.cuh"
#include "dense.cuh"

#include <algorithm>
#include <cmath>

namespace slemm {

// Gs (rows = rows[0 … cnt), tiled like G, rows ≥ cnt zero) from G: one 16-byte tile row each.
__global__ void gather_rows_kernel(const uint4* __restrict__ G, int64_t K_tiles, const int64_t* __restrict__ rows,
                                   int64_t cnt, int64_t total, uint4* __restrict__ Gs)
{
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // destination order
  if (q >= total) return;
  const int64_t r = q % 128, t = q / 128, kt = t % K_tiles, mt = t / K_tiles;
  const int64_t jd = mt * 128 + r;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (jd < cnt) {
    const int64_t js = rows[jd];
    v = G[((js / 128) * K_tiles + kt) * 128 + (js % 128)];
  }
  Gs[q] = v;
}

// F_b = lower triangle of (A_b + diag(ridge_b)), A_b = A + b·stride + off[b] (ld lda), factored.
__global__ void __launch_bounds__(kCholThreads)
chol_batch_kernel(const float* __restrict__ A, int64_t lda, int64_t stride, const int64_t* __restrict__ off,
                  const float* __restrict__ ridge, int s, float* __restrict__ F, int* __restrict__ status)
{
  __shared__ float S[kCholB][kCholB + 1];
  __shared__ int bad;
  const int b = blockIdx.x;
  const float* Ab = A + (int64_t)b * stride + off[b];
  const float* rb = ridge + (int64_t)b * s;
  float* Fb = F + (int64_t)b * s * s;
  if (threadIdx.x == 0) bad = 0;
  for (int64_t q = threadIdx.x; q < (int64_t)s * s; q += blockDim.x) {
    const int i = (int)(q % s), j = (int)(q / s);
    if (i >= j) Fb[(int64_t)j * s + i] = Ab[(int64_t)j * lda + i] + (i == j ? rb[i] : 0.f);
  }
  __syncthreads();
  if (!chol_blocked(Fb, s, s, S, &bad) && threadIdx.x == 0) atomicOr(status, 1);
}

// One task = up to R right-hand sides of one block: Y = L⁻¹Z in shared memory (s×R, row-major),
// q_c = ‖Y_c‖² (FP64).  task[4·t …] = factor offset, Z offset, ld of Z, q offset; ncols[t].
__global__ void __launch_bounds__(256)
trsm_quad_kernel(const float* __restrict__ F, int s, const float* __restrict__ Z, const int64_t* __restrict__ task,
                 const int* __restrict__ ncols, int R, double* __restrict__ q)
{
  extern __shared__ float Y[];
  const int64_t* t = task + 4 * (int64_t)blockIdx.x;
  const float* L = F + t[0];
  const float* Zb = Z + t[1];
  const int64_t ldz = t[2];
  double* qb = q + t[3];
  const int nc = ncols[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  for (int64_t idx = tid; idx < (int64_t)s * R; idx += blockDim.x) {
    const int i = (int)(idx % s), c = (int)(idx / s);
    Y[(int64_t)i * R + c] = (c < nc) ? Zb[(int64_t)c * ldz + i] : 0.f;
  }
  __syncthreads();
  for (int p0 = 0; p0 < s; p0 += 32) {
    const int pb = min(32, s - p0);
    // rows p0 … p0+pb−1 minus the solved rows above: lanes are rows, warps stride the columns
    for (int c = warp; c < R; c += nwarps) {
      if (lane < pb) {
        float acc = 0.f;
#pragma unroll 8
        for (int k = 0; k < p0; ++k) acc = fmaf(L[(int64_t)k * s + p0 + lane], Y[(int64_t)k * R + c], acc);
        Y[(int64_t)(p0 + lane) * R + c] -= acc;
      }
    }
    __syncthreads();
    // the 32×32 diagonal block, one thread per column
    if (tid < R) {
      for (int i = 0; i < pb; ++i) {
        float v = Y[(int64_t)(p0 + i) * R + tid];
        for (int k = 0; k < i; ++k) v -= L[(int64_t)(p0 + k) * s + p0 + i] * Y[(int64_t)(p0 + k) * R + tid];
        Y[(int64_t)(p0 + i) * R + tid] = v / L[(int64_t)(p0 + i) * s + p0 + i];
      }
    }
    __syncthreads();
  }
  for (int c = warp; c < nc; c += nwarps) {
    double a = 0.0;
    for (int i = lane; i < s; i += 32) {
      const double y = (double)Y[(int64_t)i * R + c];
      a += y * y;
    }
    for (int o = 16; o; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) qb[c] = a;
  }
}

// Model-SNP copy of a handle: only what rows_product and the projections read.
struct ModelCopy {
  slemm_geno h;
  ModelCopy(slemm_geno* g, const std::vector<int64_t>& model)
  {
    h.device = g->device;
    h.stream = g->stream;
    h.own_stream = false;
    h.bind_stream();
    h.n = g->n;
    h.n_pad = g->n_pad;
    h.m = (int64_t)model.size();
    h.m_pad = round_up(h.m, kPadRows);
    h.prec = SLEMM_PREC_FP16X2;
    h.weights_set = true;
    const int64_t K_tiles = g->n_pad / kTileK;
    const int64_t total = h.m_pad * K_tiles;   // 16-byte tile rows
    h.G.ensure((size_t)total * 16);
    DevBuf d_rows(g->stream);
    d_rows.ensure(model.size() * sizeof(int64_t));
    CUDA_TRY(cudaMemcpyAsync(d_rows.p, model.data(), model.size() * sizeof(int64_t), cudaMemcpyHostToDevice, g->stream));
    gather_rows_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, g->stream>>>(g->G.as<uint4>(), K_tiles,
                                                                                d_rows.as<int64_t>(), h.m, total,
                                                                                h.G.as<uint4>());
    LAUNCH_CHECK();
    h.err.ensure(sizeof(int));
    CUDA_TRY(cudaMemsetAsync(h.err.p, 0, sizeof(int), g->stream));
  }
  ~ModelCopy()
  {
    h.for_each_buf([](DevBuf& b) { b.release(); });
  }
};

}  // namespace slemm

using namespace slemm;

extern "C" int slemm_gpu_gwa_windows(slemm_geno* g, const float* y, const float* R, const float* covar, int64_t ldc,
                                     int c, const int64_t* model_idx, int64_t n_model, int64_t test_begin,
                                     int64_t test_end, int block_size, float tau, int64_t model_snp_ct, float cfactor,
                                     float snp_var, int mac, float* beta, float* se, float* chisq, double* pval)
{
  return guarded([&] {
    CHECK_ARG(g && y && covar && model_idx && beta && se && chisq && pval, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_gwa_windows reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    const int64_t n = g->n, m = g->m;
    CHECK_ARG(c >= 1 && c <= SLEMM_MAX_COVARIATES && ldc >= n, "bad covariate matrix");
    CHECK_ARG(n_model >= 2 && test_begin >= 0 && test_end < m && test_begin <= test_end, "bad SNP ranges");
    for (int64_t k = 0; k < n_model; ++k)
      CHECK_ARG(model_idx[k] >= 0 && model_idx[k] < m && (k == 0 || model_idx[k] > model_idx[k - 1]),
                "model SNP indices must be increasing handle indices");
    // as in the script, the model SNPs and the tested variants are those of one chromosome, so
    // every block's share of the tested range (below) is a non-empty or empty interval
    CHECK_ARG(model_idx[0] >= test_begin && model_idx[n_model - 1] <= test_end,
              "model SNPs must lie inside the tested range (one chromosome)");
    CHECK_ARG(tau > 0.f && std::isfinite(tau), "tau must be positive");
    cudaStream_t st = g->stream;
    // blocks and the tested range each serves (bin/slemm_gwa.py:319-344)
    int bs = block_size;
    if (bs > n_model) bs = (int)(n_model / 2) * 2;
    CHECK_ARG(bs >= 4 && bs <= 5000, "block size out of [4, 5000]");
    const int step = bs / 2, ext = step / 2;
    std::vector<int64_t> start;
    for (int64_t i = 0; i < (n_model - step) / step; ++i) start.push_back(i * step);
    if ((n_model - step) % step != 0) start.push_back(n_model - bs);
    const int nb = (int)start.size();
    std::vector<int64_t> lo(nb), hi(nb);
    lo[0] = test_begin;
    hi[0] = model_idx[start[0] + bs - ext];
    for (int i = 1; i < nb; ++i) {
      lo[i] = hi[i - 1];
      hi[i] = model_idx[start[i] + bs - ext];
    }
    hi[nb - 1] = test_end + 1;
    for (int i = 0; i < nb; ++i)
      CHECK_ARG(test_begin <= lo[i] && lo[i] <= hi[i] && hi[i] <= test_end + 1, "inconsistent block ranges");
    // rr, Q of the covariates (scipy's economic QR in the script; any orthonormal basis gives the
    // same projection)
    std::vector<float> rr(g->n_pad, 0.f);
    for (int64_t i = 0; i < n; ++i) {
      const float r = R ? R[i] : 1.0f;
      CHECK_ARG(r > 0.f && std::isfinite(r), "R must be positive");
      rr[i] = 1.0f / std::sqrt(r);
    }
    std::vector<double> A((size_t)n * c), Qd;
    for (int j = 0; j < c; ++j)
      for (int64_t i = 0; i < n; ++i) A[(size_t)j * n + i] = (double)(covar[(size_t)j * ldc + i] * rr[i]);
    const int rank = orthonormal_columns(A, n, c, Qd);
    CHECK_ARG(rank == c, "covariate matrix is not of full rank");
    // per-SNP means (allele-2) of the whole handle; the model copy with its own means
    std::vector<float> mean(g->m_pad, 0.f);
    std::vector<int64_t> pc(m);
    {
      DevBuf b(st);
      int64_t* d_pc = (int64_t*)b.ensure((size_t)m * 16);
      row_counts_device(g, d_pc, (int32_t*)(d_pc + m), (int32_t*)(d_pc + m) + m);
      CUDA_TRY(cudaMemcpyAsync(pc.data(), d_pc, m * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      for (int64_t j = 0; j < m; ++j) mean[j] = (float)pc[j] / (float)n;
    }
    std::vector<int64_t> model(model_idx, model_idx + n_model);
    ModelCopy mc(g, model);
    slemm_geno* M = &mc.h;
    {
      std::vector<float> gmm(M->m_pad, 0.f), corr(M->m_pad, 0.f), Qf((size_t)g->n_pad * c, 0.f);
      for (int64_t k = 0; k < n_model; ++k) {
        gmm[k] = mean[model[k]];
        corr[k] = (float)((double)pc[model[k]] - (double)n * (double)gmm[k]);   // Z_cᵀ1 of the copy's rows
      }
      for (int j = 0; j < c; ++j)
        for (int64_t i = 0; i < n; ++i) Qf[(size_t)j * g->n_pad + i] = (float)Qd[(size_t)j * n + i];
      M->gm.ensure(gmm.size() * sizeof(float));
      M->rr.ensure(rr.size() * sizeof(float));
      M->Q.ensure(Qf.size() * sizeof(float));
      M->gcorr.ensure(corr.size() * sizeof(float));
      CUDA_TRY(cudaMemcpyAsync(M->gcorr.p, corr.data(), corr.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(M->gm.p, gmm.data(), gmm.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(M->rr.p, rr.data(), rr.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(M->Q.p, Qf.data(), Qf.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      M->c = c;
      CUDA_TRY(cudaStreamSynchronize(st));
    }
    DevBuf d_mean(st), d_y(st);
    float* dmean = (float*)d_mean.ensure(mean.size() * sizeof(float));
    float* dy = (float*)d_y.ensure(n * sizeof(float));
    CUDA_TRY(cudaMemcpyAsync(dmean, mean.data(), mean.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(dy, y, n * sizeof(float), cudaMemcpyHostToDevice, st));
    const float* drr = M->rr.as<float>();
    const int64_t K_tiles = g->n_pad / kTileK;
    const int64_t rows_max = round_up(bs, kPadRows) + kPadRows;
    const int64_t ntest = test_end - test_begin + 1;
    std::vector<float> xx2(ntest, 0.f), xy2(ntest, 0.f);
    std::vector<double> qv(ntest, 0.0);
    // blocks in batches (bounded memory)
    const int batch = 32;
    DevBuf d_U(st), d_gram(st), d_F(st), d_ridge(st), d_off(st), d_status(st), d_X(st), d_Z(st), d_sc(st),
        d_qt(st), d_task(st), d_nc(st), d_q(st);
    int* status = (int*)d_status.ensure(sizeof(int));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    for (int b0 = 0; b0 < nb; b0 += batch) {
      const int bn = std::min(batch, nb - b0);
      float* gram = (float*)d_gram.ensure((size_t)bn * rows_max * bs * sizeof(float));
      float* U = (float*)d_U.ensure((size_t)n * bs * sizeof(float));
      double* qtv = (double*)d_qt.ensure((size_t)c * bs * sizeof(double));
      std::vector<int64_t> off(bn);
      std::vector<float> ridge((size_t)bn * bs);
      // 1. block Grams: Cc_blockᵀ·rr∘P(rr∘Cc_block)
      for (int bi = 0; bi < bn; ++bi) {
        const int64_t s0 = start[b0 + bi];
        const int64_t r0 = s0 / kPadRows * kPadRows;
        const int64_t r1 = std::min<int64_t>(round_up(s0 + bs, kPadRows), M->m_pad);
        off[bi] = s0 - r0;
        for (int t = 0; t < bs; ++t) {
          const float mu = mean[model[s0 + t]];
          ridge[(size_t)bi * bs + t] = (float)model_snp_ct * tau * ((2.0f - mu) * mu / 2.0f);
        }
        centred_rows_kernel<<<dim3((unsigned)ceil_div(n, 256), bs), 256, 0, st>>>(
            M->G.as<uint32_t>(), K_tiles, nullptr, s0, M->gm.as<float>(), drr, n, U, n);
        LAUNCH_CHECK();
        proj_coeffs(M, U, n, bs, qtv);
        proj_apply(M, U, n, bs, qtv);
        scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), bs), 256, 0, st>>>(U, n, drr, n);
        LAUNCH_CHECK();
        rows_product(M, r0, r1 - r0, U, n, bs, gram + (size_t)bi * rows_max * bs, rows_max, SLEMM_PREC_FP16X2);
      }
      // 2. factor every block of the batch (one CTA each)
      float* F = (float*)d_F.ensure((size_t)bn * bs * bs * sizeof(float));
      float* dr = (float*)d_ridge.ensure(ridge.size() * sizeof(float));
      int64_t* doff = (int64_t*)d_off.ensure(bn * sizeof(int64_t));
      CUDA_TRY(cudaMemcpyAsync(dr, ridge.data(), ridge.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(doff, off.data(), bn * sizeof(int64_t), cudaMemcpyHostToDevice, st));
      chol_batch_kernel<<<bn, kCholThreads, 0, st>>>(gram, rows_max, rows_max * bs, doff, dr, bs, F, status);
      LAUNCH_CHECK();
      // 3. tested variants of each block: x'y, ‖x̃‖², and Z = Cc_blockᵀ(rr∘x̃)
      int64_t tb_tot = 0;
      for (int bi = 0; bi < bn; ++bi) tb_tot += hi[b0 + bi] - lo[b0 + bi];
      float* Zall = (float*)d_Z.ensure((size_t)std::max<int64_t>(tb_tot, 1) * rows_max * sizeof(float));
      double* sc = (double*)d_sc.ensure((size_t)std::max<int64_t>(tb_tot, 1) * 2 * sizeof(double));
      std::vector<int64_t> zoff(bn);
      int64_t acc = 0;
      for (int bi = 0; bi < bn; ++bi) {
        const int64_t tb = hi[b0 + bi] - lo[b0 + bi];
        zoff[bi] = acc;
        if (tb <= 0) continue;
        float* X = (float*)d_X.ensure((size_t)n * tb * sizeof(float));
        centred_rows_kernel<<<dim3((unsigned)ceil_div(n, 256), (unsigned)tb), 256, 0, st>>>(
            g->G.as<uint32_t>(), K_tiles, nullptr, lo[b0 + bi], dmean, nullptr, n, X, n);
        LAUNCH_CHECK();
        col_dots(M, X, n, dy, 0, n, (int)tb, sc + 2 * acc);   // x'y
        scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), (unsigned)tb), 256, 0, st>>>(X, n, drr, n);
        LAUNCH_CHECK();
        double* qt2 = (double*)d_qt.ensure((size_t)c * std::max<int64_t>(bs, tb) * sizeof(double));
        proj_coeffs(M, X, n, (int)tb, qt2);
        proj_apply(M, X, n, (int)tb, qt2);
        col_dots(M, X, n, nullptr, 0, n, (int)tb, sc + 2 * acc + tb);   // ‖x̃‖²
        scale_rows_rr_kernel<<<dim3((unsigned)ceil_div(n, 256), (unsigned)tb), 256, 0, st>>>(X, n, drr, n);
        LAUNCH_CHECK();
        const int64_t s0 = start[b0 + bi];
        const int64_t r0 = s0 / kPadRows * kPadRows;
        const int64_t r1 = std::min<int64_t>(round_up(s0 + bs, kPadRows), M->m_pad);
        rows_product(M, r0, r1 - r0, X, n, (int)tb, Zall + (size_t)acc * rows_max, rows_max, SLEMM_PREC_FP16X2);
        acc += tb;
      }
      // 4. q = ‖L⁻¹z‖² for every tested variant of the batch
      const int Rc = std::max(1, std::min(32, (int)((160 * 1024) / (4 * (int64_t)bs))));
      std::vector<int64_t> task;
      std::vector<int> ncol;
      for (int bi = 0; bi < bn; ++bi) {
        const int64_t tb = hi[b0 + bi] - lo[b0 + bi];
        for (int64_t c0 = 0; c0 < tb; c0 += Rc) {
          task.push_back((int64_t)bi * bs * bs);
          task.push_back((zoff[bi] + c0) * rows_max + off[bi]);
          task.push_back(rows_max);
          task.push_back(zoff[bi] + c0);
          ncol.push_back((int)std::min<int64_t>(Rc, tb - c0));
        }
      }
      if (!ncol.empty()) {
        int64_t* dt = (int64_t*)d_task.ensure(task.size() * sizeof(int64_t));
        int* dn = (int*)d_nc.ensure(ncol.size() * sizeof(int));
        double* dq = (double*)d_q.ensure((size_t)acc * sizeof(double));
        CUDA_TRY(cudaMemcpyAsync(dt, task.data(), task.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(dn, ncol.data(), ncol.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        const size_t smem = (size_t)bs * Rc * sizeof(float);
        CUDA_TRY(cudaFuncSetAttribute(trsm_quad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        trsm_quad_kernel<<<(unsigned)ncol.size(), 256, smem, st>>>(F, bs, Zall, dt, dn, Rc, dq);
        LAUNCH_CHECK();
        std::vector<double> hsc((size_t)2 * acc), hq(acc);
        CUDA_TRY(cudaMemcpyAsync(hsc.data(), sc, hsc.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(hq.data(), dq, hq.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (int bi = 0; bi < bn; ++bi) {
          const int64_t tb = hi[b0 + bi] - lo[b0 + bi];
          for (int64_t t = 0; t < tb; ++t) {
            const int64_t j = lo[b0 + bi] + t - test_begin;
            xy2[j] = (float)hsc[2 * zoff[bi] + t];
            xx2[j] = (float)hsc[2 * zoff[bi] + tb + t];
            qv[j] = hq[zoff[bi] + t];
          }
        }
      }
    }
    check_device_error(M);
    int hs = 0;
    CUDA_TRY(cudaMemcpy(&hs, status, sizeof(int), cudaMemcpyDeviceToHost));
    if (hs) SLEMM_THROW(SLEMM_ERR_NUMERIC, "a block's BBᵀ + ridge is not positive definite in FP32");
    // statistics (bin/slemm_gwa.py:413-434), allele-1 orientation
    for (int64_t t = 0; t < ntest; ++t) {
      const int64_t j = test_begin + t;
      const int64_t s_a1 = 2 * n - pc[j];   // allele-1 count sum
      const bool drop = s_a1 <= mac || 2 * n - s_a1 <= mac;
      if (drop) {
        beta[t] = se[t] = chisq[t] = NAN;
        pval[t] = NAN;
        continue;
      }
      const float xx = (float)((double)xx2[t] - qv[t]) / tau;
      const float xy = -xy2[t];
      beta[t] = xy / xx * cfactor;
      se[t] = std::sqrt((snp_var * cfactor) / xx);
      const float z = beta[t] / se[t];
      chisq[t] = z * z;
      pval[t] = std::erfc(std::sqrt((double)chisq[t] / 2.0));
    }
  });
}
