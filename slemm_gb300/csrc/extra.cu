// extra.cu — GEBV prediction (src/pred.cpp:4-141) and the GRAMMAR-Gamma per-variant terms of
// slemm_gamma (bin/slemm_gamma.py:302-325) as packed-genotype passes with FP64 accumulation.
//
// GEBV: tgv = Σ_j (flip_j ? 2 − x_j : x_j)·α_j = Cnt·α' + 2·Σ_{flip} α_j with α'_j = ±α_j, one
// pass over the individual-major copy (thread = individual, K = SNPs).
//
// Score terms, with x = allele-1 count = 2 − count (pgenlib's convention) and z = count − gm:
//   x − x̄ = −z, so xy = −zᵀy and xx = ‖(I − QQᵀ)(rr∘z)‖²
//        = Σ rr²z² − Σ_l (Q_lᵀ(rr∘z))²,
//   Σ rr²z² = (S1 + 2·S2) − 2·gm·S1 + gm²·Σrr²   (count² = count + 2·[count = 2])
// where S1 = Σ rr²·count, S2 = Σ rr²·[count = 2], and Q_lᵀ(rr∘z) = Σ rr·Q_l·count − gm·Σ rr·Q_l.
// One pass over the SNP-major copy (thread = SNP) accumulates Σ y·count, S1, S2 and the c
// projections in FP64.
#include "internal.h"
#include "decode.cuh"

namespace slemm {

constexpr int kXStage = 8;   // tiles per shared-memory stage

// tgv_partial[s][i] = Σ_{SNPs in split s} count[i,j]·alpha[j]
__global__ void __launch_bounds__(128)
gebv_kernel(const uint4* __restrict__ GT, int64_t K_tiles, const double* __restrict__ alpha,
            int tiles_per_split, int64_t n_pad, double* __restrict__ part)
{
  __shared__ double sa[kXStage * kTileK];
  const int t = threadIdx.x;
  const int64_t mt = blockIdx.x;
  const int s = blockIdx.y;
  const int64_t kt0 = (int64_t)s * tiles_per_split, kt1 = min64(K_tiles, kt0 + tiles_per_split);
  double acc = 0.0;
  for (int64_t ks = kt0; ks < kt1; ks += kXStage) {
    const int nt = (int)min64(kXStage, kt1 - ks);
    __syncthreads();
    for (int q = t; q < nt * kTileK; q += 128) sa[q] = alpha[ks * kTileK + q];
    __syncthreads();
    for (int u = 0; u < nt; ++u) {
      const uint4 pk = GT[(mt * K_tiles + ks + u) * 128 + t];
      const uint32_t w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float xe, xo;
          f32pair_of(w4[w], q, xe, xo);
          const int kk = u * kTileK + w * 16 + 2 * q;
          acc = fma((double)xe, sa[kk], acc);
          acc = fma((double)xo, sa[kk + 1], acc);
        }
      }
    }
  }
  part[(int64_t)s * n_pad + mt * 128 + t] = acc;
}

__global__ void gebv_finish_kernel(const double* __restrict__ part, int splits, int64_t n_pad, int64_t n,
                                   double shift, double* __restrict__ tgv)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = shift;
  for (int q = 0; q < splits; ++q) s += part[(int64_t)q * n_pad + i];
  tgv[i] = s;
}

// Per SNP row (thread): acc[0] = Σ y·x, acc[1] = S1, acc[2] = S2, acc[3+l] = Σ rr·Q_l·x.
// B rows: 0 = y, 1 = rr², 2.. = rr·Q_l (row stride K_pad); C = 2 + c rows, c ≤ 16.
template <int C>
__global__ void __launch_bounds__(128)
score_kernel(const uint4* __restrict__ G, int64_t K_tiles, const float* __restrict__ B, int64_t K_pad,
             int tiles_per_split, int64_t m_pad, double* __restrict__ part)
{
  __shared__ float sb[kXStage * kTileK][C];
  const int t = threadIdx.x;
  const int64_t mt = blockIdx.x;
  const int s = blockIdx.y;
  const int64_t kt0 = (int64_t)s * tiles_per_split, kt1 = min64(K_tiles, kt0 + tiles_per_split);
  double acc[C + 1];
#pragma unroll
  for (int q = 0; q <= C; ++q) acc[q] = 0.0;
  for (int64_t ks = kt0; ks < kt1; ks += kXStage) {
    const int nt = (int)min64(kXStage, kt1 - ks);
    __syncthreads();
    for (int q = t; q < nt * kTileK * C; q += 128) {
      const int r = q / (nt * kTileK), kk = q % (nt * kTileK);
      sb[kk][r] = B[(int64_t)r * K_pad + ks * kTileK + kk];
    }
    __syncthreads();
    for (int u = 0; u < nt; ++u) {
      const uint4 pk = G[(mt * K_tiles + ks + u) * 128 + t];
      const uint32_t w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const uint32_t cnt = count_at(w4[w], e);
          if (!cnt) continue;
          const int kk = u * kTileK + w * 16 + e;
          const double x = (double)cnt;
          acc[0] = fma(x, (double)sb[kk][0], acc[0]);
          const double r2 = (double)sb[kk][1];
          acc[1] = fma(x, r2, acc[1]);
          if (cnt == 2u) acc[2] += r2;
#pragma unroll
          for (int l = 2; l < C; ++l) acc[l + 1] = fma(x, (double)sb[kk][l], acc[l + 1]);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q <= C; ++q) part[((int64_t)s * (C + 1) + q) * m_pad + mt * 128 + t] = acc[q];
}

// xy, xx per SNP from the accumulated sums (FP64), MAC filter → NaN.
__global__ void score_finish_kernel(const double* __restrict__ part, int splits, int nacc, int64_t m_pad,
                                    int64_t m, int64_t n, const int64_t* __restrict__ pc, int c,
                                    double sum_y, double sum_r2, const double* __restrict__ sum_rq,
                                    int mac, float* __restrict__ xy, float* __restrict__ xx)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double a[3 + 64];
  for (int q = 0; q < nacc; ++q) {
    double s = 0.0;
    for (int p = 0; p < splits; ++p) s += part[((int64_t)p * nacc + q) * m_pad + j];
    a[q] = s;
  }
  const double s_a1 = 2.0 * (double)n - (double)pc[j];   // Σ x with x = 2 − count
  if (s_a1 <= mac || 2.0 * (double)n - s_a1 <= mac) {
    xy[j] = __int_as_float(0x7fc00000);
    xx[j] = __int_as_float(0x7fc00000);
    return;
  }
  const double gm = (double)pc[j] / (double)n;
  xy[j] = (float)(-(a[0] - gm * sum_y));
  double v = (a[1] + 2.0 * a[2]) - 2.0 * gm * a[1] + gm * gm * sum_r2;
  for (int l = 0; l < c; ++l) {
    const double ql = a[3 + l] - gm * sum_rq[l];
    v -= ql * ql;
  }
  xx[j] = (float)v;
}

// The same xy, xx from the tensor-core product when every rr is 1 (slemm_gamma's is_one_rr
// case): out[l·m + j] = Z_hᵀv_l for the columns v = [y | Q_0 … Q_{c−1}] with Z_h centred by the
// handle's gm_h; Σx·y and Σx·Q_l follow as out + gm_h·Σv, and Σx², the only rr-weighted sums, are
// the integer counts pc + 2·n2.  Centred by the true mean gm = pc/n in FP64, as the FP64 kernel.
__global__ void score_finish_tc_kernel(const float* __restrict__ out, int64_t m, int64_t n, int c,
                                       const float* __restrict__ gmh, const int64_t* __restrict__ pc,
                                       const int32_t* __restrict__ n2, double sum_y,
                                       const double* __restrict__ sum_q, int mac, float* __restrict__ xy,
                                       float* __restrict__ xx)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const double s_a1 = 2.0 * (double)n - (double)pc[j];
  if (s_a1 <= mac || 2.0 * (double)n - s_a1 <= mac) {
    xy[j] = __int_as_float(0x7fc00000);
    xx[j] = __int_as_float(0x7fc00000);
    return;
  }
  const double gm = (double)pc[j] / (double)n;
  const double dg = (double)gmh[j] - gm;   // Σx·v − gm·Σv = out + (gm_h − gm)·Σv
  xy[j] = (float)(-((double)out[j] + dg * sum_y));
  double v = ((double)pc[j] + 2.0 * (double)n2[j]) - 2.0 * gm * (double)pc[j] + gm * gm * (double)n;
  for (int l = 0; l < c; ++l) {
    const double ql = (double)out[(int64_t)(1 + l) * m + j] + dg * sum_q[l];
    v -= ql * ql;
  }
  xx[j] = (float)v;
}

}  // namespace slemm

using namespace slemm;

extern "C" {

int slemm_gpu_gebv(slemm_geno* g, const double* alpha, const uint8_t* flip, double* tgv)
{
  return guarded([&] {
    CHECK_ARG(g && alpha && tgv, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_gebv reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    cudaStream_t st = g->stream;
    std::vector<double> a(g->m_pad, 0.0);
    double shift = 0.0;
    for (int64_t j = 0; j < g->m; ++j) {
      CHECK_ARG(std::isfinite(alpha[j]), "non-finite SNP effect");
      const bool f = flip && flip[j];
      a[j] = f ? -alpha[j] : alpha[j];
      if (f) shift += 2.0 * alpha[j];
    }
    const int64_t M_tiles = g->n_pad / kTileM, K_tiles = g->m_pad / kTileK;
    const int splits = choose_splits(M_tiles, K_tiles, 8, num_sms());
    const int tps = (int)ceil_div(K_tiles, splits);
    DevBuf d_a(st), d_part(st), d_out(st);
    d_a.ensure(a.size() * sizeof(double));
    d_part.ensure((size_t)splits * g->n_pad * sizeof(double));
    d_out.ensure((size_t)g->n * sizeof(double));
    CUDA_TRY(cudaMemcpyAsync(d_a.p, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    gebv_kernel<<<dim3((unsigned)M_tiles, splits), 128, 0, st>>>(g->GT.as<uint4>(), K_tiles, d_a.as<double>(), tps,
                                                                 g->n_pad, d_part.as<double>());
    LAUNCH_CHECK();
    gebv_finish_kernel<<<(unsigned)ceil_div(g->n, 256), 256, 0, st>>>(d_part.as<double>(), splits, g->n_pad, g->n,
                                                                      shift, d_out.as<double>());
    LAUNCH_CHECK();
    CUDA_TRY(cudaMemcpyAsync(tgv, d_out.p, g->n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

}  // extern "C"

template <int C>
static void launch_score(slemm_geno* g, const float* B, int64_t K_pad, int splits, int tps, double* part)
{
  const int64_t M_tiles = g->m_pad / kTileM, K_tiles = g->n_pad / kTileK;
  score_kernel<C><<<dim3((unsigned)M_tiles, splits), 128, 0, g->stream>>>(g->G.as<uint4>(), K_tiles, B, K_pad, tps,
                                                                          g->m_pad, part);
  LAUNCH_CHECK();
}

extern "C" {

int slemm_gpu_score_terms(slemm_geno* g, const float* y, int mac, float* xy, float* xx)
{
  return guarded([&] {
    CHECK_ARG(g && y && xy && xx, "null argument");
    if (g->is_view)
      SLEMM_THROW(SLEMM_ERR_UNSUPPORTED, "slemm_gpu_score_terms reads the packed copies directly and is not available on a "
                                         "trait view; create a handle with the keep list instead");
    CHECK_ARG(g->weights_set, "set_weights (rr) must be called first");
    const int c = g->c;
    CHECK_ARG(c <= 14, "score terms support up to 14 projection columns");
    cudaStream_t st = g->stream;
    const int64_t n = g->n, n_pad = g->n_pad;
    // host-side B rows: y, rr², rr·Q_l (FP32), and the FP64 column sums
    std::vector<float> rr(n_pad, 0.f), Q((size_t)n_pad * std::max(c, 1), 0.f);
    CUDA_TRY(cudaMemcpyAsync(rr.data(), g->rr.p, n_pad * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (c) CUDA_TRY(cudaMemcpyAsync(Q.data(), g->Q.p, (size_t)n_pad * c * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    bool one_rr = true;
    for (int64_t i = 0; i < n && one_rr; ++i) one_rr = rr[i] == 1.0f;
    if (one_rr) {
      // the packed tensor-core product of [y | Q] (column-scaled FP16 hi+lo pieces, FP32 accumulation);
      // the FP64 per-genotype kernel below serves general rr
      const int k = 1 + c;
      std::vector<float> V((size_t)k * n);
      double sum_y = 0.0;
      std::vector<double> sum_q(std::max(c, 1), 0.0);
      for (int64_t i = 0; i < n; ++i) {
        V[i] = y[i];
        sum_y += (double)y[i];
      }
      for (int l = 0; l < c; ++l)
        for (int64_t i = 0; i < n; ++i) {
          const float q = Q[(size_t)l * n_pad + i];
          V[(size_t)(1 + l) * n + i] = q;
          sum_q[l] += (double)q;
        }
      std::vector<int64_t> pc(g->m);
      std::vector<int32_t> n2(g->m);
      {
        const int s2 = slemm_gpu_genotype_counts(g, pc.data(), nullptr, nullptr, n2.data());
        if (s2 != SLEMM_OK) SLEMM_THROW(s2, "genotype counts failed");
      }
      DevBuf dV(st), dO(st), dpc(st), dn2(st), dsq(st), dxy(st), dxx(st);
      dV.ensure(V.size() * sizeof(float));
      dO.ensure((size_t)k * g->m * sizeof(float));
      dpc.ensure(g->m * sizeof(int64_t));
      dn2.ensure(g->m * sizeof(int32_t));
      dsq.ensure(sum_q.size() * sizeof(double));
      dxy.ensure(g->m * sizeof(float));
      dxx.ensure(g->m * sizeof(float));
      CUDA_TRY(cudaMemcpyAsync(dV.p, V.data(), V.size() * sizeof(float), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(dpc.p, pc.data(), g->m * sizeof(int64_t), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(dn2.p, n2.data(), g->m * sizeof(int32_t), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(dsq.p, sum_q.data(), sum_q.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      const int prec = g->prec;
      g->prec = SLEMM_PREC_FP16X2;
      try {
        op_device(g, SLEMM_OP_RMATVEC, 0.f, dV.as<float>(), n, k, dO.as<float>(), g->m);
      } catch (...) {
        g->prec = prec;
        throw;
      }
      g->prec = prec;
      score_finish_tc_kernel<<<(unsigned)ceil_div(g->m, 256), 256, 0, st>>>(
          dO.as<float>(), g->m, n, c, g->gm.as<float>(), dpc.as<int64_t>(), dn2.as<int32_t>(), sum_y,
          dsq.as<double>(), mac, dxy.as<float>(), dxx.as<float>());
      LAUNCH_CHECK();
      CUDA_TRY(cudaMemcpyAsync(xy, dxy.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(xx, dxx.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      return;
    }
    const int C = 2 + c;
    std::vector<float> B((size_t)C * n_pad, 0.f);
    double sum_y = 0.0, sum_r2 = 0.0;
    std::vector<double> sum_rq(std::max(c, 1), 0.0);
    for (int64_t i = 0; i < n; ++i) {
      B[i] = y[i];
      B[n_pad + i] = rr[i] * rr[i];
      sum_y += (double)y[i];
      sum_r2 += (double)rr[i] * rr[i];
      for (int l = 0; l < c; ++l) {
        const float v = rr[i] * Q[(size_t)l * n_pad + i];
        B[(size_t)(2 + l) * n_pad + i] = v;
        sum_rq[l] += (double)v;
      }
    }
    const int64_t M_tiles = g->m_pad / kTileM, K_tiles = n_pad / kTileK;
    const int splits = choose_splits(M_tiles, K_tiles, 8, num_sms());
    const int tps = (int)ceil_div(K_tiles, splits);
    DevBuf dB(st), dpart(st), dsrq(st), dxy(st), dxx(st), dpc(st);
    dB.ensure(B.size() * sizeof(float));
    dpart.ensure((size_t)splits * (C + 1) * g->m_pad * sizeof(double));
    dsrq.ensure(sum_rq.size() * sizeof(double));
    dxy.ensure(g->m * sizeof(float));
    dxx.ensure(g->m * sizeof(float));
    dpc.ensure(g->m * sizeof(int64_t));
    std::vector<int64_t> pc(g->m);
    {
      int s2 = slemm_gpu_genotype_counts(g, pc.data(), nullptr, nullptr, nullptr);
      if (s2 != SLEMM_OK) SLEMM_THROW(s2, "genotype counts failed");
    }
    CUDA_TRY(cudaMemcpyAsync(dpc.p, pc.data(), g->m * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(dB.p, B.data(), B.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(dsrq.p, sum_rq.data(), sum_rq.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    double* part = dpart.as<double>();
    switch (C) {
      case 2: launch_score<2>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      case 3: launch_score<3>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      case 4: launch_score<4>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      case 5: launch_score<5>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      case 6: launch_score<6>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      case 8: launch_score<8>(g, dB.as<float>(), n_pad, splits, tps, part); break;
      default: {
        // widths 7 and 9..16: pad the B rows up to the next supported width with zero rows
        const int Cp = C <= 8 ? 8 : 16;
        std::vector<float> Bp((size_t)Cp * n_pad, 0.f);
        std::copy(B.begin(), B.end(), Bp.begin());
        DevBuf dBp(st), dpp(st);
        dBp.ensure(Bp.size() * sizeof(float));
        dpp.ensure((size_t)splits * (Cp + 1) * g->m_pad * sizeof(double));
        CUDA_TRY(cudaMemcpyAsync(dBp.p, Bp.data(), Bp.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        if (Cp == 8) launch_score<8>(g, dBp.as<float>(), n_pad, splits, tps, dpp.as<double>());
        else launch_score<16>(g, dBp.as<float>(), n_pad, splits, tps, dpp.as<double>());
        score_finish_kernel<<<(unsigned)ceil_div(g->m, 256), 256, 0, st>>>(
            dpp.as<double>(), splits, Cp + 1, g->m_pad, g->m, n, dpc.as<int64_t>(), c, sum_y, sum_r2,
            dsrq.as<double>(), mac, dxy.as<float>(), dxx.as<float>());
        LAUNCH_CHECK();
        CUDA_TRY(cudaMemcpyAsync(xy, dxy.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(xx, dxx.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return;
      }
    }
    score_finish_kernel<<<(unsigned)ceil_div(g->m, 256), 256, 0, st>>>(
        part, splits, C + 1, g->m_pad, g->m, n, dpc.as<int64_t>(), c, sum_y, sum_r2, dsrq.as<double>(), mac,
        dxy.as<float>(), dxx.as<float>());
    LAUNCH_CHECK();
    CUDA_TRY(cudaMemcpyAsync(xy, dxy.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(xx, dxx.p, g->m * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
