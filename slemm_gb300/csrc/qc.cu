// qc.cu — marker quality control on the packed genotypes: minor-allele frequency and the exact
// Hardy–Weinberg test per SNP (src/input.cpp:388-394), and decoded count rows.
//
// MAF (src/weight.cpp:3-15): f = popcount/float(2n) over the kept individuals' 2n bits (a missing
// call counts as one set bit), maf = |[f > 0.5] − f| in FP32.
//
// HWE (src/snphwe.cpp:18 SNPHWE2, called as SNPHWE2(n1, n0, n2, midp) at src/input.cpp:20 with
// n2 = calls with both bits set, n1 = one bit set — hets and missing calls — and n0 = neither):
// the exact test of Wigginton, Cutler & Abecasis (2005).  With N calls and r rare alleles the het
// count h (parity of r) has, under HWE, P(h+2)/P(h) = 4·hom_r·hom_c / ((h+2)(h+1)), hom_r = (r−h)/2,
// hom_c = N − h − hom_r.  p = Σ_{P(h) ≤ P(obs)} P(h) / Σ_h P(h), with a relative tie tolerance of
// 1e-7; the mid-p variant subtracts P(obs)/2.  One thread per SNP works in FP64 relative to the
// mode of the distribution (unimodal, so the terms fall monotonically on both sides), walks each
// side outward and stops where a term is below 1e-18 of min(P(obs), P(mode)) — smaller terms
// cannot move the sums in FP64.  The reference stores the result as FP32 (VectorXf hwep).
#include "internal.h"

namespace slemm {

__device__ __forceinline__ double hwe_up(int64_t h, int64_t rare, int64_t n)   // P(h+2)/P(h)
{
  const int64_t hr = (rare - h) / 2, hc = n - h - hr;
  return 4.0 * (double)hr * (double)hc / ((double)(h + 2) * (double)(h + 1));
}

__device__ double hwe_exact_p(int64_t het, int64_t hom1, int64_t hom2, int midp)
{
  const int64_t n = het + hom1 + hom2;
  if (n == 0) return midp ? 0.5 : 1.0;
  const int64_t rare = 2 * min64(hom1, hom2) + het;
  const int64_t hmax = min64(rare, 2 * n - rare);
  const int64_t par = rare & 1;
  int64_t h = (int64_t)((double)rare * (double)(2 * n - rare) / (double)(2 * n - 1));
  if ((h & 1) != par) h += (h + 1 <= hmax) ? 1 : -1;
  h = max64(par, min64(h, hmax));
  while (h + 2 <= hmax && hwe_up(h, rare, n) > 1.0) h += 2;
  while (h >= 2 && hwe_up(h - 2, rare, n) < 1.0) h -= 2;
  const int64_t mode = h;
  double pobs = 1.0;
  if (het > mode)
    for (int64_t k = mode; k < het && pobs > 0.0; k += 2) pobs *= hwe_up(k, rare, n);
  else
    for (int64_t k = mode; k > het && pobs > 0.0; k -= 2) pobs /= hwe_up(k - 2, rare, n);
  const double cut = pobs * (1.0 + 1e-7);
  const double stop = fmin(pobs, 1.0) * 1e-18;
  double tot = 1.0, tail = (1.0 <= cut) ? 1.0 : 0.0;
  double p = 1.0;
  for (int64_t k = mode; k + 2 <= hmax;) {
    p *= hwe_up(k, rare, n);
    k += 2;
    tot += p;
    if (p <= cut) tail += p;
    if (p < stop || p == 0.0) break;
  }
  p = 1.0;
  for (int64_t k = mode; k >= 2;) {
    p /= hwe_up(k - 2, rare, n);
    k -= 2;
    tot += p;
    if (p <= cut) tail += p;
    if (p < stop || p == 0.0) break;
  }
  if (midp) tail -= 0.5 * pobs;
  return fmin(1.0, tail / tot);
}

__global__ void hwe_kernel(const int32_t* __restrict__ het, const int32_t* __restrict__ hom1,
                           const int32_t* __restrict__ hom2, int64_t m, int midp, double* __restrict__ p)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) p[j] = hwe_exact_p(het[j], hom1[j], hom2[j], midp);
}

// From the per-row counts of the G copy: maf (FP32, reference formula) and the HWE p-value.
__global__ void marker_qc_kernel(const int64_t* __restrict__ pc, const int32_t* __restrict__ c1,
                                 const int32_t* __restrict__ c2, int64_t m, int64_t n, int midp,
                                 float* __restrict__ maf, float* __restrict__ hwep)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const float f = (float)(int)pc[j] / (float)(2 * n);
  maf[j] = fabsf((f > 0.5f ? 1.0f : 0.0f) - f);
  const int64_t n1 = c1[j], n2 = c2[j], n0 = n - n1 - n2;
  hwep[j] = (float)hwe_exact_p(n1, n0, n2, midp);
}

// out[c·ld + i] = count of SNP rows[c] for kept individual i (i < n), from the G copy (at packed
// position map[i] for a trait view, else i).
__global__ void genotype_rows_kernel(const uint32_t* __restrict__ G, int64_t K_tiles, const int64_t* __restrict__ rows,
                                     int64_t n, const int32_t* __restrict__ map, float* __restrict__ out, int64_t ld)
{
  const int c = blockIdx.y;
  const int64_t iv = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (iv >= n) return;
  const int64_t i = map ? (int64_t)map[iv] : iv;
  const int64_t j = rows[c];
  const int64_t mt = j / 128, r = j % 128, kt = i / 64, e = i % 64;
  const uint32_t w = G[((mt * K_tiles + kt) * 128 + r) * 4 + e / 16];
  const int q = (int)(e % 16);
  const int sh = (q & 1) ? 16 + (q & ~1) : q;   // even element 2p at bits 2p, odd 2p+1 at 16+2p
  out[(int64_t)c * ld + iv] = (float)((w >> sh) & 3u);
}

}  // namespace slemm

using namespace slemm;

extern "C" {

int slemm_gpu_hwe_exact(const int32_t* het, const int32_t* hom1, const int32_t* hom2, int64_t m, int midp,
                        double* p)
{
  return guarded([&] {
    CHECK_ARG(m >= 0, "m < 0");
    if (m == 0) return;
    CHECK_ARG(het && hom1 && hom2 && p, "null argument");
    for (int64_t j = 0; j < m; ++j)
      CHECK_ARG(het[j] >= 0 && hom1[j] >= 0 && hom2[j] >= 0, "negative genotype count");
    DevBuf d;
    int32_t* dc = (int32_t*)d.ensure((size_t)m * (3 * sizeof(int32_t) + sizeof(double)) + sizeof(double));
    double* dp = reinterpret_cast<double*>(dc + 3 * m + (m & 1));   // 8-byte aligned
    CUDA_TRY(cudaMemcpy(dc, het, m * sizeof(int32_t), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dc + m, hom1, m * sizeof(int32_t), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dc + 2 * m, hom2, m * sizeof(int32_t), cudaMemcpyHostToDevice));
    hwe_kernel<<<(unsigned)ceil_div(m, 128), 128>>>(dc, dc + m, dc + 2 * m, m, midp ? 1 : 0, dp);
    LAUNCH_CHECK();
    CUDA_TRY(cudaMemcpy(p, dp, m * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

int slemm_gpu_marker_qc(slemm_geno* g, int midp, float* maf, float* hwep)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && maf != nullptr && hwep != nullptr, "null argument");
    const int64_t m = g->m;
    DevBuf buf(g->stream);
    uint8_t* b = (uint8_t*)buf.ensure((size_t)m * (sizeof(int64_t) + 2 * sizeof(int32_t) + 2 * sizeof(float)) + 64);
    int64_t* d_pc = reinterpret_cast<int64_t*>(b);
    int32_t* d_c1 = reinterpret_cast<int32_t*>(d_pc + m);
    int32_t* d_c2 = d_c1 + m;
    float* d_maf = reinterpret_cast<float*>(d_c2 + m);
    float* d_hwe = d_maf + m;
    row_counts_device(g, d_pc, d_c1, d_c2);
    marker_qc_kernel<<<(unsigned)ceil_div(m, 128), 128, 0, g->stream>>>(d_pc, d_c1, d_c2, m, g->n, midp ? 1 : 0,
                                                                        d_maf, d_hwe);
    LAUNCH_CHECK();
    CUDA_TRY(cudaMemcpyAsync(maf, d_maf, m * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaMemcpyAsync(hwep, d_hwe, m * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
  });
}

int slemm_gpu_genotype_rows(slemm_geno* g, const int64_t* rows, int cnt, float* out, int64_t ld, int mem)
{
  return guarded([&] {
    CHECK_ARG(g != nullptr && rows != nullptr && out != nullptr, "null argument");
    CHECK_ARG(cnt >= 1 && cnt <= 65535 && ld >= g->n, "bad count or leading dimension");
    for (int c = 0; c < cnt; ++c) CHECK_ARG(rows[c] >= 0 && rows[c] < g->m, "SNP index out of range");
    DevBuf d_rows(g->stream), d_out(g->stream);
    d_rows.ensure(cnt * sizeof(int64_t));
    CUDA_TRY(cudaMemcpyAsync(d_rows.p, rows, cnt * sizeof(int64_t), cudaMemcpyHostToDevice, g->stream));
    float* dst = out;
    int64_t ldd = ld;
    if (mem == SLEMM_MEM_HOST) {
      dst = (float*)d_out.ensure((size_t)g->n * cnt * sizeof(float));
      ldd = g->n;
    }
    genotype_rows_kernel<<<dim3((unsigned)ceil_div(g->n, 256), cnt), 256, 0, g->stream>>>(
        g->G.as<uint32_t>(), g->n_pad / kTileK, d_rows.as<int64_t>(), g->n,
        g->is_view ? g->ind_map.as<int32_t>() : nullptr, dst, ldd);
    LAUNCH_CHECK();
    if (mem == SLEMM_MEM_HOST)
      CUDA_TRY(cudaMemcpy2DAsync(out, ld * sizeof(float), dst, g->n * sizeof(float), g->n * sizeof(float), cnt,
                                 cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
  });
}

}  // extern "C"
