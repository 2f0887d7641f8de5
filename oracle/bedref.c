/*
 * bedref.c — ORACLE (test infrastructure only; never linked into the product).
 *
 * Plain-C restatement of the reference's integer genotype path, used by tests/, smoke() and
 * bench.py's cpu_baseline leg as the checker.  Each function cites what it restates
 * (paths inside jiang18/slemm).
 */
#include <stdint.h>
#include <stddef.h>

/* src/input.cpp:343-386 — SNP-major .bed decode.  For each 2-bit code the reference reads bits
 * b[k], b[k+1] of the byte (LSB first) into kmat, which starts all-true (option.cpp:347) and only
 * receives `false` for zero bits; the allele count used everywhere is b[k] + b[k+1]
 * (reml.cpp:33).  So 00→0, 01(missing)→1, 10(het)→1, 11→2.  Individuals with keep[i]==0 are
 * skipped (input.cpp:370).  rows: m rows of row_bytes; out: m×n counts, row-major. */
void oracle_bed_decode(const uint8_t* rows, int64_t m, int64_t n_fam, int64_t row_bytes,
                       const uint8_t* keep, uint8_t* out, int64_t n)
{
  for (int64_t j = 0; j < m; ++j) {
    const uint8_t* r = rows + j * row_bytes;
    int64_t kk = 0;
    for (int64_t i = 0; i < n_fam; ++i) {
      if (keep && !keep[i]) continue;
      unsigned byte = r[i >> 2];
      unsigned code = (byte >> (2 * (i & 3))) & 3u;
      unsigned b0 = code & 1u, b1 = (code >> 1) & 1u;
      if (kk < n) out[j * n + kk] = (uint8_t)(b0 + b1);
      ++kk;
    }
  }
}

/* src/reml.cpp:28-35 (and 136-142, 174-181, 212-219) — one SNP subset of the reference's
 * operator loop: kmat bits of SNPs j … j+m−1 (all individuals) decoded to the FP32 column
 * count − gm (b[k] + b[k+1] − gm, the missing code counting 1), written row-major as m rows of n
 * floats (the subset matrix the reference's SGEMMs read).  Used by the timed CPU baseline. */
void oracle_decode_centred_f32(const uint8_t* rows, int64_t m, int64_t n, int64_t row_bytes,
                               const float* gm, float* out)
{
  for (int64_t j = 0; j < m; ++j) {
    const uint8_t* r = rows + j * row_bytes;
    float* o = out + j * n;
    const float g = gm[j];
    const float v[4] = {0.0f - g, 1.0f - g, 1.0f - g, 2.0f - g};   /* by 2-bit code */
    const int64_t full = n >> 2;
    for (int64_t b = 0; b < full; ++b) {
      const unsigned byte = r[b];
      o[4 * b + 0] = v[byte & 3u];
      o[4 * b + 1] = v[(byte >> 2) & 3u];
      o[4 * b + 2] = v[(byte >> 4) & 3u];
      o[4 * b + 3] = v[(byte >> 6) & 3u];
    }
    for (int64_t i = full * 4; i < n; ++i) o[i] = v[(r[i >> 2] >> (2 * (i & 3))) & 3u];
  }
}

/* src/reml.cpp:613-621 (and weight.cpp:7-12) — number of set kmat bits per SNP row. */
void oracle_popcounts(const uint8_t* counts, int64_t m, int64_t n, int64_t* pc)
{
  for (int64_t j = 0; j < m; ++j) {
    int64_t s = 0;
    for (int64_t i = 0; i < n; ++i) s += counts[j * n + i];
    pc[j] = s;
  }
}

/* src/input.cpp:10-22 — genotype class counts: both bits set → n2, one bit → n1, none → n0
 * (a missing code 01 has one bit set, so it lands in n1). */
void oracle_hwe_counts(const uint8_t* counts, int64_t m, int64_t n, int32_t* n0, int32_t* n1,
                       int32_t* n2)
{
  for (int64_t j = 0; j < m; ++j) {
    int32_t c0 = 0, c1 = 0, c2 = 0;
    for (int64_t i = 0; i < n; ++i) {
      uint8_t c = counts[j * n + i];
      if (c == 2) c2++;
      else if (c == 1) c1++;
      else c0++;
    }
    n0[j] = c0; n1[j] = c1; n2[j] = c2;
  }
}

/* src/weight.cpp:3-15 — MAF in FP32: f = nz_bits/float(2n); maf = |[f>0.5] − f|. */
void oracle_maf(const int64_t* pc, int64_t m, int64_t n, float* maf)
{
  for (int64_t j = 0; j < m; ++j) {
    int nz = (int)pc[j];
    float f = nz / (float)(2 * n);
    float g = (f > 0.5f) ? 1.0f : 0.0f;
    float d = g - f;
    maf[j] = d < 0 ? -d : d;
  }
}

/* src/reml.cpp:620 — gm = nz_bits/float(n), FP32. */
void oracle_gm(const int64_t* pc, int64_t m, int64_t n, float* gm)
{
  for (int64_t j = 0; j < m; ++j) gm[j] = (int)pc[j] / (float)n;
}

/* src/pred.cpp:154-172 — GEBV accumulation: tgv += (flip ? 2−z : z)·alpha_j in FP64, SNP by SNP
 * in file order. counts: m×n row-major (full .fam, no filtering in --pred). */
void oracle_gebv(const uint8_t* counts, int64_t m, int64_t n, const double* alpha,
                 const uint8_t* flip, double* tgv)
{
  for (int64_t i = 0; i < n; ++i) tgv[i] = 0.0;
  for (int64_t j = 0; j < m; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      int z = counts[j * n + i];
      if (flip && flip[j]) z = 2 - z;
      tgv[i] += (double)z * alpha[j];
    }
  }
}
