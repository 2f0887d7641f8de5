// internal.h — handle layout and internal entry points shared by the translation units.
#pragma once

#include "common.h"

struct slemm_geno {
  int device = 0;
  int64_t n = 0, m = 0;           // kept individuals, SNPs
  int64_t n_pad = 0, m_pad = 0;   // padded to kTileM
  // Two tiled 2-bit copies of the count matrix (layout in geno.cu):
  //   G : M = SNPs (m_pad rows),        K = individuals (n_pad)  → Z_cᵀU direction
  //   GT: M = individuals (n_pad rows), K = SNPs (m_pad)         → Z_c V direction
  slemm::DevBuf G, GT;
  slemm::DevBuf gm, w, rr;        // FP32, padded with zeros (rr padded with 0)
  slemm::DevBuf Q;                // n_pad × c column-major, zero padded rows
  int c = 0;
  bool weights_set = false;
  int prec = SLEMM_PREC_FP16X2;
  int per_vector = 0;
  int lanczos_mode = 0;           // SLEMM_LANCZOS_* bits of the seeds run on this handle
  int autotune = 0;               // tensor-core plans: 0 the fixed rule, 1 the tuner's, 2 the fixed rule
                                  // with two CTAs per SM wherever N ≤ 64
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // work buffers
  slemm::DevBuf ws_B, ws_D, ws_red, ws_small, ws_T, ws_in, ws_out;
  slemm::DevBuf err;              // int error word of the kernels' bounded waits (zeroed at create)
  slemm::HostScal scal;           // mapped host scalars of the Lanczos steps
  // per-SNP class counts n1, n2 in device memory ([2][m_pad] int32), summed by the pack kernel
  // while it builds the tiles (every handle genotype_create packs; a copy derived from another
  // handle's tiles, like slemm_gwa's model-SNP copy, has none and counts its tiles instead —
  // `dcounts_valid` says which)
  slemm::DevBuf dcounts;
  bool dcounts_valid = false;
  // Z_cᵀ1 per SNP, pc_j − n·gm_j (FP64, stored FP32): the exact product of the centred matrix
  // with a constant vector, set with the weights; the operators remove each input column's mean
  // and add it back through this term (see ops.cu)
  slemm::DevBuf gcorr;
  // A trait view (slemm_gpu_genotype_view) aliases its parent's packed copies (G, GT, n_pad, m_pad
  // are the parent's) and analyses a subset of the parent's individuals: ind_map[r] is the packed
  // individual position of view row r (n entries), ind_inv[i] the view row of position i or −1
  // (n_pad entries), kmask the field masks of the kept positions per K-tile (4 words each, the low
  // bit of each kept 2-bit field) for its own integer counts.
  bool is_view = false;
  slemm::DevBuf ind_map, ind_inv, kmask;
  // per-SNP popcount and class counts of the packed copy (immutable): host copies on first request
  std::vector<int64_t> counts_pc;
  std::vector<int32_t> counts_c1, counts_c2;
  // optional per-launch timing of the packed products (CUDA events on `stream`)
  struct GemmRecord {
    cudaEvent_t start, stop;
    int tc, N, k, pieces, splits, dir;   // dir 1: Zᵀ pass (M = SNPs), 2: Z pass (M = individuals)
    int plan;                            // tensor-core ring plan (GemmArgs::plan)
  };
  bool profiling = false;
  std::vector<GemmRecord> prof_pending;
  std::vector<cudaEvent_t> event_pool;
  struct GemmStat {
    int tc, N, k, pieces, dir, splits, plan;
    int64_t launches;
    double ms;
  };
  std::vector<GemmStat> prof_stats;
  // Every device buffer of the handle: all are stream-ordered on `stream` (the pool keeps freed
  // blocks cached, so building and dropping handles costs no device-wide synchronisation).
  template <class F>
  void for_each_buf(F&& f)
  {
    for (slemm::DevBuf* b : {&G, &GT, &gm, &w, &rr, &Q, &ws_B, &ws_D, &ws_red, &ws_small, &ws_T, &ws_in, &ws_out, &err,
                             &dcounts, &gcorr, &ind_map, &ind_inv, &kmask})
      f(*b);
  }
  void bind_stream()
  {
    for_each_buf([&](slemm::DevBuf& b) {
      b.stream = stream;
      b.ordered = true;
    });
  }
};

namespace slemm {

// ops.cu — one operator application on device buffers (column-major, ld given).
void op_device(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
               float* out, int64_t ld_out);
// H0 operator on a mixed block: columns 0 … nq−1 as H0_quadform_mv, the rest as H0_ldet_mv
// (kind LDET; QUADFORM means nq = k).
void op_device_mixed(slemm_geno* g, int kind, float tau0, const float* in, int64_t ld_in, int k,
                     float* out, int64_t ld_out, int nq);

// Centred Z_cᵀU over SNP rows [r0, r0 + rows) (multiples of 256) on the tensor cores at precision
// prec (SLEMM_PREC_FP16X2, BF16X2 or BF16X3; ops.cu).
void rows_product(slemm_geno* g, int64_t r0, int64_t rows, const float* U, int64_t ldu, int k, float* out,
                  int64_t ldo, int prec);

// reml.cu — orthonormal basis (FP64 column-pivoted QR) of an n×c matrix; returns the rank.
int orthonormal_columns(const std::vector<double>& A, int64_t n, int c, std::vector<double>& Q);

// Column reductions with FP64 accumulation, deterministic two-stage (ops.cu).
// dots[c] = Σ_i a[i,c]·b[i,c] over i < n for c < k (b == nullptr → Σ a²).  Result on device.
void col_dots(slemm_geno* g, const float* a, int64_t lda, const float* b, int64_t ldb,
              int64_t n, int k, double* d_out);
// QtX[l,c] = Σ_i Q[i,l]·X[i,c], double c×k on device.
void proj_coeffs(slemm_geno* g, const float* X, int64_t ldx, int k, double* d_QtX);
// X[:,c] -= Σ_l Q[:,l] QtX[l,c].
void proj_apply(slemm_geno* g, float* X, int64_t ldx, int k, const double* d_QtX);

// lanczos.cu — seed on a device RHS block (n×t, ld = n); `groups` splits the columns into
// groups with their own stopping rule (empty = one group).
slemm_lseed* lanczos_seed_device(slemm_geno* g, int kind, float tau0, const float* dB, int t,
                                 float tol, int maxit, bool verbose, std::vector<int> groups,
                                 int p_freq, int nq = 0);
// Solve for the columns of group `grp`; X has that group's columns (ld = ldx) on device.
int lanczos_solve_device(slemm_lseed* S, double sigma, double tol, float* dX, int64_t ldx, int grp);
// Batched tridiagonal eigensolve on the host (FP64 implicit QL per probe over host threads): delta
// nld×t and beta (nld+1)×t in, D and W2 nld×t out, eigenvalues ascending per probe.
void tridiag_eig_host(const double* delta, const double* beta, int t, int nld, double* D, double* W2);
// L_Solve coefficients of group grp at shift σ (X = Σ_i coef[i·tc+c]·V_i[:,c], V_0 = B, V_i = U_i).
int solve_coeffs(const slemm_lseed* S, double sigma, double tol, int grp, std::vector<double>& coef);
// Inner products B[:,a]ᵀV_i[:,b] for i = 0 … J and each (a, b) pair (V_0 = B), host result
// mom[i·npairs + p].
void lanczos_moments(slemm_lseed* S, const std::vector<std::pair<int, int>>& pairs, int J, std::vector<double>& mom);
// Accessors of the seed object (defined in lanczos.cu).
int lseed_iters(const slemm_lseed* S, int grp);
const double* lseed_delta(const slemm_lseed* S);   // iters × t (row j = step j)
const double* lseed_beta(const slemm_lseed* S);    // (iters+1) × t
int lseed_t(const slemm_lseed* S);
void lseed_free(slemm_lseed* S);

// probes.cu — the reference's normalised Rademacher block (n×n_V, ld) on the device.
void rademacher_device(int seed, int64_t n, int n_V, float* dV, int64_t ld, cudaStream_t st);

// geno.cu — per-SNP popcounts (missing = 1) and class counts n1 (fields 01), n2 (fields 10).
void row_counts_device(slemm_geno* g, int64_t* pc, int32_t* c1, int32_t* c2);

int64_t workspace_bytes(const slemm_geno* g);
// Reads (and clears) the device error word; throws if a kernel gave up a bounded wait.
void check_device_error(slemm_geno* g);
void profile_collect(slemm_geno* g);

}  // namespace slemm
