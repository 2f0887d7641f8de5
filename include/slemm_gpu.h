/*
 * slemm_gpu.h — C ABI of the GB300 engine for SLEMM's packed-genotype path.
 *
 * Every entry point returns an int status (SLEMM_OK = 0, negative on error) and never throws
 * across the ABI.  slemm_gpu_last_error() returns a thread-local message for the last failure.
 * Pointers are plain host or device pointers as stated per call; matrices are column-major
 * FP32 with an explicit leading dimension, like the Eigen MatrixXf the reference passes around.
 *
 * Threading: one host thread per handle; all work is ordered on the handle's CUDA stream.
 * The library starts no host threads of its own.
 *
 * Reference interfaces replaced (paths inside jiang18/slemm):
 *   - the genotype store `std::vector<std::vector<bool>> kmat`      src/option.cpp:347
 *     filled by the .bed decoder                                    src/input.cpp:343-386
 *   - the operator family H0_quadform_mv / H0_ldet_mv / lnr_op_select,
 *     weighted_rmatvec / rmatvec / matvec                          src/reml.cpp:8-233
 *   - L_Seed / L_Solve / SLQ_LDet                                  src/reml.cpp:246-451
 *   - SLDF_REML (DF-REML, --reml --lrt)                            src/reml.cpp:549-690
 *   - LMC_REML  (MC-REML, --reml)                                  src/reml.cpp:730-883
 *   - computeTotalGeneticValuePLINK (--pred GEBV)                  src/pred.cpp:4-141
 *   - the per-variant GRAMMAR-Gamma loop of slemm_gamma            bin/slemm_gamma.py:302-325
 */
#ifndef SLEMM_GPU_H_
#define SLEMM_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define SLEMM_OK               0
#define SLEMM_ERR_ARG         -1   /* invalid argument (null pointer, bad size, bad enum)     */
#define SLEMM_ERR_CUDA        -2   /* a CUDA runtime call failed                               */
#define SLEMM_ERR_NOMEM       -3   /* device or host allocation failed                         */
#define SLEMM_ERR_STATE       -4   /* call out of order (e.g. op before set_weights)           */
#define SLEMM_ERR_RANK        -5   /* fixed-effect design matrix not of full rank              */
#define SLEMM_ERR_NUMERIC     -6   /* non-finite value where a finite one is required          */
#define SLEMM_ERR_UNSUPPORTED -7   /* no sm_103a device, or a size beyond a kernel's limit      */

/* ---- operator kinds (src/reml.cpp:8-233) ------------------------------------------------ */
#define SLEMM_OP_QUADFORM  0  /* out = rr∘ΣZ W Zᵀ(rr∘(v−QQᵀv)) + τ0 v − QQᵀ(·)  H0_quadform_mv :8   */
#define SLEMM_OP_LDET      1  /* out = rr∘Z W Zᵀ(rr∘v) + τ0 v                    H0_ldet_mv     :52  */
#define SLEMM_OP_MATVEC    2  /* out(n×k) = Z_c v,      v is m×k                 matvec         :198 */
#define SLEMM_OP_RMATVEC   3  /* out(m×k) = Z_cᵀ v,     v is n×k                 rmatvec        :160 */
#define SLEMM_OP_WRMATVEC  4  /* out(m×k) = W Z_cᵀ v                              weighted_rmatvec :121 */

/* ---- precision of the packed products --------------------------------------------------- */
#define SLEMM_PREC_FP32    0  /* CUDA-core FP32 FMA on exact integer counts                      */
#define SLEMM_PREC_BF16X2  1  /* tcgen05 BF16 MMA, dense side split hi+lo, FP32 accumulation     */
#define SLEMM_PREC_BF16X3  2  /* tcgen05 BF16 MMA, dense side split hi+mid+lo (≈FP32 mantissa)   */
#define SLEMM_PREC_FP16X2  3  /* tcgen05 FP16 MMA, dense side scaled by a power of two per column
                                 and split hi+lo (22 mantissa bits) at the cost of hi+lo BF16     */

/* Largest number of fixed-effect covariates (columns of X, and so of the projection Q) a fit takes,
 * including the SNPs that --iter_weighting appends as fixed effects. */
#define SLEMM_MAX_COVARIATES 256

/* ---- memory location flags ---------------------------------------------------------------- */
#define SLEMM_MEM_HOST     0
#define SLEMM_MEM_DEVICE   1

/* ---- genotype_create flags ---------------------------------------------------------------- */
#define SLEMM_ROWS_DEVICE  1  /* bed_rows is a device pointer on the current device             */

typedef struct slemm_geno  slemm_geno;   /* packed genotypes resident in HBM + weights         */
typedef struct slemm_lseed slemm_lseed;  /* Lanczos seed system (basis, Jacobi coefficients)  */

/* ---- library / device ------------------------------------------------------------------------ */
const char* slemm_gpu_last_error(void);
int slemm_gpu_version(void);                       /* 10000*major + 100*minor + patch */
/* Selects the device, checks it is sm_103 class. */
int slemm_gpu_init(int device);
/* Number of GPU kernel launches issued by this library since load (all handles). */
int64_t slemm_gpu_launch_count(void);

/* ---- genotype handle ------------------------------------------------------------------------- */
/* Replaces kmat + read_plink_bin_geno_file_and_generate_pxvb_data's decode (src/input.cpp:343-386).
 * bed_rows: host pointer to m SNP-major .bed rows (magic bytes already skipped), row j at
 *   bed_rows + j*row_stride, each row ceil(n_fam/4) bytes, selected SNPs in analysis order.
 * keep_idx: host pointer to n indices into [0, n_fam) of the individuals kept, in order
 *   (NULL = all n_fam individuals; then n must equal n_fam).  The handle's counts, allele
 *   frequencies and centring are those of the kept individuals, so several traits with their
 *   own individual sets take one handle each, all packed from the same rows (with
 *   SLEMM_ROWS_DEVICE, straight from device memory).  n_fam and m must be below 2^31.
 * Codes follow PLINK: 00→0, 10(het)→1, 11→2, 01(missing)→1 allele-2 copies, exactly like the
 * reference's bit decode (missing counts as one copy).  The handle keeps two packed 2-bit
 * copies (SNP-major and individual-major) in HBM.  flags: 0, or SLEMM_ROWS_DEVICE when bed_rows
 * is already in device memory (keep_idx stays a host pointer).  Host rows (pinned or pageable)
 * are copied in 4096-row chunks into device staging buffers while the previous chunk is packed;
 * the call returns when both copies are built and the host rows are no longer read. */
int slemm_gpu_genotype_create(const uint8_t* bed_rows, int64_t n_fam, int64_t m,
                              int64_t row_stride, const int64_t* keep_idx, int64_t n,
                              int flags, slemm_geno** out);
int slemm_gpu_genotype_destroy(slemm_geno* g);
/* A trait view: a handle over the individuals keep_idx (n increasing indices into the parent's
 * individuals) that shares the parent's packed copies instead of packing its own — for several
 * traits with their own missing individuals over one .bed (the reference analyses each trait on its
 * own individual set, src/input.cpp:287, src/option.cpp:320, and so does a view: its counts, allele
 * frequencies, centring, weights and fits are those of its individuals).  The operators read
 * inputs and write outputs through the view's individual map; the products stream the parent's
 * copies.  The view has its own stream, weights, projection and precision; the parent must outlive
 * it and must not be changed meanwhile.  Entry points that read the packed copies directly
 * (gebv, score_terms, gwa_windows, lmm_quadforms, wls, rmatvec_noalloc) return
 * SLEMM_ERR_UNSUPPORTED on a view.  Destroy with slemm_gpu_genotype_destroy. */
int slemm_gpu_genotype_view(slemm_geno* parent, const int64_t* keep_idx, int64_t n, slemm_geno** out);
int slemm_gpu_genotype_dims(const slemm_geno* g, int64_t* n, int64_t* m);
/* Binds the handle's work to a caller stream (cudaStream_t passed as void*; NULL = own stream). */
int slemm_gpu_set_stream(slemm_geno* g, void* stream);
int slemm_gpu_get_stream(const slemm_geno* g, void** stream);

/* Bit-exact integer side outputs (host pointers, length m each, may be NULL):
 * popcnt = Σ_i count_ji (src/reml.cpp:613-621 nz_bits); n0/n1/n2 = genotype classes with
 * missing counted as a heterozygote (src/input.cpp:10-22). */
int slemm_gpu_genotype_counts(slemm_geno* g, int64_t* popcnt, int32_t* n0, int32_t* n1,
                              int32_t* n2);

/* Marker QC (src/input.cpp:388-394; replaces cal_maf_from_genobits, src/weight.cpp:3-15, and
 * cal_hwep_from_genobits, src/input.cpp:10-22): per SNP, maf = |[f>0.5] − f| with
 * f = popcount/float(2n) (FP32), and hwep = float(SNPHWE2(n1, n0, n2, midp)) — the exact HWE test
 * (src/snphwe.cpp:18).  Host pointers, length m each. */
int slemm_gpu_marker_qc(slemm_geno* g, int hwe_midp, float* maf, float* hwep);

/* The exact HWE test alone (SNPHWE2(obs_hets, obs_hom1, obs_hom2, midp), src/snphwe.cpp:18) for m
 * count triples; host pointers; p in FP64. */
int slemm_gpu_hwe_exact(const int32_t* het, const int32_t* hom1, const int32_t* hom2, int64_t m,
                        int midp, double* p);

/* Decoded allele-2 counts (missing = 1) of SNP rows `rows[0 … cnt−1]` for the kept individuals:
 * out[c·ld + i], i < n (the kmat[j][2i] + kmat[j][2i+1] reads of src/option.cpp:471-472). */
int slemm_gpu_genotype_rows(slemm_geno* g, const int64_t* rows, int cnt, float* out, int64_t ld,
                            int mem);

/* gm (m), w (m), rr (n) — host pointers.  gm is the per-SNP mean count, w the per-SNP
 * weight (gw in the reference, src/reml.cpp:622), rr = R^{-1/2} (NULL = all ones). */
int slemm_gpu_set_weights(slemm_geno* g, const float* gm, const float* w, const float* rr);
/* Q: host n×c column-major orthonormal basis of R^{-1/2}X (src/reml.cpp:583-585). c may be 0. */
int slemm_gpu_set_projection(slemm_geno* g, const float* Q, int64_t ldq, int c);
/* prec: SLEMM_PREC_* (a new handle, or view, starts at SLEMM_PREC_FP16X2). */
int slemm_gpu_set_precision(slemm_geno* g, int prec);
/* per_vector != 0 makes every operator run one column at a time (the plain per-vector path). */
int slemm_gpu_set_per_vector(slemm_geno* g, int per_vector);

/* One operator application (src/reml.cpp:8-233).  `in` is n×k (QUADFORM, LDET, RMATVEC,
 * WRMATVEC) or m×k (MATVEC); `out` is n×k or m×k accordingly.  mem = SLEMM_MEM_HOST or
 * SLEMM_MEM_DEVICE for both pointers.  Host calls copy in, run, copy out and synchronise. */
int slemm_gpu_op(slemm_geno* g, int op_kind, float tau0, const float* in, int64_t ld_in, int k,
                 float* out, int64_t ld_out, int mem);

/* ---- Lanczos seed / shifted solves (src/reml.cpp:246-431) ------------------------------- */
/* Lanczos mode of a handle (bits; 0, the default, is the reference's recurrence):
 * SLEMM_LANCZOS_REORTH  each new basis vector is made orthogonal to every stored vector of its
 *                       column (classical Gram-Schmidt with FP64-accurate coefficients over the FP32
 *                       basis in HBM; two passes over the stored basis per step).  The reference
 *                       runs the plain three-term recurrence (src/reml.cpp:293-322), which on
 *                       ill-conditioned systems (window-weighted GREML) needs more steps and stops
 *                       at a step that depends on rounding.
 * The mode applies to every seed run on the handle afterwards (L_Seed, the REML drivers, the
 * gradient, --lmm, --iter_weighting). */
#define SLEMM_LANCZOS_REORTH 1
int slemm_gpu_set_lanczos(slemm_geno* g, int mode);

/* Runs the per-column Lanczos/CG recurrence on B (n×t) with operator op_kind (QUADFORM or LDET)
 * at shift tau0 until max_col |ρ|·‖u‖/‖b‖ ≤ tol or maxit, storing the basis in HBM.  The
 * recurrence scalars are accumulated in FP64.  *iters receives the number of steps j. */
int slemm_gpu_lanczos_seed(slemm_geno* g, int op_kind, float tau0, const float* B, int64_t ldb,
                           int t, float tol, int maxit, int mem, slemm_lseed** out, int* iters);
int slemm_gpu_lseed_destroy(slemm_lseed* s);
/* Jacobi coefficients: beta is t×(iters+1), delta is t×iters, column-major, host FP64. */
int slemm_gpu_lseed_coeffs(const slemm_lseed* s, double* beta, double* delta);
/* X = (A + sigma I)^{-1} B via the stored basis (L_Solve, src/reml.cpp:369-431), CG stopped at
 * relative residual tol.  B must be the seed's right-hand side block. */
int slemm_gpu_lanczos_solve(slemm_lseed* s, float sigma, float tol, float* X, int64_t ldx,
                            int mem);

/* ---- probes (src/reml.cpp:597-605) ------------------------------------------------------------ */
/* The reference's normalised Rademacher block: V (n×n_V, column-major, ld) gets ±1/√n with the
 * signs of std::mt19937(seed + 54321) + uniform_real_distribution<float>(0,1) < 0.5, draw for
 * draw, generated on the GPU.  mem selects a host or device V. */
int slemm_gpu_rademacher(int seed, int64_t n, int n_V, float* V, int64_t ldv, int mem);

/* ---- batched tridiagonal eigensolve + SLQ (src/reml.cpp:440-451, 638-646) -------------- */
/* For t Jacobi matrices (diag delta t×nld, off-diag beta t×(nld+1) with beta[:,1:nld] used),
 * returns eigenvalues D (t×nld, ascending per probe) and squared first eigenvector components W2
 * (t×nld), FP64, computed on the host: an implicit QL per probe, the probes spread over the host's
 * threads (a serial chain of FP64 rotations, which GB300's low FP64 rate makes ~100× slower on the
 * GPU).  Host pointers, column-major. */
int slemm_gpu_tridiag_eig(const double* delta, const double* beta, int t, int nld, double* D,
                          double* W2);

/* ---- REML drivers ----------------------------------------------------------------------------- */
typedef struct {
  int   n_V;        /* Rademacher probes (SLDF) or MC samples n_MC (LMC)                 */
  int   seed;       /* --seed                                                             */
  float tol_L;      /* --rel_tol (Lanczos relative tolerance)                              */
  float s2max;      /* --max_heritability                                                  */
  float s2min;      /* 1e-4 in the reference                                               */
  float tol_VC;     /* 1e-4 in the reference (golden-section tolerance on h2)              */
  int   maxit;      /* 600 in the reference                                                */
  int   verbose;    /* print the reference's progress lines to stdout                      */
} slemm_reml_opts;

#define SLEMM_TRACE_MAX 64
typedef struct {
  float vg, ve, h2, lrt;  /* variance components, h2 = vg/(vg+ve), LRT (SLDF only, else 0) */
  int   iters_y, iters_Q, iters_V;   /* Lanczos steps per seed system                     */
  int   n_criterion;      /* REML criterion (or first-order function) evaluations          */
  double seconds;         /* wall time inside the call                                     */
  double t_setup;         /* QR, weights, probe or MC draws                                */
  double t_seed;          /* Lanczos recurrence (operator applications)                    */
  double t_search;        /* golden-section or secant search on h2                         */
  double t_final;         /* BLUP, BLUE and copies back                                    */
  /* The search's evaluations in order (the first SLEMM_TRACE_MAX): h2 of each point and its
   * criterion — 2logLL of the golden-section search (src/reml.cpp:512-541) or the first-order
   * function of the secant iterations (src/reml.cpp:821-851).  Two runs took the same branches
   * exactly when their h2_points agree. */
  int    n_points;
  float  h2_points[SLEMM_TRACE_MAX];
  double f_points[SLEMM_TRACE_MAX];
  /* --iter_weighting only (0 otherwise): the equal-weight first stage's Lanczos steps of its
   * probe block (iters_V of that fit) and its criterion evaluations. */
  int    first_iters_V, first_n_criterion;
} slemm_reml_result;

/* DF-REML with Rademacher probes + golden-section search (src/reml.cpp:549-690).
 * Host pointers: rvec (n; NULL = ones), X (n×c col-major, ldx), y (n), persnp (m, already
 * normalised to mean 1 by the caller as option.cpp:424 does).  Outputs (host): Py (n),
 * snp_blup (m), blue (c), var_blue (c×c, may be NULL). */
int slemm_gpu_reml_sldf(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                        const float* y, const float* persnp, const slemm_reml_opts* opts,
                        float* Py, float* snp_blup, float* blue, float* var_blue,
                        slemm_reml_result* res);
/* MC-REML with secant iterations (src/reml.cpp:730-883), same argument conventions. */
int slemm_gpu_reml_lmc(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                       const float* y, const float* persnp, const slemm_reml_opts* opts,
                       float* Py, float* snp_blup, float* blue, slemm_reml_result* res);

/* Gradient of the REML log-likelihood of the DF-REML model at (sigma_g2, sigma_e2) with respect to
 * the variance components and to per-window SNP weights: Var(y) = sigma_g2·Z_c W Z_cᵀ + sigma_e2·R,
 * W_j = gw_j·wwin[window[j]] with gw the reference's per-SNP weights (src/reml.cpp:613-622 from
 * persnp) and window[j] in [-1, n_win) (-1: weight 1, no window).  Traces by Hutchinson with the
 * reference's n_V normalised Rademacher probes of `seed` (src/reml.cpp:597-605); P·[y | probes]
 * by one projected Lanczos seed and solve (tolerance tol).  grad[0] = ∂ℓ/∂sigma_g2,
 * grad[1] = ∂ℓ/∂sigma_e2, grad[2 + k] = ∂ℓ/∂wwin[k].  Host pointers; leaves the handle's weights
 * set to W. */
int slemm_gpu_reml_grad(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                        const float* y, const float* persnp, const int32_t* window, int n_win,
                        const float* wwin, double sigma_g2, double sigma_e2, int n_V, int seed,
                        float tol, double* grad);

/* Iterative window weighting (`--iter_weighting`, src/option.cpp:437-530): equal-weight GREML
 * (DF-REML when lrt and n < 5000, else MC-REML with n_MC samples), per-SNP variance
 * 2·maf(1−maf)·b² normalised to mean 1, fixed-effect SNPs by clumping (largest variance above
 * sig_chisq, kept when independent at indep_r2), window weights over window_size+1 SNPs, then the
 * window-weighted GREML (DF-REML when lrt, else MC-REML with n_MC_final samples) with the fixed
 * SNPs appended to the covariates; their snp_blup entries are their BLUE.  maf is per SNP (the
 * marker QC values).  Outputs (host): Py (n), snp_blup (m), blue (c + max_fixed; the first
 * c + n_fixed used), var_blue ((c+n_fixed)², DF-REML only, may be NULL), persnp_out (m, the final
 * weights, may be NULL), fixed_idx (max_fixed, may be NULL), n_fixed. */
typedef struct {
  int   window_size;  /* --window_size, even (20 unless given, src/option.cpp:303-307)     */
  float sig_chisq;    /* --sig_chisq (1e6)                                                */
  float indep_r2;     /* --indep_r2 (0.5)                                                 */
  int   lrt;          /* --lrt                                                            */
  int   n_MC;         /* MC samples of an MC-REML first stage (0: max(min(4e9/n², 30), 3))  */
  int   n_MC_final;   /* MC samples of an MC-REML second stage (0: n_MC; --using_nr_opt: n_V) */
  int   max_fixed;    /* capacity of blue / fixed_idx beyond the c covariates              */
} slemm_window_opts;
int slemm_gpu_reml_iter_weighting(slemm_geno* g, const float* rvec, const float* X, int64_t ldx,
                                  int c, const float* y, const float* persnp, const float* maf,
                                  const slemm_reml_opts* opts, const slemm_window_opts* wopts,
                                  float* Py, float* snp_blup, float* blue, float* var_blue,
                                  float* persnp_out, int64_t* fixed_idx, int* n_fixed,
                                  slemm_reml_result* res);

/* GWAS step 1 quadratic forms (`--lmm` with real markers, src/reml.cpp:919-981) for the
 * .gstat.txt file: samples min(num_qf, #eligible) markers with gm·n > 20 and (2−gm)·n > 20 in
 * the reference's order (std::random_shuffle on the C library's unseeded rand(), restated) and
 * returns per marker xPy, xPx, xBx (window of window_size markers, even, ≤ 5000) and xSx.
 * Uses the handle's weights (gm, gw, rr) and projection Q, as left by the REML driver; Py (n) and
 * tau1 = ve/vg are that fit's.  Host pointers; variants/x* hold num_qf entries; *count = sampled. */
int slemm_gpu_lmm_quadforms(slemm_geno* g, const float* Py, float tau1, float tol_L, int num_qf,
                            int window_size, int64_t* variants, float* xPy, float* xPx, float* xBx,
                            float* xSx, int* count);

/* Windowed MLMA of slemm_gwa.py (bin/slemm_gwa.py:259-434) for the variants test_begin …
 * test_end (handle indices, one chromosome).  The handle holds every variant of the .bed for the
 * GWA samples.  y = the Py column of .reml.py.txt, R its last column (NULL = ones), covar its
 * covariates (n×c, ldc); model_idx = increasing handle indices of the chromosome's model SNPs
 * (.reml.snp.csv); block_size = the .gstat.txt WindowSize; tau = Ve/Vg; model_snp_ct, snp_var
 * from .reml.vc.csv; cfactor = mean(xBx/xPx) of .gstat.txt; mac the final minor-allele-count
 * filter.  Outputs per tested variant (host): beta, se, chisq (FP32, allele 1 = the .bim's
 * allele 1 as pgenlib counts it) and pval (FP64); NaN where filtered. */
int slemm_gpu_gwa_windows(slemm_geno* g, const float* y, const float* R, const float* covar,
                          int64_t ldc, int c, const int64_t* model_idx, int64_t n_model,
                          int64_t test_begin, int64_t test_end, int block_size, float tau,
                          int64_t model_snp_ct, float cfactor, float snp_var, int mac,
                          float* beta, float* se, float* chisq, double* pval);

/* SNP effects by weighted least squares (`--wls`, src/wls.cpp:4-129): with
 * Z̃ = (I − QQᵀ)(rr∘(Cnt − gm)), rr = rvec^(−1/2), Q an orthonormal basis of rr∘X,
 * snp_blup = (Z̃ᵀZ̃ + 1e-4·mean(diag)·I)⁻¹ Z̃ᵀ(I − QQᵀ)(rr∘y), Cholesky in FP32 like the reference.
 * Sets the handle's weights (gm = popcount/n, rr) and projection.  Needs 4·m² bytes of device
 * memory for the m×m system.  Host pointers: rvec (n, NULL = ones), X (n×c, ldx), y (n),
 * snp_blup (m). */
int slemm_gpu_wls(slemm_geno* g, const float* rvec, const float* X, int64_t ldx, int c,
                  const float* y, float* snp_blup);

/* ---- prediction and GWAS score statistics ------------------------------------------------- */
/* GEBV: tgv_i = Σ_j (flip_j ? 2−count_ij : count_ij)·alpha_j, FP64 accumulation of exact
 * integer counts (src/pred.cpp:112-130).  Uses the handle's genotypes (no centring). flip: m
 * bytes or NULL.  Host pointers. */
int slemm_gpu_gebv(slemm_geno* g, const double* alpha, const uint8_t* flip, double* tgv);
/* GRAMMAR-Gamma per-SNP terms (bin/slemm_gamma.py:302-325), counting allele 1 like pgenlib:
 * x = 2 − count.  For every SNP j: s_j = Σx; if s_j ≤ mac or 2n − s_j ≤ mac → NaN; else
 * xy_j = (x − s/n)·y and xx_j = ‖(I−QQᵀ)(rr∘(x − s/n))‖².  y is n (host).  Projection and rr
 * come from the handle.  Outputs xy, xx (m, host). */
int slemm_gpu_score_terms(slemm_geno* g, const float* y, int mac, float* xy, float* xx);

/* ---- operator without device allocation ----------------------------------------------------------- */
/* No counterpart in the reference.  out (m×k) = Z_cᵀ v (n×k) on the FP32 CUDA-core path, the same
 * product as slemm_gpu_op(SLEMM_OP_RMATVEC), for callers that cannot allocate device memory (a
 * framework that has reserved the GPU's memory for its own pool, or a loop where cudaMalloc's
 * device-wide synchronisation is not allowed).  v and out are device pointers; the call allocates
 * nothing and returns without synchronising (work queued on the handle's stream).  Its scratch is
 * one static device array of SLEMM_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library;
 * calls needing more (about 4·k·(n + m) bytes plus split-K partials) fail with
 * SLEMM_ERR_UNSUPPORTED.  The call runs with the handle's device current (the caller's current
 * device is restored on return), so the array and the launches are always those of the handle's
 * GPU.  The first call on a device looks up the array's address — make it before any stream
 * capture; the address is kept for the life of the process (do not use the call after a
 * cudaDeviceReset).  Calls share the array: calls that overlap on the GPU race. */
#define SLEMM_NOALLOC_SCRATCH_BYTES (32u << 20)
int slemm_gpu_rmatvec_noalloc(slemm_geno* g, const float* v, int64_t ldv, int k, float* out,
                              int64_t ldo);

/* ---- split-K autotuner (no counterpart in the reference, whose subset size is a flag,
 * src/option.cpp:53-78) ------------------------------------------------------------------------- */
/* on = 1: the handle's tensor-core passes pick their split-K count and ring plan by timing, at the
 * first pass of each shape (device, N, pieces, K-tiles, padded rows), the fixed rule's count and
 * up to five counts near it that fill the last wave of CTAs well — and, for N ≤ 64, the plan with
 * one 128-row tile per CTA and two CTAs per SM at up to three counts — one warm-up and two timed
 * launches each, CUDA events on the handle's stream — and keep the fastest when it beats the
 * rule's by ≥ 3 %.
 * Decisions are cached for the process (shared by all handles); nothing is tuned while the stream
 * is being captured.  Plans change the order of the split-K sums, so results of a tuned handle
 * may differ from a default one's in the last bits.  on = 0 (the default): the fixed rule. */
/* on = 2: no timing; every tensor-core pass with N ≤ 64 takes the two-CTAs-per-SM plan at its own
 * fixed-rule count. */
int slemm_gpu_set_autotune(slemm_geno* g, int on);
/* The cached decisions: *rows = their number; for r < max_rows, info[7r …] = {device, N, pieces,
 * rule's splits, chosen splits, chosen plan (0: the default ring, 1: two CTAs per SM), candidates
 * timed}, shape[2r …] = {K-tiles, padded rows},
 * ms[2r …] = {rule's ms per launch, chosen ms per launch}.  Any of info, shape, ms may be NULL. */
int slemm_gpu_autotune_table(int max_rows, int* rows, int32_t* info, int64_t* shape, double* ms);

/* ---- measurement ---------------------------------------------------------------------------------- */
/* Per-launch timing of the packed products with CUDA events on the handle's stream (no
 * counterpart in the reference, which only prints wall-clock times, src/option.cpp:21-34).
 * Reads the statistics gathered so far (rows of info, 7 per shape = {tc, N, k, pieces, dir,
 * splits, plan}, launch count, total ms), then: enable = 1 clears and starts recording, 0 clears and stops, −1 leaves the
 * state as it is.  *rows receives the number of distinct launch shapes. */
int slemm_gpu_profile(slemm_geno* g, int enable, int max_rows, int* rows, int32_t* info,
                      int64_t* launches, double* ms);

/* ---- failure-path test support -------------------------------------------------------------- */
/* No counterpart in the reference.  Every wait inside the tensor-core product is bounded (2 s);
 * a wait that runs out sets the handle's device error word, makes the CTA drain its copies in
 * flight and free its tensor memory, and the call returns SLEMM_ERR_CUDA.  This makes the next
 * tensor-core launch (any handle, this process) skip the dense-operand copy of stage `stage` in
 * its first CTA, so that CTA's waits run out exactly as they would if a copy never arrived;
 * stage < 0 clears a pending request.  One-shot: the launch that uses it resets it. */
int slemm_gpu_test_withhold_b_stage(int stage);

#ifdef __cplusplus
}
#endif
#endif /* SLEMM_GPU_H_ */
