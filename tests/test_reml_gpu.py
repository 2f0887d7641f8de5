"""GPU parity of the Lanczos engine, the REML drivers, GEBV prediction and the GWAS score terms
against the oracle (reference src/reml.cpp, src/pred.cpp, bin/slemm_gamma.py).

Tolerances (stated per the target accuracy of the port):
  h² vs the FP64 oracle                         |Δ| ≤ 1e-4 (DF-REML and MC-REML), with the DF-REML
                                                 golden-section points equal to the oracle's up to
                                                 the first branch the oracle takes by a 2logLL margin
                                                 ≤ 2e-3 (conftest.check_gss_branches)
  SNP-BLUP / GEBV correlation with the oracle    ≥ 0.99999
  GWAS −log10 p vs the reference script output   |Δ| ≤ 1e-3
"""
import math
import os

import numpy as np
import pytest

from conftest import check_gss_branches, make_case
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _problem(n=1500, m=2000, seed=31, h2=0.5, c=2, rvar=True):
    counts, _ = synth.simulate_counts(n, m, seed=seed)
    rows = synth.encode_bed(counts)
    y, _, _ = synth.simulate_phenotype(counts, h2, n_causal=200, seed=seed)
    rng = np.random.default_rng(seed)
    rvec = rng.uniform(0.8, 1.4, n).astype(np.float32) if rvar else None
    X = np.column_stack([np.ones(n)] + [rng.standard_normal(n) for _ in range(c - 1)]).astype(np.float32)
    persnp = rng.uniform(0.5, 1.5, m).astype(np.float32)
    persnp /= persnp.mean()
    return counts, rows, y.astype(np.float32), rvec, X, persnp


def test_lanczos_seed_and_solve_vs_oracle(gpu):
    counts, rows, y, rvec, X, persnp = _problem(n=900, m=700)
    n, m = counts.shape[1], counts.shape[0]
    pc = orc.popcounts(counts)
    gm = orc.genotype_mean(pc, n)
    gw = orc.snp_weights(gm, persnp)
    rr = (1 / np.sqrt(rvec)).astype(np.float32)
    Q, _, _ = orc.qr_colpiv(rr[:, None] * X)
    B = np.random.default_rng(1).standard_normal((n, 4)).astype(np.float32)
    B /= np.linalg.norm(B, axis=0)
    ref = orc.Operators(counts, gm, gw, rr, Q, dtype=np.float64)
    tau0 = 0.4285714
    rs = orc.L_Seed(ref, "ldet", tau0, B, tol=5e-4)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, gw, rr)
        g.set_projection(Q)
        g.set_precision(_lib.PREC_BF16X3)
        s = g.L_Seed("ldet", tau0, B, tol=5e-4)
        beta, delta = s.coeffs()
        assert abs(s.iters - rs["iters"]) <= 1
        k = min(s.iters, rs["iters"], 8)
        assert np.allclose(delta[:, :k], rs["delta"][:, :k], rtol=1e-5)
        assert np.allclose(beta[:, :k + 1], rs["beta"][:, :k + 1], rtol=1e-5)
        for sigma in (0.0, 0.8):
            X_ = s.L_Solve(sigma, 1e-6)
            Xr = orc.L_Solve(rs, B.astype(np.float64), sigma, 1e-6)
            assert np.linalg.norm(X_ - Xr) / np.linalg.norm(Xr) < 1e-4
        s.close()


def test_tridiag_eig_vs_scipy(gpu):
    from scipy.linalg import eigh_tridiagonal
    rng = np.random.default_rng(5)
    t, nld = 7, 45
    delta = rng.uniform(1, 3, (t, nld))
    beta = np.abs(rng.normal(0, 0.5, (t, nld + 1)))
    D, W2 = api.tridiag_eig(delta, beta)
    for p in range(t):
        d, v = eigh_tridiagonal(delta[p], beta[p, 1:nld])
        assert np.allclose(D[p], d, rtol=1e-12, atol=1e-12)
        assert np.allclose(W2[p], v[0] ** 2, rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("prec", [_lib.PREC_FP16X2, _lib.PREC_BF16X2, _lib.PREC_FP32])
def test_sldf_reml_vs_oracle(gpu, prec):
    counts, rows, y, rvec, X, persnp = _problem()
    n, m = counts.shape[1], counts.shape[0]
    r64 = orc.SLDF_REML(counts, rvec, X, y, persnp, seed=3, n_V=12, dtype=np.float64)
    with api.Genotypes(rows, n) as g:
        g.set_precision(prec)
        r = g.SLDF_REML(rvec, X, y, persnp, seed=3, n_V=12)
    check_gss_branches(r["trace"], r64["gss"], 2e-3)
    assert abs(r["h2"] - r64["h2"]) <= 1e-4
    assert math.isclose(r["vg"], r64["vg"], rel_tol=2e-3)
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
    assert np.allclose(r["blue"], r64["blue"], rtol=5e-3, atol=5e-3)
    assert abs(r["lrt"] - r64["lrt"]) <= 1e-2 * max(1.0, abs(r64["lrt"]))


@pytest.mark.parametrize("c", [70, 256])
def test_sldf_reml_many_covariates_vs_oracle(gpu, c):
    """Covariate counts above the one-block limits of the reduction kernels (a warp per covariate
    in the projection's coefficient loads): 70 and the maximum, SLEMM_MAX_COVARIATES = 256 —
    --iter_weighting appends the fixed SNPs to the covariates, so a large c is ordinary input.
    One more covariate is refused with an argument error."""
    counts, rows, y, rvec, X, persnp = _problem(n=1500, m=1200, seed=37, c=c)
    n = counts.shape[1]
    r64 = orc.SLDF_REML(counts, rvec, X, y, persnp, seed=3, n_V=12, dtype=np.float64)
    with api.Genotypes(rows, n) as g:
        g.set_precision(_lib.PREC_FP16X2)
        r = g.SLDF_REML(rvec, X, y, persnp, seed=3, n_V=12)
        check_gss_branches(r["trace"], r64["gss"], 2e-3)
        assert abs(r["h2"] - r64["h2"]) <= 1e-4
        assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
        assert np.allclose(r["blue"], r64["blue"], rtol=5e-3, atol=5e-3)
        if c == 256:
            X2 = np.column_stack([X, np.random.default_rng(2).standard_normal(n)]).astype(np.float32)
            with pytest.raises(_lib.SlemmError) as e:
                g.SLDF_REML(rvec, X2, y, persnp, seed=3, n_V=12)
            assert e.value.code == -1


def test_per_trait_individual_sets_vs_oracle(gpu):
    """Several traits with their own missing individuals (5 %, 20 %, 40 %) from one set of .bed
    rows held in device memory: each trait's handle is packed for its individuals (the reference
    analyses each trait on its own individual set, src/input.cpp:287, src/option.cpp:320), so
    its counts, means and fit equal the oracle's on that subset."""
    import torch
    n_fam, m = 1600, 1500
    counts, _ = synth.simulate_counts(n_fam, m, seed=43)
    rows_dev = torch.from_numpy(synth.encode_bed(counts)).cuda()
    rng = np.random.default_rng(43)
    persnp = np.ones(m, np.float32)
    for t, frac in enumerate((0.05, 0.2, 0.4)):
        keep = np.sort(rng.choice(n_fam, size=n_fam - int(frac * n_fam), replace=False)).astype(np.int64)
        ct = np.ascontiguousarray(counts[:, keep])
        y, _, _ = synth.simulate_phenotype(ct, 0.5, n_causal=150, seed=100 + t)
        y = y.astype(np.float32)
        X = np.column_stack([np.ones(keep.size), rng.standard_normal(keep.size)]).astype(np.float32)
        r64 = orc.SLDF_REML(ct, None, X, y, persnp, seed=3, n_V=12, dtype=np.float64)
        with api.Genotypes(rows_dev, n_fam, keep_idx=keep) as g:
            assert np.array_equal(g.counts()[0], orc.popcounts(ct))
            r = g.SLDF_REML(None, X, y, persnp, seed=3, n_V=12)
        check_gss_branches(r["trace"], r64["gss"], 2e-3)
        assert abs(r["h2"] - r64["h2"]) <= 1e-4
        assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999


def test_lmc_reml_vs_oracle(gpu):
    counts, rows, y, rvec, X, persnp = _problem(seed=37, h2=0.4)
    n = counts.shape[1]
    r64 = orc.LMC_REML(counts, rvec, X, y, persnp, seed=5, n_MC=4, dtype=np.float64)
    with api.Genotypes(rows, n) as g:
        r = g.LMC_REML(rvec, X, y, persnp, seed=5, n_MC=4)
    assert abs(r["h2"] - r64["h2"]) <= 1e-4
    assert math.isclose(r["vg"], r64["vg"], rel_tol=1e-3)
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
    assert np.allclose(r["blue"], r64["blue"], rtol=1e-3, atol=1e-3)


def test_gebv_vs_oracle(gpu):
    rows, _, dec = make_case(1003, 517, seed=41, missing=0.01)
    rng = np.random.default_rng(2)
    alpha = rng.standard_normal(517)
    flip = (rng.random(517) < 0.3).astype(np.uint8)
    ref = orc.gebv(dec, alpha, flip)
    with api.Genotypes(rows, 1003) as g:
        out = g.gebv(alpha, flip)
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-10)
    assert np.corrcoef(out, ref)[0, 1] >= 0.99999


def test_score_terms_vs_reference_script(gpu):
    """GRAMMAR-Gamma statistics through the GPU terms vs the reference slemm_gamma.py output."""
    d = os.path.join(GOLD, "gamma_case")
    n_fam = sum(1 for _ in open(os.path.join(d, "geno.fam")))
    raw = np.fromfile(os.path.join(d, "geno.bed"), dtype=np.uint8)[3:]
    rows = raw.reshape(-1, (n_fam + 3) // 4)
    py = [l.split() for l in open(os.path.join(d, "s1.reml.py.txt")).read().splitlines()[1:]]
    Py = np.array([float(r[1]) for r in py], np.float32)
    cov = np.array([[float(v) for v in r[2:-1]] for r in py], np.float32)
    R = np.array([float(r[-1]) for r in py], np.float32)
    rr = (1.0 / np.sqrt(R)).astype(np.float32)
    from scipy import linalg
    Q = linalg.qr(np.transpose(np.transpose(cov) * rr), mode="economic")[0]
    gs = [l.split() for l in open(os.path.join(d, "s1.gstat.txt")).read().splitlines()[1:]]
    cf = orc.mean_wo_outliers([float(r[9]) / float(r[7]) for r in gs])
    snp_var = float(open(os.path.join(d, "s1.reml.vc.csv")).read().splitlines()[2].split(",")[1])
    m = rows.shape[0]
    with api.Genotypes(rows, n_fam) as g:
        g.set_weights(np.zeros(m, np.float32), np.zeros(m, np.float32), rr)
        g.set_projection(Q)
        xy, xx = g.score_terms(Py, mac=20)
    beta, se, chisq, p = orc.gamma_stats(xy, xx, cf, snp_var)
    ref = [l.split("\t") for l in open(os.path.join(d, "gamma.txt")).read().splitlines()[1:]]
    rp = np.array([float(r[9]) for r in ref])
    ok = np.isfinite(rp)
    assert np.array_equal(ok, np.isfinite(p))
    assert np.max(np.abs(np.log10(p[ok]) - np.log10(rp[ok]))) <= 1e-3


def test_reml_gradient_vs_oracle(gpu):
    """Gradient of the REML log-likelihood (σ_g², σ_e², 8 window weights) against the FP64 oracle
    with the same 30 Rademacher probes: the Hutchinson estimate is deterministic given them."""
    counts, rows, y, rvec, X, persnp = _problem(n=1500, m=1200, seed=73)
    n, m = counts.shape[1], counts.shape[0]
    window = np.repeat(np.arange(8), m // 8).astype(np.int32)
    window[:30] = -1
    wwin = np.random.default_rng(4).uniform(0.5, 2.0, 8).astype(np.float32)
    sg2, se2, n_V, seed = 0.55, 0.8, 30, 3
    ref = orc.reml_grad_dense(counts, rvec, X, y, persnp, window, wwin, sg2, se2,
                              probes=orc.rademacher(seed, n, n_V))
    with api.Genotypes(rows, n) as g:
        r = g.REML_grad(rvec, X, y, persnp, window, wwin, sg2, se2, n_V=n_V, seed=seed, tol=1e-6)
    assert abs(r["d_sigma_g2"] - ref[0]) <= 2e-3 * abs(ref[0])
    assert abs(r["d_sigma_e2"] - ref[1]) <= 2e-3 * abs(ref[1])
    assert np.max(np.abs(r["d_w"] - ref[2])) <= 2e-3 * np.max(np.abs(ref[2]))


@pytest.mark.parametrize("unit_rr", [True, False])
def test_score_terms_both_paths_vs_oracle(gpu, unit_rr):
    """slemm_gamma's per-variant xy, xx (bin/slemm_gamma.py:302-319) through both GPU paths: the
    tensor-core product when every rr is 1, the FP64 per-genotype kernel otherwise."""
    counts, rows, _, rvec, X, _ = _problem(n=3001, m=900, seed=71, c=3, rvar=not unit_rr)
    n, m = counts.shape[1], counts.shape[0]
    rr = np.ones(n, np.float32) if unit_rr else (1 / np.sqrt(rvec)).astype(np.float32)
    Q, _, _ = orc.qr_colpiv(rr[:, None] * X)
    Py = np.random.default_rng(5).standard_normal(n).astype(np.float32)
    want_xy, want_xx = orc.gamma_terms(counts, Py, rr, Q, 20)
    with api.Genotypes(rows, n) as g:
        g.set_weights(np.zeros(m, np.float32), np.zeros(m, np.float32), rr)
        g.set_projection(Q.astype(np.float32))
        xy, xx = g.score_terms(Py, mac=20)
    ok = np.isfinite(want_xy)
    assert np.array_equal(ok, np.isfinite(xy)) and np.array_equal(ok, np.isfinite(xx))
    assert np.allclose(xy[ok], want_xy[ok], rtol=1e-4, atol=1e-4 * np.max(np.abs(want_xy[ok])))
    assert np.allclose(xx[ok], want_xx[ok], rtol=1e-5)


@pytest.mark.parametrize("seed,n,n_V", [(0, 37, 3), (1, 1000, 5), (42, 2049, 2), (7, 100003, 1),
                                        (5, 1, 1000), (9, 200, 3000), (11, 79872, 4), (3, 100000, 64)])
def test_gpu_probes_match_reference_draws(gpu, seed, n, n_V):
    """The GPU MT19937 probe block equals the libstdc++ draws of src/reml.cpp:597-605 bit for bit.

    The cases cover one chunk (no jump), several doubling levels, a column shorter than one
    generator phase (n < 227), chunk boundaries that fall on column boundaries, and the
    64-probe block of the n = 100,000 benchmark (21 chunks)."""
    import ctypes
    V = np.zeros((n, n_V), np.float32, order="F")
    _lib.check(gpu.slemm_gpu_rademacher(seed, n, n_V, V.ctypes.data_as(ctypes.c_void_p), n, 0))
    ref = orc.rademacher(seed, n, n_V)
    assert np.array_equal(V, ref)


def _strong_problem(n=1500, m=2000, seed=43):
    """A polygenic trait plus three large-effect SNPs (their per-SNP variance is >100× the mean;
    the next largest is ~14×), so the fixed-SNP selection is clear-cut."""
    counts, _ = synth.simulate_counts(n, m, seed=seed)
    rows = synth.encode_bed(counts)
    y, _, _ = synth.simulate_phenotype(counts, 0.3, n_causal=200, seed=seed)
    for j in (300, 301, 1200):
        x = counts[j].astype(np.float64)
        y = y + 0.35 * (x - x.mean()) / x.std()
    X = np.ones((n, 1), np.float32)
    return counts, rows, y.astype(np.float32), X


@pytest.mark.parametrize("lrt", [True, False])
def test_iter_weighting_vs_oracle(gpu, lrt):
    """--iter_weighting (src/option.cpp:437-530): same fixed SNPs, final weights, h² and BLUE as
    the oracle's restatement of the two-stage flow."""
    counts, rows, y, X = _strong_problem()
    n, m = counts.shape[1], counts.shape[0]
    persnp = np.ones(m, np.float32)
    maf = orc.maf(orc.popcounts(counts), n)
    kw = dict(lrt=lrt, seed=1, n_V=12, n_MC=4, window_size=20, sig_chisq=30.0, indep_r2=0.5)
    r64 = orc.REML_iter_weighting(counts, None, X, y, persnp, maf, dtype=np.float64, **kw)
    with api.Genotypes(rows, n) as g:
        gmaf, _ = g.marker_qc()
        assert np.array_equal(gmaf, maf)
        r = g.REML_iter_weighting(None, X, y, persnp, gmaf, **kw)
    assert r["fixed"] == r64["fixed"] == [1200, 300, 301]
    assert np.allclose(r["persnp"], r64["persnp"], rtol=2e-3, atol=1e-4)
    assert abs(r["h2"] - r64["h2"]) <= 1e-4
    assert np.allclose(r["blue"], r64["blue"], rtol=5e-3, atol=5e-3)
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.9999


@pytest.mark.parametrize("window_size,c", [(100, 2), (1000, 1)])
def test_lmm_quadforms_vs_oracle(gpu, window_size, c):
    """--lmm quadratic forms (src/reml.cpp:919-981): the reference's marker sample, and xPy, xPx,
    xBx, xSx against the FP64 oracle (relative tolerance 1e-4 on xPy, xSx; 5e-4 on xPx, xBx)."""
    counts, rows, y, rvec, X, persnp = _problem(n=1500, m=2600, seed=47, c=c)
    n, m = counts.shape[1], counts.shape[0]
    pc = orc.popcounts(counts)
    gm = orc.genotype_mean(pc, n)
    gw = orc.snp_weights(gm, persnp)
    rr = (1 / np.sqrt(rvec)).astype(np.float32)
    Q, _, _ = orc.qr_colpiv(rr[:, None] * X)
    Py = np.random.default_rng(3).standard_normal(n).astype(np.float32)
    tau1 = 1.7
    ref = orc.LMM_quadforms(counts, Py, rr, Q, gm, gw, tau1, num_qf=30, window_size=window_size)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, gw, rr)
        g.set_projection(Q.astype(np.float32))
        r = g.LMM_quadforms(Py, tau1, num_qf=30, window_size=window_size)
    assert r["variants"] == ref["variants"]
    for key, tol in (("xPy", 1e-4), ("xSx", 1e-4), ("xPx", 5e-4), ("xBx", 5e-4)):
        assert np.allclose(r[key], ref[key], rtol=tol, atol=tol * np.max(np.abs(ref[key]))), key


def test_gwa_windows_vs_reference_script(gpu):
    """Windowed MLMA (bin/slemm_gwa.py:259-434) on the golden case produced by the reference's own
    script: same NaN pattern, beta within 1e-3 relative, −log10 p within 1e-3."""
    from conftest import load_gwa_case
    c = load_gwa_case(os.path.join(GOLD, "gwa_case"))
    with api.Genotypes(c["rows"], c["n_fam"]) as g:
        beta, se, chisq, p = g.gwa_windows(c["y"], c["R"], c["covar"], c["ksnp_idx"], c["chr_start"], c["chr_end"],
                                           c["block_size"], c["tau"], c["model_snp_ct"], c["cfactor"], c["snp_var"],
                                           c["mac"])
    ref = c["ref"]
    ok = np.isfinite(ref["p"])
    assert np.array_equal(ok, np.isfinite(p))
    assert np.allclose(beta[ok], ref["beta"][ok], rtol=1e-3, atol=1e-5)
    assert np.max(np.abs(np.log10(p[ok]) - np.log10(ref["p"][ok]))) <= 1e-3


@pytest.mark.parametrize("n,m,tol", [(900, 500, 1e-4), (600, 1100, 2e-2)])
def test_wls_vs_oracle(gpu, n, m, tol):
    """--wls (src/wls.cpp:4-129) against the FP64 oracle: ‖b − b_ref‖/‖b_ref‖ ≤ 1e-4 when m < n;
    when m > n the system is ridge-regularised (1e-4·mean(diag)) and its FP32 Cholesky — the
    reference's precision — loses digits in proportion to the condition number, bound 2e-2."""
    counts, rows, y, rvec, X, _ = _problem(n=n, m=m, seed=53)
    ref = orc.WLS(counts, rvec, X, y)
    with api.Genotypes(rows, n) as g:
        b = g.weighted_least_squares(rvec, X, y)
    assert np.linalg.norm(b - ref) / np.linalg.norm(ref) <= tol
