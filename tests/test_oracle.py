"""CPU checks of the oracle itself: pinned against the reference's own code and golden vectors,
and against dense FP64 ground truth on tiny problems (known-answer tests)."""
import json
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import slemm_np as orc
from slemm_gb300 import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ---- integer path --------------------------------------------------------------------------
def test_bed_decode_known_answers():
    """Hand-built bytes: codes LSB-first 00→0, 01 (missing)→1, 10→1, 11→2 (src/input.cpp:364-378)."""
    rows = np.array([[0b11100100, 0b00000011]], dtype=np.uint8)   # codes 0,1,2,3 | 3,0,0,0
    out = orc.bed_decode(rows, 5)
    assert out.tolist() == [[0, 1, 1, 2, 2]]
    keep = np.array([1, 0, 1, 0, 1], np.uint8)                   # skip individuals 1 and 3
    assert orc.bed_decode(rows, 5, keep).tolist() == [[0, 1, 2]]
    pc = orc.popcounts(out)
    assert pc.tolist() == [6]
    n0, n1, n2 = orc.hwe_counts(out)
    assert (n0[0], n1[0], n2[0]) == (1, 2, 2)                     # missing counted as het


def test_decode_matches_generator_encoding():
    c, _ = synth.simulate_counts(333, 40, seed=5)
    rows = synth.encode_bed(c)
    assert np.array_equal(orc.bed_decode(rows, 333), c)
    rows_m = synth.encode_bed(c, missing=0.1, seed=3)
    d = orc.bed_decode(rows_m, 333)
    assert np.array_equal(d, synth.counts_of_bed(rows_m, 333))
    assert (d[c != d] == 1).all()                                 # every changed call became 1


def test_maf_and_gm_are_fp32_like_reference():
    pc = np.array([0, 1, 999, 1000, 1001, 2000], np.int64)
    n = 1000
    maf = orc.maf(pc, n)
    f = (pc / np.float32(2 * n)).astype(np.float32)
    expect = np.abs((f > 0.5).astype(np.float32) - f)
    assert np.array_equal(maf, expect)
    gm = orc.genotype_mean(pc, n)
    assert np.array_equal(gm, (pc.astype(np.float32) / np.float32(n)).astype(np.float32))


def test_rng_draws_match_golden():
    """libstdc++ mt19937 draws of the reference's generators (reml.cpp:597-605, 795-809)."""
    g = json.load(open(os.path.join(GOLD, "rng_draws.json")))
    for seed in (0, 1, 42):
        V = orc.rademacher(seed, 37, 3)
        assert np.array_equal(np.sign(V).astype(int).T, np.array(g[f"rademacher_seed{seed}_n37_nv3"]))
        assert np.allclose(np.linalg.norm(V, axis=0), 1.0, atol=1e-6)
        u, e = orc.lmc_draws(seed, 11, 7, 2)
        assert np.array_equal(u.T, np.array(g[f"lmc_seed{seed}_m11_n7_nmc2_u"], np.float32))
        assert np.array_equal(e.T, np.array(g[f"lmc_seed{seed}_m11_n7_nmc2_e"], np.float32))


def test_hwe_exact_matches_reference_snphwe2():
    """The oracle's exact HWE test reproduces every SNPHWE2 output of the reference (compiled
    from src/snphwe.cpp) in tests/golden/hwe_ref.json, including mid-p and p ~ 1e-305."""
    g = json.load(open(os.path.join(GOLD, "hwe_ref.json")))["cases"]
    for het, h1, h2, midp, p in g:
        v = orc.hwe_exact(het, h1, h2, midp)
        assert abs(v - p) <= 1e-12 * p, (het, h1, h2, midp, p, v)


def test_lmm_variant_sample_is_libstdcxx_random_shuffle():
    """The --lmm marker sample uses std::random_shuffle on the unseeded C rand(): the oracle calls
    the real library; check its first draws and the MAC > 20 filter."""
    import ctypes
    out = np.zeros(3, np.int32)
    orc._lib().oracle_libc_rand(1, 3, out.ctypes.data_as(ctypes.c_void_p))
    assert list(out) == [1804289383, 846930886, 1681692777]   # glibc's documented initial sequence
    gm = np.array([0.01, 0.5, 1.0, 1.99, 0.3, 1.5], np.float32)
    v = orc.lmm_variants(gm, 1000, 30)
    assert sorted(v) == [1, 2, 4, 5]


def test_gwa_windows_oracle_matches_reference_script():
    """The oracle restatement of bin/slemm_gwa.py:259-431 reproduces the reference script's output
    on the golden case (tests/golden/gwa_case, run with a PLINK1 stand-in for pgenlib)."""
    from conftest import load_gwa_case
    c = load_gwa_case(os.path.join(GOLD, "gwa_case"))
    beta, se, chisq, p = orc.gwa_windows(2 - c["a2"], c["y"], c["R"], c["covar"], c["ksnp_idx"], c["chr_start"],
                                         c["chr_end"], c["block_size"], c["tau"], c["model_snp_ct"], c["cfactor"],
                                         c["snp_var"], c["mac"])
    ref = c["ref"]
    ok = np.isfinite(ref["p"])
    assert np.array_equal(ok, np.isfinite(p))
    assert np.allclose(beta[ok], ref["beta"][ok], rtol=1e-4, atol=1e-6)
    assert np.max(np.abs(np.log10(p[ok]) - np.log10(ref["p"][ok]))) <= 1e-4


def test_hwe_golden_fixture_sane():
    """The fixture holds the reference SNPHWE2 outputs; p-values lie in (0, 1] and mid-p ≤ p."""
    g = json.load(open(os.path.join(GOLD, "hwe_ref.json")))["cases"]
    vals = {}
    for het, h1, h2, midp, p in g:
        assert 0.0 <= p <= 1.0 + 1e-12
        vals[(het, h1, h2, midp)] = p
    for (het, h1, h2, midp), p in vals.items():
        if midp == 1:
            assert p <= vals[(het, h1, h2, 0)] + 1e-12


# ---- operators, Lanczos, SLQ: known answers -------------------------------------------------
def _tiny(n=60, m=45, seed=1, c=2):
    counts, _ = synth.simulate_counts(n, m, seed=seed)
    pc = orc.popcounts(counts)
    gm = orc.genotype_mean(pc, n)
    rng = np.random.default_rng(seed)
    gw = orc.snp_weights(gm, rng.uniform(0.5, 1.5, m).astype(np.float32), np.float64)
    rr = rng.uniform(0.7, 1.3, n)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, c - 1))])
    Q, qrR, rank = orc.qr_colpiv(rr[:, None] * X)
    assert rank == c
    return counts, gm.astype(np.float64), gw, rr, X, Q, qrR


def test_operators_match_dense_fp64():
    counts, gm, gw, rr, X, Q, _ = _tiny()
    ops = orc.Operators(counts, gm, gw, rr, Q, subset_size=7, dtype=np.float64)
    Z = counts.T.astype(np.float64) - gm
    A = (rr[:, None] * Z) @ np.diag(gw) @ (Z.T * rr[None, :])
    P = np.eye(Z.shape[0]) - Q @ Q.T
    v = np.random.default_rng(2).standard_normal((Z.shape[0], 3))
    tau0 = 0.37
    assert np.allclose(ops.H0_quadform_mv(tau0, v), P @ A @ P @ v + tau0 * v - 0 * v, atol=1e-10)
    assert np.allclose(ops.H0_ldet_mv(tau0, v), A @ v + tau0 * v, atol=1e-10)
    assert np.allclose(ops.rmatvec(v), Z.T @ v, atol=1e-10)
    assert np.allclose(ops.weighted_rmatvec(v), gw[:, None] * (Z.T @ v), atol=1e-10)
    u = np.random.default_rng(3).standard_normal((Z.shape[1], 2))
    assert np.allclose(ops.matvec(u), Z @ u, atol=1e-10)


def test_lanczos_seed_and_shifted_solve_fp64():
    counts, gm, gw, rr, X, Q, _ = _tiny()
    ops = orc.Operators(counts, gm, gw, rr, Q, dtype=np.float64)
    Z = counts.T.astype(np.float64) - gm
    A = (rr[:, None] * Z) @ np.diag(gw) @ (Z.T * rr[None, :])
    n = A.shape[0]
    B = np.random.default_rng(4).standard_normal((n, 3))
    tau0 = 0.25
    seed = orc.L_Seed(ops, "ldet", tau0, B, tol=1e-12, maxit=400)
    for sigma in (0.0, 0.3, 2.0):
        X_ = orc.L_Solve(seed, B, sigma, tol=1e-11)
        exact = np.linalg.solve(A + (tau0 + sigma) * np.eye(n), B)
        assert np.allclose(X_, exact, rtol=1e-7, atol=1e-9)


def test_slq_equals_exact_quadratic_form_with_full_krylov():
    """With a complete Krylov basis, SLQ equals (n/n_V)·Σ vᵀ log(A+σI) v exactly."""
    counts, gm, gw, rr, X, Q, _ = _tiny(n=40, m=30)
    ops = orc.Operators(counts, gm, gw, rr, Q, dtype=np.float64)
    Z = counts.T.astype(np.float64) - gm
    A = (rr[:, None] * Z) @ np.diag(gw) @ (Z.T * rr[None, :])
    n = A.shape[0]
    V = orc.rademacher(0, n, 4).astype(np.float64)
    tau0 = 0.5
    seed = orc.L_Seed(ops, "ldet", tau0, V, tol=1e-13, maxit=n + 1)
    D, W = orc.jacobi_eig(seed)
    w, U = np.linalg.eigh(A + tau0 * np.eye(n))
    for sigma in (0.0, 0.7):
        L = U @ np.diag(np.log(w + sigma)) @ U.T
        exact = n / 4 * sum(V[:, p] @ L @ V[:, p] for p in range(4))
        assert math.isclose(orc.SLQ_LDet(D, W, n, 4, sigma), exact, rel_tol=1e-6)


def test_reml_criterion_matches_dense_fp64():
    """yᵀP̃y and log det(QᵀH⁻¹Q) of REML_criterion against dense FP64 algebra."""
    counts, gm, gw, rr, X, Q, _ = _tiny()
    ops = orc.Operators(counts, gm, gw, rr, Q, dtype=np.float64)
    n = counts.shape[1]
    y = np.random.default_rng(9).standard_normal(n)
    yp = rr * y
    yp = yp - Q @ (Q.T @ yp)
    tau0 = (1 - 0.7) / 0.7
    sy = orc.L_Seed(ops, "quadform", tau0, yp, tol=1e-12, maxit=300)
    sq = orc.L_Seed(ops, "ldet", tau0, Q, tol=1e-12, maxit=300)
    for h2 in (0.2, 0.5):
        tau = (1 - h2) / h2
        yPy = float(yp @ orc.L_Solve(sy, yp, tau - tau0, tol=1e-12)[:, 0])
        M = Q.T @ orc.L_Solve(sq, Q, tau - tau0, tol=1e-12)
        e_yPy, _, e_ld = orc.dense_reml_criterion(counts, gm, gw, rr, Q, yp, h2)
        assert math.isclose(yPy, e_yPy, rel_tol=1e-8)
        assert math.isclose(np.linalg.slogdet(M)[1], e_ld, rel_tol=1e-8, abs_tol=1e-8)


INVPHI = 0.618033988749894848204586834365638117720309179805762862135
INVPHI2 = 0.381966011250105151795413165634361882279690820194237137864


def test_gss_points_round_once_from_double():
    """src/reml.cpp:520-540 forms `c = a + invphi2 * h;` and `h *= invphi;` from float a, h and
    double constants: C++ evaluates in double and rounds once to float.  NumPy 2 keeps a float32
    times a Python float in float32, which rounds differently on a share of the points; the oracle
    must follow the reference's double evaluation on every one of them."""
    rng = np.random.default_rng(0)
    differ = 0
    for _ in range(4000):
        a = np.float32(rng.uniform(1e-4, 0.7))
        h = np.float32(rng.uniform(1e-5, 0.7))
        for k in (INVPHI2, INVPHI):
            want = np.float32(float(a) + k * float(h))      # double sum of a double product, rounded once
            assert orc.gss_point(a, k, h) == want
            if np.float32(a + k * h) != want:               # float32 arithmetic (NumPy 2 promotion)
                differ += 1
    assert differ > 0


def test_fp32_reference_gss_spread_at_config1():
    """The reference's FP32 DF-REML against the FP64 oracle on the n = 2,000, m = 10,000
    configuration (1 % missing, 30 probes, seed 1): its float criterion varies by ~1e-4 between
    neighbouring golden-section points, so the FP32 search ends within a few 1e-4 of the FP64 one,
    not within 1e-5 — the spread the GPU parity tests of that configuration take into account."""
    n, m = 2000, 10000
    counts, _ = synth.simulate_counts(n, m, seed=1)
    rows = synth.encode_bed(counts, missing=0.01, seed=12)
    dec = orc.bed_decode(rows, n)
    y, _, _ = synth.simulate_phenotype(dec, 0.5, n_causal=1000, seed=1)
    X = np.ones((n, 1), np.float32)
    ps = np.ones(m, np.float32)
    r32 = orc.SLDF_REML(dec, None, X, y.astype(np.float32), ps, seed=1, n_V=30, dtype=np.float32)
    r64 = orc.SLDF_REML(dec, None, X, y.astype(np.float32), ps, seed=1, n_V=30, dtype=np.float64)
    assert r32["iters"] == r64["iters"]
    d = abs(r32["h2"] - r64["h2"])
    assert 1e-6 < d < 5e-4, d


def test_sldf_fp32_oracle_close_to_fp64_oracle():
    """The FP32 restatement (reference arithmetic) and the FP64 oracle agree on h² within the
    golden-section resolution: the search stops on a bracket of width (b−a)·0.618^nitr ≈ 7e-5 and
    reports its last evaluated point, so two runs whose criteria differ by FP32 rounding can end
    up to two brackets apart (3e-4 here, n = 400)."""
    n, m = 400, 300
    counts, _ = synth.simulate_counts(n, m, seed=11)
    y, _, _ = synth.simulate_phenotype(counts, 0.5, n_causal=100, seed=11)
    X = np.ones((n, 1))
    r32 = orc.SLDF_REML(counts, None, X, y, np.ones(m), seed=1, n_V=10, dtype=np.float32)
    r64 = orc.SLDF_REML(counts, None, X, y, np.ones(m), seed=1, n_V=10, dtype=np.float64)
    assert abs(r32["h2"] - r64["h2"]) < 3e-4


# ---- GWAS step 2 pinned by the reference script's own output ---------------------------------
def test_gamma_oracle_matches_reference_script_output():
    d = os.path.join(GOLD, "gamma_case")
    n_fam = sum(1 for _ in open(os.path.join(d, "geno.fam")))
    raw = np.fromfile(os.path.join(d, "geno.bed"), dtype=np.uint8)[3:]
    rows = raw.reshape(-1, (n_fam + 3) // 4)
    counts = orc.bed_decode(rows, n_fam)
    py = [l.split() for l in open(os.path.join(d, "s1.reml.py.txt")).read().splitlines()[1:]]
    Py = np.array([float(r[1]) for r in py], np.float32)
    cov = np.array([[float(v) for v in r[2:-1]] for r in py], np.float32)
    R = np.array([float(r[-1]) for r in py], np.float32)
    rr = (1.0 / np.sqrt(R)).astype(np.float32)
    from scipy import linalg
    Q = linalg.qr(np.transpose(np.transpose(cov) * rr), mode="economic")[0]
    xy, xx = orc.gamma_terms(counts, Py, rr, Q, mac=20)
    gs = [l.split() for l in open(os.path.join(d, "s1.gstat.txt")).read().splitlines()[1:]]
    cf = orc.mean_wo_outliers([float(r[9]) / float(r[7]) for r in gs])
    vc = open(os.path.join(d, "s1.reml.vc.csv")).read().splitlines()
    snp_var = float(vc[2].split(",")[1])
    beta, se, chisq, p = orc.gamma_stats(xy, xx, cf, snp_var)
    ref = [l.split("\t") for l in open(os.path.join(d, "gamma.txt")).read().splitlines()[1:]]
    rb = np.array([float(r[6]) for r in ref])
    rp = np.array([float(r[9]) for r in ref])
    ok = np.isfinite(rb)
    assert np.array_equal(ok, np.isfinite(beta))
    assert np.allclose(beta[ok], rb[ok], rtol=2e-5, atol=1e-7)
    assert np.max(np.abs(np.log10(p[ok]) - np.log10(rp[ok]))) < 1e-4


# ---- window weighting -------------------------------------------------------------------------
def test_window_weights_sliding_rule():
    """option.cpp:505-511: sliding mean over window_size+1 SNPs with clamped ends, then the logistic."""
    m, ws = 50, 10
    rng = np.random.default_rng(0)
    maf_v = rng.uniform(0.05, 0.5, m)
    b = rng.standard_normal(m)
    snpvar, w = orc.window_weights(maf_v, b, ws)
    sv = 2 * maf_v.astype(np.float32) * (1 - maf_v.astype(np.float32)) * b.astype(np.float32) ** 2
    sv = sv / sv.mean()
    for i in (0, 4, 5, 25, 44, 45, 49):
        if i < ws // 2:
            seg = sv[: ws + 1]
        elif i > m - ws // 2 - 1:
            seg = sv[m - ws - 1:]
        else:
            seg = sv[i - ws // 2: i - ws // 2 + ws + 1]
        x = seg.mean()
        assert math.isclose(w[i], 0.001 / (0.001 + 0.999 * math.exp(-0.5 * x)), rel_tol=1e-5)


def _grad_problem(n=300, m=240, seed=9):
    counts, _ = synth.simulate_counts(n, m, seed=seed)
    y, _, _ = synth.simulate_phenotype(counts, 0.5, n_causal=50, seed=seed)
    rng = np.random.default_rng(seed)
    X = np.column_stack([np.ones(n), rng.standard_normal(n)])
    rvec = rng.uniform(0.8, 1.3, n)
    persnp = rng.uniform(0.5, 1.5, m)
    window = np.repeat(np.arange(6), m // 6)
    window[:10] = -1
    wwin = rng.uniform(0.5, 2.0, 6)
    return counts, rvec, X, y, persnp, window, wwin


def test_reml_gradient_matches_central_finite_differences():
    """The FP64 gradient formulas (variance components and per-window weights) against central
    differences of the exact REML log-likelihood, step 1e-4."""
    counts, rvec, X, y, persnp, window, wwin = _grad_problem()
    sg2, se2, h = 0.6, 0.9, 1e-4
    d_sg, d_se, d_w = orc.reml_grad_dense(counts, rvec, X, y, persnp, window, wwin, sg2, se2)

    def f(sg=sg2, se=se2, w=wwin):
        return orc.reml_loglik_dense(counts, rvec, X, y, persnp, window, w, sg, se)

    assert abs(d_sg - (f(sg=sg2 + h) - f(sg=sg2 - h)) / (2 * h)) <= 1e-6 * abs(d_sg)
    assert abs(d_se - (f(se=se2 + h) - f(se=se2 - h)) / (2 * h)) <= 1e-6 * abs(d_se)
    for k in range(len(wwin)):
        wp, wm = wwin.copy(), wwin.copy()
        wp[k] += h
        wm[k] -= h
        assert abs(d_w[k] - (f(w=wp) - f(w=wm)) / (2 * h)) <= 1e-6 * np.max(np.abs(d_w))


def test_reml_gradient_hutchinson_estimate_converges():
    """With the reference's Rademacher probes the trace estimate approaches the exact gradient
    (4000 probes: within 3 %)."""
    counts, rvec, X, y, persnp, window, wwin = _grad_problem()
    exact = orc.reml_grad_dense(counts, rvec, X, y, persnp, window, wwin, 0.6, 0.9)
    est = orc.reml_grad_dense(counts, rvec, X, y, persnp, window, wwin, 0.6, 0.9,
                              probes=orc.rademacher(0, counts.shape[1], 4000))
    assert abs(est[0] - exact[0]) <= 0.03 * abs(exact[0])
    assert abs(est[1] - exact[1]) <= 0.03 * abs(exact[1])
    assert np.max(np.abs(est[2] - exact[2])) <= 0.03 * np.max(np.abs(exact[2]))
